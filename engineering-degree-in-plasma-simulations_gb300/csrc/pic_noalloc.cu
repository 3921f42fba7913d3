// Number density of one species without any device allocation.
//
// Some callers cannot allocate device memory: plugins whose host application owns all device
// memory through its own allocator (a cudaMalloc of theirs would bypass that allocator's
// accounting and limits), and real-time loops that forbid allocation after start-up because an
// allocation can block for an unbounded time.  They still own the particle arrays and the
// output field, and pass them in.  The only working memory this entry point needs -- the 64-bit
// fixed-point accumulator of one node field -- lives in the file-scope device array below, sized
// for kNoAllocMaxNodes nodes.  Every GPU that loads the library holds it (8 MiB) until the
// process exits.
//
// The array name is only a host-side stand-in for a device address; the real address is
// looked up with cudaGetSymbolAddress once per device, with that device current, on the first
// call made on the device.  That first call should therefore happen before any stream
// capture.  All calls share the one array and it keeps the last call's contents, so each call
// clears the part it uses first, and calls that overlap on the GPU (different streams, or
// different host threads on the same device) race on it.
#include <cstdio>
#include <mutex>
#include "../../include/pic_gb300.h"
#include "pic_kernels.h"

namespace pic {

constexpr int kNoAllocMaxNodes = 1 << 20;  // 64 x 64 x 256 nodes
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) unsigned long long g_noalloc_acc[kNoAllocMaxNodes];

// eight corner contributions per particle, 64-bit fixed point, straight into the accumulator
// (same weights and rounding as the deposit of the fused push kernel)
__global__ void k_noalloc_deposit(GridDev g, const float4* __restrict__ pos, const float4* __restrict__ vel, long n,
                                  float scale, unsigned long long* acc) {
    const int nij = g.ni * g.nj;
    for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < n; p += (long)gridDim.x * blockDim.x) {
        float4 ps = pos[p];
        int c = __float_as_int(ps.w);
        if (c < 0) continue;
        int i, j, k;
        cell_ijk(g, c, i, j, k);
        if (i >= g.ci || j >= g.cj || k >= g.ck) continue;  // not a cell of this grid
        int b = cell_base_node(g, i, j, k);
        float w = vel[p].w;
        float wx1 = ps.x, wx0 = 1.f - ps.x, wy1 = ps.y, wy0 = 1.f - ps.y, wz1 = ps.z, wz0 = 1.f - ps.z;
        float s = w * scale;
        float s00 = s * wx0 * wy0, s10 = s * wx1 * wy0, s01 = s * wx0 * wy1, s11 = s * wx1 * wy1;
        atomicAdd(&acc[b], __float2ull_rn(s00 * wz0));
        atomicAdd(&acc[b + 1], __float2ull_rn(s10 * wz0));
        atomicAdd(&acc[b + g.ni], __float2ull_rn(s01 * wz0));
        atomicAdd(&acc[b + g.ni + 1], __float2ull_rn(s11 * wz0));
        atomicAdd(&acc[b + nij], __float2ull_rn(s00 * wz1));
        atomicAdd(&acc[b + nij + 1], __float2ull_rn(s10 * wz1));
        atomicAdd(&acc[b + nij + g.ni], __float2ull_rn(s01 * wz1));
        atomicAdd(&acc[b + nij + g.ni + 1], __float2ull_rn(s11 * wz1));
    }
}

// den = accumulated weight / node volume, periodic copies folded onto index 0
__global__ void k_noalloc_finalize(GridDev g, const unsigned long long* __restrict__ acc, double inv_scale,
                                   float* __restrict__ den) {
    const double inv_base = 1.0 / (g.dxd[0] * g.dxd[1] * g.dxd[2]);
    const int nn[3] = {g.ni, g.nj, g.nk}, stride[3] = {1, g.ni, g.ni * g.nj};
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < g.nv; n += gridDim.x * blockDim.x) {
        int ijk[3];
        int r = n / g.ni;
        ijk[0] = n - r * g.ni;
        ijk[2] = r / g.nj;
        ijk[1] = r - ijk[2] * g.nj;
        bool alias = false;
        unsigned fold = 0;
        double inv_vol = inv_base;
        for (int d = 0; d < 3; d++) {
            if (g.periodic[d]) {
                if (ijk[d] == nn[d] - 1) alias = true;
                if (ijk[d] == 0) fold |= 1u << d;
            } else if (ijk[d] == 0 || ijk[d] == nn[d] - 1) {
                inv_vol *= 2.0;
            }
        }
        if (alias) continue;
        unsigned long long tot = 0;
        for (unsigned m = 0; m < 8; m++) {
            if (m & ~fold) continue;
            int node = n;
            for (int d = 0; d < 3; d++)
                if (m & (1u << d)) node += (nn[d] - 1) * stride[d];
            tot += acc[node];
        }
        float v = (float)((double)tot * (inv_scale * inv_vol));
        for (unsigned m = 0; m < 8; m++) {
            if (m & ~fold) continue;
            int node = n;
            for (int d = 0; d < 3; d++)
                if (m & (1u << d)) node += (nn[d] - 1) * stride[d];
            den[node] = v;
        }
    }
}

namespace {
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[kNoAllocMaxDevices] = {};
}  // namespace

}  // namespace pic

using namespace pic;

extern "C" int pic_number_density_noalloc(int ni, int nj, int nk, const double* x0, const double* xm,
                                          const int* periodic, const void* pos4, const void* vel4, long n,
                                          double scale, float* den_out, void* stream) {
    long long nv = (long long)ni * nj * nk;
    if (!x0 || !xm || (n > 0 && (!pos4 || !vel4)) || !den_out || n < 0 || !(scale > 0))
        return set_last_error(PIC_ERR_ARG, "pic_number_density_noalloc: null array, negative count or scale <= 0");
    // the packed particle cell keeps 9 bits for i and j and 13 for k (pic_world_create's limits)
    if (ni < 2 || nj < 2 || nk < 2 || ni - 1 > kCellMaxIJ || nj - 1 > kCellMaxIJ || nk - 1 > kCellMaxK)
        return set_last_error(PIC_ERR_ARG, "pic_number_density_noalloc: grid must have 2..513 x 2..513 x 2..8193 nodes");
    if (nv > kNoAllocMaxNodes) {
        char msg[160];
        snprintf(msg, sizeof(msg), "pic_number_density_noalloc: %lld nodes exceed the %d-node accumulator", nv,
                 kNoAllocMaxNodes);
        return set_last_error(PIC_ERR_ARG, msg);
    }
    for (int d = 0; d < 3; d++)
        if (!(xm[d] > x0[d])) return set_last_error(PIC_ERR_ARG, "pic_number_density_noalloc: xm must exceed x0");
    {
        const int nn3[3] = {ni, nj, nk};
        for (int d = 0; d < 3; d++)  // as pic_world_set_boundaries
            if (periodic && periodic[d] && nn3[d] < 4)
                return set_last_error(PIC_ERR_ARG, "pic_number_density_noalloc: periodic axis needs at least 4 nodes");
    }
    // the deposit scales in FP32; the finalize divides by the same FP32 value
    const float fscale = (float)scale;
    if (!(fscale > 0.f) || !(fscale < 3.0e38f))
        return set_last_error(PIC_ERR_ARG, "pic_number_density_noalloc: scale is not a finite FP32 value");
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices)
        return set_last_error(PIC_ERR_CUDA, "pic_number_density_noalloc: no current CUDA device");
    void* acc = nullptr;
    {
        // first call on this device: look up the device address of the file-scope array
        std::lock_guard<std::mutex> lock(g_noalloc_mutex);
        if (!g_noalloc_ptr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_acc) != cudaSuccess || !p)
                return set_last_error(PIC_ERR_CUDA, "pic_number_density_noalloc: cudaGetSymbolAddress failed");
            g_noalloc_ptr[dev] = p;
        }
        acc = g_noalloc_ptr[dev];
    }
    GridDev g{};
    g.ni = ni;
    g.nj = nj;
    g.nk = nk;
    g.ci = ni - 1;
    g.cj = nj - 1;
    g.ck = nk - 1;
    g.nv = (int)nv;
    g.nc = g.ci * g.cj * g.ck;
    int nn[3] = {ni, nj, nk};
    for (int d = 0; d < 3; d++) {
        g.x0[d] = x0[d];
        g.xm[d] = xm[d];
        g.dxd[d] = (xm[d] - x0[d]) / (nn[d] - 1);
        g.dx[d] = (float)g.dxd[d];
        g.inv_dx[d] = (float)(1.0 / g.dxd[d]);
        g.periodic[d] = periodic ? (periodic[d] != 0) : 0;
    }
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * nv, s) != cudaSuccess)
        return set_last_error(PIC_ERR_CUDA, "pic_number_density_noalloc: clearing the accumulator failed");
    // launched through cudaLaunchKernel, whose return value is this launch's own status: an error
    // the caller left pending before this call is neither reported nor cleared here
    unsigned long long* accp = (unsigned long long*)acc;
    if (n > 0) {
        long blocks = (n + 255) / 256;
        if (blocks > 4096) blocks = 4096;
        const float4* p4 = (const float4*)pos4;
        const float4* v4 = (const float4*)vel4;
        void* args[] = {&g, &p4, &v4, &n, (void*)&fscale, &accp};
        if (cudaLaunchKernel((const void*)k_noalloc_deposit, dim3((unsigned)blocks), dim3(256), args, 0, s) !=
            cudaSuccess)
            return set_last_error(PIC_ERR_CUDA, "pic_number_density_noalloc: deposit launch failed");
    }
    int fb = (int)((nv + 255) / 256);
    if (fb > 4096) fb = 4096;
    const unsigned long long* caccp = accp;
    double inv_scale = 1.0 / (double)fscale;
    void* fargs[] = {&g, &caccp, &inv_scale, &den_out};
    if (cudaLaunchKernel((const void*)k_noalloc_finalize, dim3((unsigned)fb), dim3(256), fargs, 0, s) != cudaSuccess)
        return set_last_error(PIC_ERR_CUDA, "pic_number_density_noalloc: finalize launch failed");
    return PIC_OK;
}
