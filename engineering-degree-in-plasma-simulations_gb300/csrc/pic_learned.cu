// Learned multilevel Poisson preconditioner: inference, training and the flexible CG that
// uses it, plus a one-tile tcgen05 GEMM check of the tensor-core operand layout.
//
// Level transfers are cell-centred trilinear: along one axis the fine point f receives
// 3/4 of coarse point f/2 and 1/4 of its neighbour on the side of f (f even: f/2 - 1, f odd:
// f/2 + 1); restriction is the exact transpose.  Periodic axes wrap at every level (over
// the level's own extent), other axes read zero outside the box.
#include <algorithm>
#include <cmath>
#include <type_traits>
#include <vector>
#include <cuda_bf16.h>
#include <cstring>
#include "pic_learned.h"
#include "pic_stencil.cuh"
#include "pic_tc.cuh"

namespace pic {

constexpr long long kTcWaitLimit = kMbarWaitPolls;
// polls of a first wait for MMA completion, as PushArgs::wait_polls (0: kTcWaitLimit); the wait
// for the MMAs in flight after a timeout always allows kTcWaitLimit before TMEM is freed
static __device__ long long g_tc_wait_arg = 0;

// D (128 x N, FP32, row-major) = A (128 x K, bf16, row-major) * B^T (B: N x K, bf16, row-major)
// 128 threads; K a multiple of 16, N in {16, 32, 64, 128}
__global__ void __launch_bounds__(128) k_tc_gemm_tile(const __nv_bfloat16* __restrict__ A,
                                                      const __nv_bfloat16* __restrict__ B, float* __restrict__ D,
                                                      int N, int K, unsigned* err) {
    extern __shared__ __align__(128) unsigned char smem[];
    __nv_bfloat16* sA = reinterpret_cast<__nv_bfloat16*>(smem);
    const int slices = K / 16;
    __nv_bfloat16* sB = sA + slices * 128 * 16;
    __shared__ uint32_t tmem_base;
    __shared__ __align__(8) uint64_t bar;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int idx = tid; idx < 128 * K; idx += 128) {
        int m = idx / K, k = idx - m * K;
        sA[(k >> 4) * 2048 + tc_slice_offset(m, k & 15)] = A[idx];
    }
    for (int idx = tid; idx < N * K; idx += 128) {
        int nn = idx / K, k = idx - nn * K;
        sB[(k >> 4) * (N * 16) + tc_slice_offset(nn, k & 15)] = B[idx];
    }
    tc_fence_smem();
    const uint32_t ncols = N < 32 ? 32 : N;
    if (warp == 0) {
        tc_alloc(&tmem_base, ncols);
        tc_relinquish();
    }
    if (tid == 0) tc_mbar_init(&bar, 1);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tm = tmem_base;
    if (tid == 0) {
        const uint32_t idesc = tc_idesc_bf16(128, N);
        for (int s = 0; s < slices; s++)
            tc_mma_bf16(tm, tc_smem_desc(sA + s * 2048, 128, 256), tc_smem_desc(sB + s * N * 16, 128, 256), idesc,
                        s > 0 ? 1u : 0u);
        tc_commit(&bar);
    }
    bool ok = tc_mbar_wait(&bar, 0, wait_poll_limit(g_tc_wait_arg, kTcWaitLimit));
    if (!ok) {
        if (tid == 0) set_error(err, kErrBarrierTimeout);
        tc_mbar_wait(&bar, 0, kTcWaitLimit);  // bounded wait for the MMAs in flight before freeing TMEM
    }
    tc_fence_after();
    if (ok) {
        for (int c0 = 0; c0 < N; c0 += 16) {
            float v[16];
            tc_ld16(tm + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
#pragma unroll
            for (int c = 0; c < 16; c++) D[(32 * warp + lane) * N + c0 + c] = v[c];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_dealloc(tm, ncols);
}


// =====================================================================================
// level views and transfers
// =====================================================================================
LView lp_view(float* a, const int n[3], int sy, int sz, const int per[3]) {
    LView v;
    v.a = a;
    for (int d = 0; d < 3; d++) {
        v.n[d] = n[d];
        v.per[d] = per[d];
    }
    v.sy = sy;
    v.sz = sz;
    v.fx = make_fastdiv((unsigned)n[0]);
    v.fxy = make_fastdiv((unsigned)(n[0] * n[1]));
    v.nvox = n[0] * n[1] * n[2];
    return v;
}
LView lp_level_view(const LpState& L, int l, float* a) {
    return lp_view(a, L.dims[l], L.dims[l][0], L.dims[l][0] * L.dims[l][1], L.per);
}
LView lp_node_view(const GridDev& g, const LpState& L, float* a) {
    return lp_view(a, L.dims[0], g.ni, g.ni * g.nj, L.per);
}

__device__ __forceinline__ void lv_decode(const LView& v, unsigned idx, int& x, int& y, int& z) {
    unsigned t = fdiv(idx, v.fx);
    x = (int)(idx - t * (unsigned)v.n[0]);
    unsigned zz = fdiv(idx, v.fxy);
    z = (int)zz;
    y = (int)(t - zz * (unsigned)v.n[1]);
}
__device__ __forceinline__ int lv_off(const LView& v, int x, int y, int z) { return x + y * v.sy + z * v.sz; }
// coordinate c + d along an axis of extent n (|d| <= 2, n >= 2): wrapped, or -1 outside
__device__ __forceinline__ int lv_nb(int c, int d, int n, int per) {
    int u = c + d;
    if (per) return u < 0 ? u + n : (u >= n ? u - n : u);
    return (u < 0 || u >= n) ? -1 : u;
}

// z_coarse = R z_fine at coarse voxel idx
__device__ __forceinline__ void lp_restrict_at(const LView& f, const LView& c, unsigned idx) {
    {
        int cc[3];
        lv_decode(c, idx, cc[0], cc[1], cc[2]);
        const float w4[4] = {0.25f, 0.75f, 0.75f, 0.25f};
        if (cc[0] >= 1 && 2 * cc[0] + 2 < f.n[0] && cc[1] >= 1 && 2 * cc[1] + 2 < f.n[1] && cc[2] >= 1 &&
            2 * cc[2] + 2 < f.n[2]) {
            // interior: the 4 x 4 x 4 fine points are inside the box, no wrap
            const float* p0 = f.a + (2 * cc[0] - 1) + (2 * cc[1] - 1) * f.sy + (2 * cc[2] - 1) * f.sz;
            float acc = 0.f;
#pragma unroll
            for (int kz = 0; kz < 4; kz++) {
                float az = 0.f;
#pragma unroll
                for (int ky = 0; ky < 4; ky++) {
                    const float* row = p0 + ky * f.sy + kz * f.sz;
                    az += w4[ky] * (w4[0] * row[0] + w4[1] * row[1] + w4[2] * row[2] + w4[3] * row[3]);
                }
                acc += w4[kz] * az;
            }
            c.a[lv_off(c, cc[0], cc[1], cc[2])] = acc;
            return;
        }
        int fi[3][4];
#pragma unroll
        for (int ax = 0; ax < 3; ax++) {
#pragma unroll
            for (int k = 0; k < 4; k++) {
                int raw = 2 * cc[ax] + k - 1;
                int nc2 = 2 * c.n[ax];
                if (f.per[ax]) {
                    raw = raw < 0 ? raw + nc2 : (raw >= nc2 ? raw - nc2 : raw);
                    fi[ax][k] = raw < f.n[ax] ? raw : -1;
                } else {
                    fi[ax][k] = (raw >= 0 && raw < f.n[ax]) ? raw : -1;
                }
            }
        }
        float acc = 0.f;
#pragma unroll
        for (int kz = 0; kz < 4; kz++) {
            if (fi[2][kz] < 0) continue;
            float az = 0.f;
#pragma unroll
            for (int ky = 0; ky < 4; ky++) {
                if (fi[1][ky] < 0) continue;
                const float* row = f.a + fi[1][ky] * f.sy + fi[2][kz] * f.sz;
                float ay = 0.f;
#pragma unroll
                for (int kx = 0; kx < 4; kx++)
                    if (fi[0][kx] >= 0) ay += w4[kx] * row[fi[0][kx]];
                az += w4[ky] * ay;
            }
            acc += w4[kz] * az;
        }
        c.a[lv_off(c, cc[0], cc[1], cc[2])] = acc;
    }
}
__global__ void k_lp_restrict(LView f, LView c, const int* flag) {
    if (flag && flag[0]) return;
    for (unsigned idx = blockIdx.x * blockDim.x + threadIdx.x; idx < (unsigned)c.nvox; idx += gridDim.x * blockDim.x)
        lp_restrict_at(f, c, idx);
}

// sum_c P(f, c) e_coarse[c] at fine point f
__device__ __forceinline__ float lp_prolong_at(const LView& cv, const int f[3]) {
    const float w2[2] = {0.75f, 0.25f};
    {
        // interior: both coarse neighbours of every axis inside the box, no wrap
        const int c0x = f[0] >> 1, c0y = f[1] >> 1, c0z = f[2] >> 1;
        const int sx = (f[0] & 1) ? 1 : -1, sy = (f[1] & 1) ? 1 : -1, sz = (f[2] & 1) ? 1 : -1;
        if ((unsigned)(c0x + sx) < (unsigned)cv.n[0] && (unsigned)(c0y + sy) < (unsigned)cv.n[1] &&
            (unsigned)(c0z + sz) < (unsigned)cv.n[2]) {
            const float* p = cv.a + c0x + c0y * cv.sy + c0z * cv.sz;
            const int oy = sy * cv.sy, oz = sz * cv.sz;
            const float a0 = w2[0] * p[0] + w2[1] * p[sx];
            const float a1 = w2[0] * p[oy] + w2[1] * p[oy + sx];
            const float a2 = w2[0] * p[oz] + w2[1] * p[oz + sx];
            const float a3 = w2[0] * p[oz + oy] + w2[1] * p[oz + oy + sx];
            return w2[0] * (w2[0] * a0 + w2[1] * a1) + w2[1] * (w2[0] * a2 + w2[1] * a3);
        }
    }
    int ci[3][2];
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
        int c0 = f[ax] >> 1;
        ci[ax][0] = c0;
        ci[ax][1] = lv_nb(c0, (f[ax] & 1) ? 1 : -1, cv.n[ax], cv.per[ax]);
    }
    float acc = 0.f;
#pragma unroll
    for (int kz = 0; kz < 2; kz++) {
        if (ci[2][kz] < 0) continue;
        float az = 0.f;
#pragma unroll
        for (int ky = 0; ky < 2; ky++) {
            if (ci[1][ky] < 0) continue;
            const float* row = cv.a + ci[1][ky] * cv.sy + ci[2][kz] * cv.sz;
            float ay = 0.f;
#pragma unroll
            for (int kx = 0; kx < 2; kx++)
                if (ci[0][kx] >= 0) ay += w2[kx] * row[ci[0][kx]];
            az += w2[ky] * ay;
        }
        acc += w2[kz] * az;
    }
    return acc;
}

// 3x3x3 stencil (taps t = 9(dz+1) + 3(dy+1) + (dx+1)) at point c
__device__ __forceinline__ float lp_stencil27(const LView& v, const float* __restrict__ S, const int c[3]) {
    if (c[0] >= 1 && c[0] + 1 < v.n[0] && c[1] >= 1 && c[1] + 1 < v.n[1] && c[2] >= 1 && c[2] + 1 < v.n[2]) {
        // interior: constant offsets, no wrap
        const float* p = v.a + (c[0] - 1) + (c[1] - 1) * v.sy + (c[2] - 1) * v.sz;
        float acc = 0.f;
#pragma unroll
        for (int dz = 0; dz < 3; dz++)
#pragma unroll
            for (int dy = 0; dy < 3; dy++) {
                const float* row = p + dy * v.sy + dz * v.sz;
                const float* k = S + 9 * dz + 3 * dy;
                acc += k[0] * row[0] + k[1] * row[1] + k[2] * row[2];
            }
        return acc;
    }
    float acc = 0.f;
#pragma unroll
    for (int dz = -1; dz <= 1; dz++) {
        int z = lv_nb(c[2], dz, v.n[2], v.per[2]);
        if (z < 0) continue;
#pragma unroll
        for (int dy = -1; dy <= 1; dy++) {
            int y = lv_nb(c[1], dy, v.n[1], v.per[1]);
            if (y < 0) continue;
            const float* row = v.a + y * v.sy + z * v.sz;
#pragma unroll
            for (int dx = -1; dx <= 1; dx++) {
                int x = lv_nb(c[0], dx, v.n[0], v.per[0]);
                if (x >= 0) acc += S[9 * (dz + 1) + 3 * (dy + 1) + dx + 1] * row[x];
            }
        }
    }
    return acc;
}

// folded network level: away from non-periodic faces the 5x5x5 stencil K5; on a face point the
// exact form sum_{t: c + o_t inside} sum_t' K27[t][t'] z[c + o_t + o_t'] (the network reads its
// intermediate channels as zero outside the box)
__device__ float lp_net_op(const LView& v, const float* __restrict__ fold, const float* __restrict__ fold_var,
                           const int c[3]) {
    bool interior = true;
#pragma unroll
    for (int ax = 0; ax < 3; ax++)
        if (!v.per[ax] && (c[ax] == 0 || c[ax] == v.n[ax] - 1)) interior = false;
    float acc = 0.f;
    if (c[0] >= 2 && c[0] + 2 < v.n[0] && c[1] >= 2 && c[1] + 2 < v.n[1] && c[2] >= 2 && c[2] + 2 < v.n[2]) {
        // all 125 taps inside the box: constant offsets
        const float* p = v.a + (c[0] - 2) + (c[1] - 2) * v.sy + (c[2] - 2) * v.sz;
        const float* K5 = fold + 729;
        for (int dz = 0; dz < 5; dz++)
#pragma unroll
            for (int dy = 0; dy < 5; dy++) {
                const float* row = p + dy * v.sy + dz * v.sz;
                const float* k = K5 + 25 * dz + 5 * dy;
#pragma unroll
                for (int dx = 0; dx < 5; dx++) acc += k[dx] * row[dx];
            }
        return acc;
    }
    if (interior) {
        const float* K5 = fold + 729;
        for (int dz = -2; dz <= 2; dz++) {
            int z = lv_nb(c[2], dz, v.n[2], v.per[2]);
            if (z < 0) continue;
            for (int dy = -2; dy <= 2; dy++) {
                int y = lv_nb(c[1], dy, v.n[1], v.per[1]);
                if (y < 0) continue;
                const float* row = v.a + y * v.sy + z * v.sz;
                const float* k = K5 + 25 * (dz + 2) + 5 * (dy + 2) + 2;
#pragma unroll
                for (int dx = -2; dx <= 2; dx++) {
                    int x = lv_nb(c[0], dx, v.n[0], v.per[0]);
                    if (x >= 0) acc += k[dx] * row[x];
                }
            }
        }
        return acc;
    }
    // a point on a non-periodic face: the 5x5x5 variant of its face class (precomputed from K27
    // with the first-stage taps outside the box left out), unless an axis has a single point
    int cls = 0, mul = 1;
    bool single = false;
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
        if (!v.per[ax]) {
            if (v.n[ax] == 1) single = true;
            cls += mul * (c[ax] == 0 ? 1 : (c[ax] == v.n[ax] - 1 ? 2 : 0));
        }
        mul *= 3;
    }
    if (!single && fold_var) {
        const float* K5 = fold_var + 125 * cls;
        for (int dz = -2; dz <= 2; dz++) {
            int z = lv_nb(c[2], dz, v.n[2], v.per[2]);
            if (z < 0) continue;
            for (int dy = -2; dy <= 2; dy++) {
                int y = lv_nb(c[1], dy, v.n[1], v.per[1]);
                if (y < 0) continue;
                const float* row = v.a + y * v.sy + z * v.sz;
                const float* k = K5 + 25 * (dz + 2) + 5 * (dy + 2) + 2;
#pragma unroll
                for (int dx = -2; dx <= 2; dx++) {
                    int x = lv_nb(c[0], dx, v.n[0], v.per[0]);
                    if (x >= 0) acc += k[dx] * row[x];
                }
            }
        }
        return acc;
    }
    for (int t = 0; t < 27; t++) {
        int u[3] = {lv_nb(c[0], t % 3 - 1, v.n[0], v.per[0]), lv_nb(c[1], (t / 3) % 3 - 1, v.n[1], v.per[1]),
                    lv_nb(c[2], t / 9 - 1, v.n[2], v.per[2])};
        if (u[0] < 0 || u[1] < 0 || u[2] < 0) continue;
        acc += lp_stencil27(v, fold + 27 * t, u);
    }
    return acc;
}

// e_l = op_l(z_l) + P e_{l+1} at voxel idx of level l; mode 1: network level (fold: its folded
// stencils in shared memory, fold_g the same in global memory with the face variants after them),
// 2: diagonal scaling
__device__ __forceinline__ void lp_up_at(const LView& zin, const LView& cin, const LView& out, int mode,
                                         const float* fold, const float* __restrict__ fold_g, float inv_diag,
                                         unsigned idx) {
    int c[3];
    lv_decode(out, idx, c[0], c[1], c[2]);
    float v = mode == 1 ? lp_net_op(zin, fold, fold_g + kLpFold, c) : inv_diag * zin.a[lv_off(zin, c[0], c[1], c[2])];
    if (cin.a) v += lp_prolong_at(cin, c);
    out.a[lv_off(out, c[0], c[1], c[2])] = v;
}
// e_l = op_l(z_l) + P e_{l+1}; mode 1: network level (fold), 2: diagonal scaling
__global__ void k_lp_up(LView zin, LView cin, LView out, int mode, const float* __restrict__ fold_g, float inv_diag,
                        const int* flag) {
    if (flag && flag[0]) return;
    __shared__ float fold[kLpFold];  // the level's folded stencils, read by every voxel
    if (mode == 1) {
        for (int x = threadIdx.x; x < kLpFold; x += blockDim.x) fold[x] = fold_g[x];
        __syncthreads();
    }
    for (unsigned idx = blockIdx.x * blockDim.x + threadIdx.x; idx < (unsigned)out.nvox;
         idx += gridDim.x * blockDim.x)
        lp_up_at(zin, cin, out, mode, fold, fold_g, inv_diag, idx);
}

// The coarse end of the hierarchy in one CTA: the restrictions from level l0 - 1 down to the
// last level, then the level operators from the last level back up to l0, with a block barrier
// between levels.  These levels hold a few thousand voxels or fewer, so one kernel instead of a
// launch per level and direction removes a chain of latency-bound launches; every voxel is
// computed by the same device functions as k_lp_restrict and k_lp_up.
struct LpCoarseArgs {
    int l0, nlev;
    LView f0;                        // level l0 - 1 (its restricted input; the residual if l0 == 1)
    LView z[kLpMaxLevels], e[kLpMaxLevels];
    int mode[kLpMaxLevels];          // 1: network level (folded stencils), 2: diagonal scaling
    const float* fold[kLpMaxLevels];
    float inv_diag[kLpMaxLevels];
};
constexpr int kLpCoarseThreads = 512;
constexpr int kLpCoarseMaxVox = 8192;    // diagonal levels up to this size join the fused chain
constexpr int kLpCoarseMaxNetVox = 1024;  // network levels up to this size
__global__ void __launch_bounds__(kLpCoarseThreads) k_lp_coarse(LpCoarseArgs a, const int* flag) {
    if (flag && flag[0]) return;
    __shared__ float fold[kLpFold];
    for (int l = a.l0; l < a.nlev; l++) {
        const LView& f = l == a.l0 ? a.f0 : a.z[l - 1];
        for (unsigned idx = threadIdx.x; idx < (unsigned)a.z[l].nvox; idx += blockDim.x) lp_restrict_at(f, a.z[l], idx);
        __syncthreads();
    }
    LView none{};
    none.a = nullptr;
    for (int l = a.nlev - 1; l >= a.l0; l--) {
        if (a.mode[l] == 1) {
            for (int x = threadIdx.x; x < kLpFold; x += blockDim.x) fold[x] = a.fold[l][x];
            __syncthreads();
        }
        const LView& cin = l + 1 < a.nlev ? a.e[l + 1] : none;
        for (unsigned idx = threadIdx.x; idx < (unsigned)a.e[l].nvox; idx += blockDim.x)
            lp_up_at(a.z[l], cin, a.e[l], a.mode[l], fold, a.fold[l], a.inv_diag[l], idx);
        __syncthreads();
    }
}

// level 0 on the node array: z = mask * (S0 * r + P e_1); with out != nullptr also z.r -> out[0]
// and z.q -> out[1] (deterministic grid sums)
__global__ void __launch_bounds__(kNodeThreads) k_lp_up0(GridDev g, LView rin, LView cin, float* __restrict__ z,
                                                         const uint16_t* __restrict__ kind,
                                                         const float* __restrict__ S0, const float* __restrict__ q,
                                                         double* gpart, int gstride, unsigned* ticket, double* out,
                                                         const int* flag) {
    if (flag && flag[0]) return;
    __shared__ float S[27];
    if (threadIdx.x < 27) S[threadIdx.x] = S0[threadIdx.x];
    __syncthreads();
    float f_zr = 0.f, f_zq = 0.f;
    const int base = blockIdx.x * kNodeTile + threadIdx.x;
#pragma unroll
    for (int q4 = 0; q4 < kNodeTile / kNodeThreads; q4++) {
        const int n = base + q4 * kNodeThreads;
        if (n >= g.nv) break;
        if ((kind[n] & 3) != kFree) {
            z[n] = 0.f;
            continue;
        }
        int c[3];
        node_ijk(g, n, c[0], c[1], c[2]);
        float v = lp_stencil27(rin, S, c);
        if (cin.a) v += lp_prolong_at(cin, c);
        z[n] = v;
        f_zr += v * rin.a[n];
        if (q) f_zq += v * q[n];
    }
    if (out) {
        const float vv[2] = {f_zr, f_zq};
        grid_sum<2>(vv, gpart, gstride, ticket, out);
    }
}

constexpr int kUp0X = 32, kUp0Y = 8, kUp0Z = 8;
constexpr int kUp0HX = kUp0X + 2, kUp0HY = kUp0Y + 2, kUp0HZ = kUp0Z + 2;
__device__ __forceinline__ int lv_map(int u, int n, int per) {
    if ((unsigned)u < (unsigned)n) return u;
    if (!per) return -1;
    // a tile past the end of a short periodic axis can reach beyond one period: reduce fully so
    // that every staged read stays on the grid
    const int m = u % n;
    return m < 0 ? m + n : m;
}
// Stages a halo tile of HX x R values (R rows of HX) in shared memory: element e = hx + HX row
// reads src[mx[hx] + myz[row]] (0 when either offset is -1).  The trip count is a constant, so
// every load of a thread is issued before its first shared store.
template <int HX, int R, int NT>
__device__ __forceinline__ void stage_tile(float* __restrict__ dst, const float* __restrict__ src, const int* mx,
                                           const int* myz) {
    constexpr int kN = HX * R, kPer = (kN + NT - 1) / NT;
    float v[kPer];
#pragma unroll
    for (int k = 0; k < kPer; k++) {
        const int e = threadIdx.x + k * NT;
        v[k] = 0.f;
        if (e < kN) {
            const int ox = mx[e % HX], oyz = myz[e / HX];
            if (ox >= 0 && oyz >= 0) v[k] = src[ox + oyz];
        }
    }
#pragma unroll
    for (int k = 0; k < kPer; k++) {
        const int e = threadIdx.x + k * NT;
        if (e < kN) dst[e] = v[k];
    }
}

// coarse tile of the prolongation for a 32 x 8 x 8 fine tile: coarse x0/2-1 .. x0/2+16 etc.
constexpr int kPcX = kUp0X / 2 + 2, kPcY = kUp0Y / 2 + 2, kPcZ = kUp0Z / 2 + 2;
// a staged residual row: slot 3 holds x0 - 1, slots 4 .. 35 x0 .. x0 + 31 (16-byte aligned), slot 36
// x0 + 32; the row pitch keeps every row's body 16-byte aligned
constexpr int kUp0P = 40, kUp0O = 3;
constexpr int kUp0Tile = kUp0P * kUp0HY * kUp0HZ, kPcTile = kPcX * kPcY * kPcZ;
constexpr int kUp0CtasPerSM = 4;
constexpr int kUp0DynSmem = 4 * 2 * (kUp0Tile + kPcTile + kUp0Z * kUp0X * kUp0Y + kUp0Z * kUp0Y);

// asynchronous 4-byte global -> shared copy (cp.async); with ok false nothing is read and the
// shared word is zero-filled (src-size 0; src is then any valid address)
__device__ __forceinline__ void cp_async_f32(float* dst, const float* src, bool ok) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(tc_smem_u32(dst)), "l"(src), "r"(ok ? 4 : 0)
                 : "memory");
}
// the same for 16 bytes (both addresses 16-byte aligned)
__device__ __forceinline__ void cp_async_16(float* dst, const float* src, bool ok) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(tc_smem_u32(dst)), "l"(src), "r"(ok ? 16 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// The fine level z = mask (S0 * r + P e_1), z.r and z.q, on 32 x 8 x 8 tiles of nodes by
// persistent CTAs that pipeline the tiles: while a CTA computes one tile from shared memory, the
// residual tile of its next tile (34 x 10 x 10 with the one-node halo, rows at a 40-float pitch
// with 16-byte aligned bodies, view neighbour rules:
// wrapped on periodic axes, zero outside) and the coarse tile of the prolongation (18 x 6 x 6) are
// already on their way into the other buffer through cp.async, which needs no registers.  A thread
// owns the columns of R adjacent output rows (R p .. R p + R - 1 of the tile): it walks the ten tile
// planes, reads the plane's R + 2 rows around them once, forms each row's three 3 x 3 partial sums
// and rolls them into the outputs of planes p+1, p, p-1.  R = 2 (128 threads, the 27 weights in
// registers: 12 shared reads per plane for two rows instead of 18) for grids with at least four
// tiles per persistent CTA; R = 1 (256 threads, weights read from shared memory within 64
// registers) below that, where eight warps per tile hide more of a tile's latency.
template <int R>
__global__ void __launch_bounds__(kUp0X * kUp0Y / R, kUp0CtasPerSM)
    k_lp_up0_pipe(GridDev g, LView rin, LView cin, float* __restrict__ z, const uint16_t* __restrict__ kind,
                  const float* __restrict__ S0, const float* __restrict__ q, double* gpart, int gstride,
                  unsigned* ticket, double* out, const int* flag, int bx_n, int by_n, int ntiles) {
    if (flag && flag[0]) return;
    __shared__ float S[27];
    __shared__ int mx[kUp0HX], myz[kUp0HY * kUp0HZ];  // halo offsets per axis (-1: outside)
    __shared__ int cmx[kPcX], cmyz[kPcY * kPcZ];
    // double buffers in dynamic shared memory (kUp0DynSmem bytes): residual tile, coarse tile,
    // q at the tile's outputs, FREE bits of the tile's output rows (x0 is a multiple of 32)
    extern __shared__ __align__(16) float up0_dyn[];
    float(*t)[kUp0Tile] = reinterpret_cast<float(*)[kUp0Tile]>(up0_dyn);
    float(*pc)[kPcTile] = reinterpret_cast<float(*)[kPcTile]>(up0_dyn + 2 * kUp0Tile);
    float(*qs)[kUp0Z][kUp0X * kUp0Y] = reinterpret_cast<float(*)[kUp0Z][kUp0X * kUp0Y]>(up0_dyn + 2 * (kUp0Tile + kPcTile));
    unsigned(*fm)[kUp0Z * kUp0Y] =
        reinterpret_cast<unsigned(*)[kUp0Z * kUp0Y]>(up0_dyn + 2 * (kUp0Tile + kPcTile + kUp0Z * kUp0X * kUp0Y));
    constexpr int kThr = kUp0X * kUp0Y / R;
    const int tid = threadIdx.x;
    const int tx = tid % kUp0X, ty0 = R * (tid / kUp0X);  // rows ty0 .. ty0 + R - 1 of the tile
    constexpr int kWarps = kThr / 32;
    if (tid < 27) S[tid] = S0[tid];
    // the halo maps of a tile, a barrier, then its copies into buffer b as one commit group
    auto issue = [&](int tile, int b) {
        int bb = tile;
        const int bx = bb % bx_n;
        bb /= bx_n;
        const int by = bb % by_n, bz = bb / by_n;
        const int x0 = bx * kUp0X, y0 = by * kUp0Y, z0 = bz * kUp0Z;
        if (tid < kUp0HX) mx[tid] = lv_map(x0 - 1 + tid, rin.n[0], rin.per[0]);
        if (tid < kUp0HY * kUp0HZ) {
            const int uy = lv_map(y0 - 1 + tid % kUp0HY, rin.n[1], rin.per[1]);
            const int uz = lv_map(z0 - 1 + tid / kUp0HY, rin.n[2], rin.per[2]);
            myz[tid] = (uy < 0 || uz < 0) ? -1 : uy * rin.sy + uz * rin.sz;
        }
        if (cin.a) {
            if (tid < kPcX) cmx[tid] = lv_map(x0 / 2 - 1 + tid, cin.n[0], cin.per[0]);
            if (tid < kPcY * kPcZ) {
                const int uy = lv_map(y0 / 2 - 1 + tid % kPcY, cin.n[1], cin.per[1]);
                const int uz = lv_map(z0 / 2 - 1 + tid / kPcY, cin.n[2], cin.per[2]);
                cmyz[tid] = (uy < 0 || uz < 0) ? -1 : uy * cin.sy + uz * cin.sz;
            }
        }
        __syncthreads();
        const int lane = tid & 31, wp = tid >> 5;
        // rows whose 32 body points are inside the box on aligned offsets go as eight 16-byte
        // copies and two halo words, three rows per warp step (lanes 10 s .. 10 s + 9 row s: slots
        // 0-7 the body chunks, 8 the left and 9 the right halo); other tiles point by point
        if (x0 + kUp0X <= rin.n[0] && ((rin.sy | rin.sz) & 3) == 0 &&
            (reinterpret_cast<uintptr_t>(rin.a) & 15) == 0) {
            const int u = lane % 10, sub = lane / 10;
            const int hxo = u == 8 ? mx[0] : (u == 9 ? mx[kUp0HX - 1] : -1);
            for (int row0 = 3 * wp; row0 < kUp0HY * kUp0HZ; row0 += 3 * kWarps) {
                const int row = row0 + sub;
                if (sub < 3 && row < kUp0HY * kUp0HZ) {
                    const int oyz = myz[row];
                    float* dst = &t[b][row * kUp0P];
                    if (u < 8) {
                        cp_async_16(dst + kUp0O + 1 + 4 * u, oyz >= 0 ? rin.a + oyz + x0 + 4 * u : rin.a, oyz >= 0);
                    } else {
                        const bool ok = hxo >= 0 && oyz >= 0;
                        cp_async_f32(dst + (u == 8 ? kUp0O : kUp0O + kUp0HX - 1), ok ? rin.a + hxo + oyz : rin.a, ok);
                    }
                }
            }
        } else {
            // lane l the row's point l (lanes 0, 1 also 32, 33): the x offsets stay in registers and
            // each row costs one shared read of its y/z offset
            const int ox0 = mx[lane], ox1 = lane < kUp0HX - 32 ? mx[32 + lane] : -1;
            for (int row = wp; row < kUp0HY * kUp0HZ; row += kWarps) {
                const int oyz = myz[row];
                float* dst = &t[b][row * kUp0P + kUp0O];
                const bool ok0 = ox0 >= 0 && oyz >= 0;
                cp_async_f32(dst + lane, ok0 ? rin.a + ox0 + oyz : rin.a, ok0);
                if (lane < kUp0HX - 32) {
                    const bool ok1 = ox1 >= 0 && oyz >= 0;
                    cp_async_f32(dst + 32 + lane, ok1 ? rin.a + ox1 + oyz : rin.a, ok1);
                }
            }
        }
        if (cin.a) {
            const int cox = lane < kPcX ? cmx[lane] : -1;
            for (int row = wp; row < kPcY * kPcZ; row += kWarps) {
                const int oyz = cmyz[row];
                if (lane < kPcX) {
                    const bool ok = cox >= 0 && oyz >= 0;
                    cp_async_f32(&pc[b][row * kPcX + lane], ok ? cin.a + cox + oyz : cin.a, ok);
                }
            }
        }
        {
            // q at the tile's outputs (16-byte copies of whole 32-point row segments when aligned),
            // and the FREE word of each output row (zero outside the grid)
            if (q && x0 + kUp0X <= g.ni && (g.ni & 3) == 0 && (reinterpret_cast<uintptr_t>(q) & 15) == 0) {
#pragma unroll
                for (int j = 0; j < kUp0Z * kUp0Y * kUp0X / 4 / kThr; j++) {
                    const int c = tid + j * kThr, seg = c / (kUp0X / 4), u = c % (kUp0X / 4);
                    const int k = seg / kUp0Y, ty = seg % kUp0Y, y = y0 + ty, zz = z0 + k;
                    const bool ok = y < g.nj && zz < g.nk;
                    cp_async_16(&qs[b][k][ty * kUp0X + 4 * u], ok ? q + (x0 + 4 * u + y * g.ni + zz * g.ni * g.nj) : q, ok);
                }
            } else {
                const int x = x0 + tx;
#pragma unroll
                for (int h = 0; h < R; h++) {
                    const int ty = ty0 + h, y = y0 + ty;
                    const bool col = x < g.ni && y < g.nj;
#pragma unroll
                    for (int k = 0; k < kUp0Z; k++) {
                        const int zz = z0 + k;
                        const bool ok = q && col && zz < g.nk;
                        cp_async_f32(&qs[b][k][ty * kUp0X + tx], ok ? q + (x + y * g.ni + zz * g.ni * g.nj) : rin.a, ok);
                    }
                }
            }
            if (tid < kUp0Z * kUp0Y) {
                const int k = tid / kUp0Y, yy = y0 + tid % kUp0Y, zz = z0 + k;
                const bool ok = yy < g.nj && zz < g.nk;
                cp_async_f32(reinterpret_cast<float*>(&fm[b][tid]),
                             ok ? reinterpret_cast<const float*>(g.free_bits + ((zz * g.nj + yy) * g.free_wpr + (x0 >> 5)))
                                : rin.a,
                             ok);
            }
        }
        cp_async_commit();
    };
    int tile = blockIdx.x;
    if (tile < ntiles) issue(tile, 0);  // its barrier also publishes S
    float w[27];  // R = 2 only (unused and removed for R = 1)
#pragma unroll
    for (int m = 0; m < 27; m++) w[m] = S[m];
    float f_zr = 0.f, f_zq = 0.f;
    for (int b = 0; tile < ntiles; tile += gridDim.x, b ^= 1) {
        const int next = tile + gridDim.x;
        __syncthreads();  // every thread is done with the other buffer and with the maps
        if (next < ntiles) issue(next, b ^ 1);
        int bb = tile;
        const int bx = bb % bx_n;
        bb /= bx_n;
        const int by = bb % by_n, bz = bb / by_n;
        const int x0 = bx * kUp0X, y0 = by * kUp0Y, z0 = bz * kUp0Z;
        const int x = x0 + tx;
        bool colr[R];
#pragma unroll
        for (int h = 0; h < R; h++) colr[h] = x < g.ni && y0 + ty0 + h < g.nj;
        if (next < ntiles)
            cp_async_wait<1>();
        else
            cp_async_wait<0>();
        __syncthreads();  // this tile's copies of every thread have landed
        const float* T = t[b];
        const float* PC = pc[b];
        // prolongation weights (0.75 own coarse point, 0.25 the neighbour on the parity side): the
        // x-y interpolation of the six coarse planes for each row (an even row takes the coarse
        // row below, an odd row the one above), then per output plane the two planes on its parity
        // side
        float px[R][kPcZ];
        if (cin.a) {
            const int lx = (x >> 1) - (x0 / 2 - 1);
            const int sx = (x & 1) ? 1 : -1;
#pragma unroll
            for (int h = 0; h < R; h++) {
                const int ty = ty0 + h, ly = ty / 2 + 1, sy = (ty & 1) ? 1 : -1;  // y0 is even
#pragma unroll
                for (int cz = 0; cz < kPcZ; cz++) {
                    auto C = [&](int cy, int cx) { return PC[(cz * kPcY + cy) * kPcX + cx]; };
                    const float a0 = 0.75f * C(ly, lx) + 0.25f * C(ly, lx + sx);
                    const float a1 = 0.75f * C(ly + sy, lx) + 0.25f * C(ly + sy, lx + sx);
                    px[h][cz] = 0.75f * a0 + 0.25f * a1;
                }
            }
        }
        float Pr[R], Qr[R];
#pragma unroll
        for (int h = 0; h < R; h++) Pr[h] = Qr[h] = 0.f;
#pragma unroll
        for (int hz = 0; hz < kUp0HZ; hz++) {
            float rr[R + 2][3];
#pragma unroll
            for (int dy = 0; dy < R + 2; dy++)
#pragma unroll
                for (int dx = 0; dx < 3; dx++) rr[dy][dx] = T[(hz * kUp0HY + ty0 + dy) * kUp0P + kUp0O + tx + dx];
            float a0[R], a1[R], a2[R];
#pragma unroll
            for (int h = 0; h < R; h++) a0[h] = a1[h] = a2[h] = 0.f;
#pragma unroll
            for (int dy = 0; dy < 3; dy++)
#pragma unroll
                for (int dx = 0; dx < 3; dx++) {
                    const int m = 3 * dy + dx;
                    // R = 2: weights in registers; R = 1: from shared memory (64 registers)
                    const float w0 = R == 2 ? w[m] : S[m], w1 = R == 2 ? w[9 + m] : S[9 + m],
                                w2 = R == 2 ? w[18 + m] : S[18 + m];
#pragma unroll
                    for (int h = 0; h < R; h++) {
                        a0[h] = fmaf(w0, rr[dy + h][dx], a0[h]);
                        a1[h] = fmaf(w1, rr[dy + h][dx], a1[h]);
                        a2[h] = fmaf(w2, rr[dy + h][dx], a2[h]);
                    }
                }
            const int k = hz - 2;  // output plane z0 + k is complete after tile plane hz = k + 2
            if (k >= 0 && z0 + k < g.nk) {
                // z0 is even: output plane k sits over coarse plane 1 + k/2, parity side k & 1
                const int lz = 1 + (k >> 1), sz = (k & 1) ? 1 : -1;
#pragma unroll
                for (int h = 0; h < R; h++) {
                    const int ty = ty0 + h;
                    if (!colr[h]) continue;
                    const int n = x + (y0 + ty) * g.ni + (z0 + k) * g.ni * g.nj;
                    if (fm[b][k * kUp0Y + ty] >> tx & 1u) {
                        float v = Pr[h] + a2[h];
                        if (cin.a) v += 0.75f * px[h][lz] + 0.25f * px[h][lz + sz];
                        z[n] = v;
                        f_zr += v * T[((k + 1) * kUp0HY + ty + 1) * kUp0P + kUp0O + tx + 1];
                        f_zq += v * qs[b][k][ty * kUp0X + tx];
                    } else {
                        z[n] = 0.f;
                    }
                }
            }
#pragma unroll
            for (int h = 0; h < R; h++) {
                Pr[h] = Qr[h] + a1[h];
                Qr[h] = a0[h];
            }
        }
    }
    if (out) {
        const float vv[2] = {f_zr, f_zq};
        grid_sum<2>(vv, gpart, gstride, ticket, out);
    }
}
// A network level's operator e = op(z) + P e_coarse on 3-D tiles of 32 x 8 x 8 voxels: the z tile with
// its two-voxel halo (36 x 12 x 12) is staged in shared memory with all loads in flight, and a
// thread rolls the five 5 x 5 plane sums of each tile plane into its column's eight outputs.
// Points on a non-periodic face take the exact face-class form through lp_net_op.
constexpr int kNetX = 32, kNetY = 8, kNetZ = 8;
constexpr int kNetHX = kNetX + 4, kNetHY = kNetY + 4, kNetHZ = kNetZ + 4;
struct K5Param {
    float k[125];
};
__global__ void __launch_bounds__(kNetX * kNetY, 2) k_lp_up_net_tiled(LView zin, LView cin, LView out,
                                                                    const float* __restrict__ fold_g, const int* flag,
                                                                    int bx_n, int by_n, K5Param K5p) {
    if (flag && flag[0]) return;
    // K5p.k is indexed with compile-time offsets only, so every coefficient is an FMA operand from
    // the constant bank (a pointer into the parameter would copy it to local memory)
    __shared__ float t[kNetHZ][kNetHY][kNetHX];
    __shared__ int mx[kNetHX], myz[kNetHY * kNetHZ];  // halo offsets per axis (-1: outside)
    const int tx = threadIdx.x % kNetX, ty = threadIdx.x / kNetX;
    int b = blockIdx.x;
    const int bx = b % bx_n;
    b /= bx_n;
    const int by = b % by_n, bz = b / by_n;
    const int x0 = bx * kNetX, y0 = by * kNetY, z0 = bz * kNetZ;
    if (threadIdx.x < kNetHX) mx[threadIdx.x] = lv_map(x0 - 2 + (int)threadIdx.x, zin.n[0], zin.per[0]);
    if (threadIdx.x < kNetHY * kNetHZ) {
        const int uy = lv_map(y0 - 2 + (int)threadIdx.x % kNetHY, zin.n[1], zin.per[1]);
        const int uz = lv_map(z0 - 2 + (int)threadIdx.x / kNetHY, zin.n[2], zin.per[2]);
        myz[threadIdx.x] = (uy < 0 || uz < 0) ? -1 : uy * zin.sy + uz * zin.sz;
    }
    // the coarse tile of the prolongation (the fine level's tile rules: wrapped or zero outside)
    __shared__ float pc[kPcZ][kPcY][kPcX];
    __shared__ int cmx[kPcX], cmyz[kPcY * kPcZ];
    if (cin.a) {
        if (threadIdx.x < kPcX) cmx[threadIdx.x] = lv_map(x0 / 2 - 1 + (int)threadIdx.x, cin.n[0], cin.per[0]);
        if (threadIdx.x < kPcY * kPcZ) {
            const int uy = lv_map(y0 / 2 - 1 + (int)threadIdx.x % kPcY, cin.n[1], cin.per[1]);
            const int uz = lv_map(z0 / 2 - 1 + (int)threadIdx.x / kPcY, cin.n[2], cin.per[2]);
            cmyz[threadIdx.x] = (uy < 0 || uz < 0) ? -1 : uy * cin.sy + uz * cin.sz;
        }
    }
    __syncthreads();
    stage_tile<kNetHX, kNetHY * kNetHZ, kNetX * kNetY>(&t[0][0][0], zin.a, mx, myz);
    if (cin.a) stage_tile<kPcX, kPcY * kPcZ, kNetX * kNetY>(&pc[0][0][0], cin.a, cmx, cmyz);
    const int x = x0 + tx, y = y0 + ty;
    const bool col = x < out.n[0] && y < out.n[1];
    __syncthreads();
    // prolongation: the x-y interpolation of this column's six coarse planes (kept in shared
    // memory, one slot per thread, as the plane loop below indexes it at run time), then per output
    // plane the two planes on its parity side (z0 is even)
    static_assert(kNetX == kUp0X && kNetY == kUp0Y && kNetZ == kUp0Z, "the coarse tile follows the fine tile");
    __shared__ float pxy[kPcZ][kNetX * kNetY];
    {
        const int lx = (x >> 1) - (x0 / 2 - 1), ly = (y >> 1) - (y0 / 2 - 1);
        const int sx = (x & 1) ? 1 : -1, sy = (y & 1) ? 1 : -1;
#pragma unroll
        for (int cz = 0; cz < kPcZ; cz++) {
            float v = 0.f;
            if (cin.a) {
                const float a0 = 0.75f * pc[cz][ly][lx] + 0.25f * pc[cz][ly][lx + sx];
                const float a1 = 0.75f * pc[cz][ly + sy][lx] + 0.25f * pc[cz][ly + sy][lx + sx];
                v = 0.75f * a0 + 0.25f * a1;
            }
            pxy[cz][threadIdx.x] = v;
        }
    }
    // rolling window: w[j] collects output plane hz - 4 + j; tile plane hz is offset dz - 2 of
    // output plane hz - dz, i.e. w[4 - dz].  Only the taps whose output plane lies in the tile are
    // formed: dz from max(0, hz - 7) to min(4, hz) (40 of the 60 plane-tap pairs), with the ranges
    // of the four first and four last planes fixed at compile time
    float w[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    auto plane = [&](auto d0c, auto d1c, int hz) {
        constexpr int d0 = decltype(d0c)::value, d1 = decltype(d1c)::value;
        float a[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
        float win[25];  // the plane's 5 x 5 window, loaded once
#pragma unroll
        for (int dy = 0; dy < 5; dy++)
#pragma unroll
            for (int dx = 0; dx < 5; dx++) win[5 * dy + dx] = t[hz][ty + dy][tx + dx];
#pragma unroll
        for (int m = 0; m < 25; m++)
#pragma unroll
            for (int dz = d0; dz <= d1; dz++) a[dz] = fmaf(K5p.k[25 * dz + m], win[m], a[dz]);
#pragma unroll
        for (int dz = d0; dz <= d1; dz++) w[4 - dz] += a[dz];
        const int k = hz - 4;  // output plane z0 + k is complete
        if (k >= 0 && col && z0 + k < out.n[2]) {
            const int c[3] = {x, y, z0 + k};
            // a point on a non-periodic face takes the 5 x 5 x 5 variant of its face class (the
            // network's first-stage taps outside the box left out), applied to the same staged
            // window: the tile holds zero outside the box and the wrap on periodic axes
            int cls = 0, mul = 1;
#pragma unroll
            for (int ax = 0; ax < 3; ax++) {
                if (!zin.per[ax]) cls += mul * (c[ax] == 0 ? 1 : (c[ax] == zin.n[ax] - 1 ? 2 : 0));
                mul *= 3;
            }
            float v = w[0];
            if (cls) {
                const float* __restrict__ K5v = fold_g + kLpFold + 125 * cls;
                v = 0.f;
                for (int dz = 0; dz < 5; dz++)
#pragma unroll
                    for (int m = 0; m < 25; m++) v = fmaf(K5v[25 * dz + m], t[k + dz][ty + m / 5][tx + m % 5], v);
            }
            // z0 is even: output plane k sits over coarse plane 1 + k/2, parity side k & 1
            const int lz = 1 + (k >> 1), sz = (k & 1) ? 1 : -1;
            out.a[lv_off(out, x, y, z0 + k)] = v + (0.75f * pxy[lz][threadIdx.x] + 0.25f * pxy[lz + sz][threadIdx.x]);
        }
#pragma unroll
        for (int j2 = 0; j2 < 4; j2++) w[j2] = w[j2 + 1];
        w[4] = 0.f;
    };
    using I0 = std::integral_constant<int, 0>;
    using I4 = std::integral_constant<int, 4>;
    static_assert(kNetHZ == 12 && kNetZ == 8, "the tap ranges below follow the 8-plane tile");
    plane(I0{}, I0{}, 0);
    plane(I0{}, std::integral_constant<int, 1>{}, 1);
    plane(I0{}, std::integral_constant<int, 2>{}, 2);
    plane(I0{}, std::integral_constant<int, 3>{}, 3);
#pragma unroll 1
    for (int hz = 4; hz < 8; hz++) plane(I0{}, I4{}, hz);
    plane(std::integral_constant<int, 1>{}, I4{}, 8);
    plane(std::integral_constant<int, 2>{}, I4{}, 9);
    plane(std::integral_constant<int, 3>{}, I4{}, 10);
    plane(I4{}, I4{}, 11);
}

// index rule of the restriction along one axis (k_lp_restrict): fine point raw of coarse level c,
// wrapped once by the coarse period on a periodic axis; -1 outside the fine box
__device__ __forceinline__ int rs_map(int raw, const LView& f, const LView& c, int ax) {
    if (f.per[ax]) {
        const int nc2 = 2 * c.n[ax];
        raw = raw < 0 ? raw + nc2 : (raw >= nc2 ? raw - nc2 : raw);
        return raw < f.n[ax] ? raw : -1;
    }
    return (raw >= 0 && raw < f.n[ax]) ? raw : -1;
}
// z_coarse = R z_fine, one warp per column of 32 x 4 x 4 coarse voxels, all in registers.  Lane l
// owns coarse x = cx0 + l.  The warp marches through the column's ten fine planes; in each it
// reads the ten fine rows of the column, lane l taking fine x 2cx and 2cx + 1 as one float2 (a
// warp reads 64 consecutive fine points) and fine x 2cx - 1 and 2cx + 2 from its neighbour lanes
// (x pass), combines four rows per coarse y (y pass) and adds the plane into the two coarse planes
// it is a tap of (z pass).  The two halo points of a row (fine x 2 cx0 - 1 and 2 cx0 + 64, read by
// lanes 0 and 31) follow the index rules of k_lp_restrict (outside the box or wrapped); a column
// whose 64 body points leave the box or wrap, or a level whose rows are not 8-byte aligned, reads
// four mapped points per lane instead.
constexpr int kRmX = 32, kRmY = 4, kRmZ = 4;
constexpr int kRmHY = 2 * kRmY + 2, kRmHZ = 2 * kRmZ + 2;
constexpr int kRmWarps = 4;  // warps per CTA
__global__ void __launch_bounds__(32 * kRmWarps, 4) k_lp_restrict_march(LView f, LView c, const int* flag, int bx_n,
                                                                      int by_n, int nwarps) {
    if (flag && flag[0]) return;
    const int gw = (int)blockIdx.x * kRmWarps + (int)(threadIdx.x >> 5);
    if (gw >= nwarps) return;  // whole warps
    const int lane = threadIdx.x & 31;
    int b = gw;
    const int bx = b % bx_n;
    b /= bx_n;
    const int by = b % by_n, bz = b / by_n;
    const int cx0 = bx * kRmX, cy0 = by * kRmY, cz0 = bz * kRmZ;
    const int fx = 2 * (cx0 + lane);  // this lane's even fine x
    const int body_end = 2 * cx0 + 2 * kRmX;
    // the body may reach one point past the view when the row's storage holds it (a periodic node
    // array keeps its alias node there); the index rules give that point zero (no wrap below the
    // coarse period 2 c.n), so its value is read and replaced by zero
    const bool fast = (body_end <= f.n[0] || (body_end == f.n[0] + 1 && f.sy >= body_end)) &&
                      (!f.per[0] || body_end <= 2 * c.n[0]) && ((f.sy | f.sz) & 1) == 0 &&
                      (reinterpret_cast<uintptr_t>(f.a) & 7) == 0;
    const bool hi_out = fx + 1 >= f.n[0];  // fast path: this lane's odd point is past the view
    // fast: xo[0] is the halo of lane 0 or 31 (-1: none); otherwise the four mapped fine x
    int xo[4];
    if (fast) {
        xo[0] = lane == 0 ? rs_map(2 * cx0 - 1, f, c, 0) : (lane == 31 ? rs_map(body_end, f, c, 0) : -1);
        xo[1] = xo[2] = xo[3] = -1;
    } else {
#pragma unroll
        for (int k = 0; k < 4; k++) xo[k] = rs_map(fx - 1 + k, f, c, 0);
    }
    // fine row offsets of the column's y range; a row outside the box reads row 0 and is dropped
    int oy[kRmHY];
    bool my[kRmHY];
#pragma unroll
    for (int r = 0; r < kRmHY; r++) {
        const int u = rs_map(2 * cy0 - 1 + r, f, c, 1);
        oy[r] = u < 0 ? 0 : u * f.sy;
        my[r] = u >= 0;
    }
    const float w4[4] = {0.25f, 0.75f, 0.75f, 0.25f};
    float acc[kRmZ][kRmY];
#pragma unroll
    for (int cz = 0; cz < kRmZ; cz++)
#pragma unroll
        for (int cy = 0; cy < kRmY; cy++) acc[cz][cy] = 0.f;
    // straight-line over the planes (no branch between the loads of consecutive planes), so that
    // the next planes' rows are in flight while one is combined
#pragma unroll
    for (int pz = 0; pz < kRmHZ; pz++) {
        const int uz = rs_map(2 * cz0 - 1 + pz, f, c, 2);
        const float* plane = f.a + (size_t)(uz < 0 ? 0 : uz) * f.sz;
        const bool mz = uz >= 0;
        float xv[kRmHY];
        if (fast) {
            float2 pv[kRmHY];
            float ph[kRmHY];
#pragma unroll
            for (int r = 0; r < kRmHY; r++) {
                pv[r] = *reinterpret_cast<const float2*>(plane + oy[r] + fx);
                if (hi_out) pv[r].y = 0.f;
                ph[r] = xo[0] >= 0 ? plane[oy[r] + xo[0]] : 0.f;
            }
#pragma unroll
            for (int r = 0; r < kRmHY; r++) {
                float left = __shfl_up_sync(0xffffffffu, pv[r].y, 1);
                float right = __shfl_down_sync(0xffffffffu, pv[r].x, 1);
                if (lane == 0) left = ph[r];
                if (lane == 31) right = ph[r];
                xv[r] = my[r] && mz ? w4[0] * left + w4[1] * pv[r].x + w4[2] * pv[r].y + w4[3] * right : 0.f;
            }
        } else {
#pragma unroll
            for (int r = 0; r < kRmHY; r++) {
                float a[4];
#pragma unroll
                for (int k = 0; k < 4; k++) a[k] = xo[k] >= 0 ? plane[oy[r] + xo[k]] : 0.f;
                xv[r] = my[r] && mz ? w4[0] * a[0] + w4[1] * a[1] + w4[2] * a[2] + w4[3] * a[3] : 0.f;
            }
        }
        // fine plane pz is tap pz - 2 cz of coarse plane cz
#pragma unroll
        for (int cz = 0; cz < kRmZ; cz++) {
            const int k = pz - 2 * cz;
            if (k < 0 || k > 3) continue;
#pragma unroll
            for (int cy = 0; cy < kRmY; cy++) {
                const float yv = w4[0] * xv[2 * cy] + w4[1] * xv[2 * cy + 1] + w4[2] * xv[2 * cy + 2] +
                                 w4[3] * xv[2 * cy + 3];
                acc[cz][cy] += w4[k] * yv;
            }
        }
    }
    const int cx = cx0 + lane;
    if (cx >= c.n[0]) return;
#pragma unroll
    for (int cz = 0; cz < kRmZ; cz++)
#pragma unroll
        for (int cy = 0; cy < kRmY; cy++)
            if (cy0 + cy < c.n[1] && cz0 + cz < c.n[2]) c.a[lv_off(c, cx, cy0 + cy, cz0 + cz)] = acc[cz][cy];
}

// z_coarse = R z_fine on 3-D tiles of 16 x 8 x 4 coarse voxels: the 34 x 18 x 10 fine points they
// read are staged in shared memory first (the same index rules as k_lp_restrict).  For the mid-size
// levels: with fewer than ~10^6 coarse voxels the marching kernel has too few warps for its chains
// of planes.
constexpr int kRsX = 16, kRsY = 8, kRsZ = 4;
constexpr int kRsHX = 2 * kRsX + 2, kRsHY = 2 * kRsY + 2, kRsHZ = 2 * kRsZ + 2;
__global__ void __launch_bounds__(256) k_lp_restrict_tiled(LView f, LView c, const int* flag, int bx_n, int by_n) {
    if (flag && flag[0]) return;
    __shared__ float t[kRsHZ][kRsHY][kRsHX];
    __shared__ int mx[kRsHX], myz[kRsHY * kRsHZ];  // fine offsets per axis (-1: outside)
    int b = blockIdx.x;
    const int bx = b % bx_n;
    b /= bx_n;
    const int by = b % by_n, bz = b / by_n;
    const int cx0 = bx * kRsX, cy0 = by * kRsY, cz0 = bz * kRsZ;
    const int tid = threadIdx.x;
    if (tid < kRsHX) mx[tid] = rs_map(2 * cx0 - 1 + tid, f, c, 0);
    if (tid < kRsHY * kRsHZ) {
        const int uy = rs_map(2 * cy0 - 1 + tid % kRsHY, f, c, 1);
        const int uz = rs_map(2 * cz0 - 1 + tid / kRsHY, f, c, 2);
        myz[tid] = (uy < 0 || uz < 0) ? -1 : uy * f.sy + uz * f.sz;
    }
    __syncthreads();
    stage_tile<kRsHX, kRsHY * kRsHZ, 256>(&t[0][0][0], f.a, mx, myz);
    __syncthreads();
    const float w4[4] = {0.25f, 0.75f, 0.75f, 0.25f};
    for (int o = threadIdx.x; o < kRsX * kRsY * kRsZ; o += 256) {
        const int ox = o % kRsX, oy = (o / kRsX) % kRsY, oz = o / (kRsX * kRsY);
        const int cx = cx0 + ox, cy = cy0 + oy, cz = cz0 + oz;
        if (cx >= c.n[0] || cy >= c.n[1] || cz >= c.n[2]) continue;
        float acc = 0.f;
#pragma unroll
        for (int kz = 0; kz < 4; kz++) {
            float az = 0.f;
#pragma unroll
            for (int ky = 0; ky < 4; ky++) {
                const float* row = &t[2 * oz + kz][2 * oy + ky][2 * ox];
                az += w4[ky] * (w4[0] * row[0] + w4[1] * row[1] + w4[2] * row[2] + w4[3] * row[3]);
            }
            acc += w4[kz] * az;
        }
        c.a[lv_off(c, cx, cy, cz)] = acc;
    }
}

// z = B r on the finest level: the tiled kernel when its CTAs fit the reduction's partial slots
static void launch_up0(const GridDev& g, LView r0, LView cin, float* z, const uint16_t* kind, const float* S0,
                       const float* q, double* gpart, int gstride, unsigned* ticket, double* out, const int* flag,
                       cudaStream_t s, int sms) {
    const int bx_n = (g.ni + kUp0X - 1) / kUp0X, by_n = (g.nj + kUp0Y - 1) / kUp0Y;
    const long tiles = (long)bx_n * by_n * ((g.nk + kUp0Z - 1) / kUp0Z);
    const long ctas = std::min(tiles, (long)std::max(1, sms) * kUp0CtasPerSM);
    if (!out || ctas <= gstride) {
        static int dyn_set = -1;  // the device whose attributes are set (one device per process here)
        int dev = 0;
        cudaGetDevice(&dev);
        if (dyn_set != dev) {
            cudaFuncSetAttribute(k_lp_up0_pipe<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUp0DynSmem);
            cudaFuncSetAttribute(k_lp_up0_pipe<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, kUp0DynSmem);
            dyn_set = dev;
        }
        if (tiles >= 4 * (long)std::max(1, sms) * kUp0CtasPerSM)
            k_lp_up0_pipe<2><<<(unsigned)ctas, kUp0X * kUp0Y / 2, kUp0DynSmem, s>>>(
                g, r0, cin, z, kind, S0, q, gpart, gstride, ticket, out, flag, bx_n, by_n, (int)tiles);
        else
            k_lp_up0_pipe<1><<<(unsigned)ctas, kUp0X * kUp0Y, kUp0DynSmem, s>>>(
                g, r0, cin, z, kind, S0, q, gpart, gstride, ticket, out, flag, bx_n, by_n, (int)tiles);
    } else {
        k_lp_up0<<<node_blocks(g.nv), kNodeThreads, 0, s>>>(g, r0, cin, z, kind, S0, q, gpart, gstride, ticket, out,
                                                            flag);
    }
}

// one thread per voxel of a level
static int lp_blocks(int nvox, int sms) {
    (void)sms;
    return std::max(1, (nvox + 255) / 256);
}
// per level the fastest of three forms (ncu launch lists of the large discharge): the marching
// kernel from 2^20 coarse voxels (level 1: 45 against 62 us for the tiled one), the tiled kernel
// from 32^3 (levels 2-3: 12 and 5 us against 14-15 us marching), one thread per voxel below
static void launch_restrict(const LView& f, const LView& c, const int* flag, cudaStream_t s, int sms) {
    if (c.nvox >= (1 << 20)) {
        const int bx_n = (c.n[0] + kRmX - 1) / kRmX, by_n = (c.n[1] + kRmY - 1) / kRmY;
        const int nwarps = bx_n * by_n * ((c.n[2] + kRmZ - 1) / kRmZ);
        k_lp_restrict_march<<<(nwarps + kRmWarps - 1) / kRmWarps, 32 * kRmWarps, 0, s>>>(f, c, flag, bx_n, by_n,
                                                                                         nwarps);
    } else if (c.nvox >= 32 * 32 * 32) {
        const int bx_n = (c.n[0] + kRsX - 1) / kRsX, by_n = (c.n[1] + kRsY - 1) / kRsY;
        const int blocks = bx_n * by_n * ((c.n[2] + kRsZ - 1) / kRsZ);
        k_lp_restrict_tiled<<<blocks, 256, 0, s>>>(f, c, flag, bx_n, by_n);
    } else {
        k_lp_restrict<<<lp_blocks(c.nvox, sms), 256, 0, s>>>(f, c, flag);
    }
}

void launch_lp_apply(const GridDev& g, const LpState& L, const float* r, float* z, const uint16_t* kind,
                     const float* q, const SolveWork* red, const int* flag, cudaStream_t s, int sms) {
    LView r0 = lp_node_view(g, L, const_cast<float*>(r));
    // the first level of the fused coarse chain: every level from it down is small, and a network
    // level only when it is tiny (one CTA is too little parallelism for the folded stencil above)
    int l0 = L.nlev;
    while (l0 > 1) {
        const long nv_l = (long)L.dims[l0 - 1][0] * L.dims[l0 - 1][1] * L.dims[l0 - 1][2];
        if (nv_l > kLpCoarseMaxVox || (l0 - 1 <= kLpNetLevels && nv_l > kLpCoarseMaxNetVox)) break;
        l0--;
    }
    for (int l = 1; l < l0; l++) {
        LView f = l == 1 ? r0 : lp_level_view(L, l - 1, L.z[l - 1]);
        LView c = lp_level_view(L, l, L.z[l]);
        launch_restrict(f, c, flag, s, sms);
    }
    if (l0 < L.nlev) {
        LpCoarseArgs ca{};
        ca.l0 = l0;
        ca.nlev = L.nlev;
        ca.f0 = l0 == 1 ? r0 : lp_level_view(L, l0 - 1, L.z[l0 - 1]);
        for (int l = l0; l < L.nlev; l++) {
            ca.z[l] = lp_level_view(L, l, L.z[l]);
            ca.e[l] = lp_level_view(L, l, L.e[l]);
            ca.mode[l] = l <= kLpNetLevels ? 1 : 2;
            ca.fold[l] = ca.mode[l] == 1 ? L.fold + (l - 1) * kLpFoldStride : nullptr;
            ca.inv_diag[l] = (float)(1.0 / L.diag[l]);
        }
        k_lp_coarse<<<1, kLpCoarseThreads, 0, s>>>(ca, flag);
    }
    LView none{};
    none.a = nullptr;
    if (!L.k5_valid) {
        const int nnet = std::min(kLpNetLevels, L.nlev - 1);
        for (int l = 1; l <= nnet; l++)
            cudaMemcpyAsync(L.k5_host[l - 1], L.fold + (l - 1) * kLpFoldStride + 729, sizeof(float) * 125,
                            cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        L.k5_valid = true;
    }
    for (int l = l0 - 1; l >= 1; l--) {
        LView zin = lp_level_view(L, l, L.z[l]);
        LView cin = l + 1 < L.nlev ? lp_level_view(L, l + 1, L.e[l + 1]) : none;
        LView out = lp_level_view(L, l, L.e[l]);
        int mode = l <= kLpNetLevels ? 1 : 2;
        const float* fold = mode == 1 ? L.fold + (l - 1) * kLpFoldStride : nullptr;
        // the tiled kernel once every axis has at least 8 points (its halo wraps at most once);
        // below that one thread per voxel
        if (mode == 1 && out.n[0] >= 8 && out.n[1] >= 8 && out.n[2] >= 8) {
            const int bx_n = (out.n[0] + kNetX - 1) / kNetX, by_n = (out.n[1] + kNetY - 1) / kNetY;
            const int blocks = bx_n * by_n * ((out.n[2] + kNetZ - 1) / kNetZ);
            K5Param k5;
            std::memcpy(k5.k, L.k5_host[l - 1], sizeof(k5.k));
            k_lp_up_net_tiled<<<blocks, kNetX * kNetY, 0, s>>>(zin, cin, out, fold, flag, bx_n, by_n, k5);
        } else {
            k_lp_up<<<lp_blocks(out.nvox, sms), 256, 0, s>>>(zin, cin, out, mode, fold, (float)(1.0 / L.diag[l]),
                                                             flag);
        }
    }
    LView cin = L.nlev > 1 ? lp_level_view(L, 1, L.e[1]) : none;
    launch_up0(g, r0, cin, z, kind, L.W + L.lay.s0, q, red ? red->gpart : nullptr, red ? red->gstride : 0,
               red ? red->ticket : nullptr, red ? red->scal + kS_RZN : nullptr, flag, s, sms);
}

// folded stencils of every network level: M = Wm Wl (C x 27), K27[t][t'] = sum_c Wp[t][c] M[c][t'],
// K5[d] = sum over t + t' = d of K27[t][t']
__global__ void k_lp_fold(const float* __restrict__ W, LpLayout lay, float* fold) {
    const int l = blockIdx.x + 1;
    const int C = lp_channels(l);
    __shared__ float M[64 * 27];
    __shared__ float K[729];
    const float* Wl = W + lay.wl[l];
    const float* Wm = W + lay.wm[l];
    const float* Wp = W + lay.wp[l];
    for (int x = threadIdx.x; x < C * 27; x += blockDim.x) {
        int c = x / 27, t = x % 27;
        float a = 0.f;
        for (int k = 0; k < C; k++) a += Wm[c * C + k] * Wl[k * 27 + t];
        M[x] = a;
    }
    __syncthreads();
    for (int x = threadIdx.x; x < 729; x += blockDim.x) {
        int t = x / 27, tp = x % 27;
        float a = 0.f;
        for (int c = 0; c < C; c++) a += Wp[t * C + c] * M[c * 27 + tp];
        K[x] = a;
        fold[(l - 1) * kLpFoldStride + x] = a;
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 125; d += blockDim.x) {
        int dx = d % 5 - 2, dy = (d / 5) % 5 - 2, dz = d / 25 - 2;
        float a = 0.f;
        for (int t = 0; t < 27; t++) {
            int tx = t % 3 - 1, ty = (t / 3) % 3 - 1, tz = t / 9 - 1;
            int ux = dx - tx, uy = dy - ty, uz = dz - tz;
            if (ux < -1 || ux > 1 || uy < -1 || uy > 1 || uz < -1 || uz > 1) continue;
            a += K[t * 27 + 9 * (uz + 1) + 3 * (uy + 1) + ux + 1];
        }
        fold[(l - 1) * kLpFoldStride + 729 + d] = a;
    }
    // face-class variants: only the first-stage taps t whose point c + o_t stays inside the box
    for (int x = threadIdx.x; x < 27 * 125; x += blockDim.x) {
        const int cls = x / 125, d = x % 125;
        const int cl[3] = {cls % 3, (cls / 3) % 3, cls / 9};
        const int dd[3] = {d % 5 - 2, (d / 5) % 5 - 2, d / 25 - 2};
        float a = 0.f;
        for (int t = 0; t < 27; t++) {
            const int ot[3] = {t % 3 - 1, (t / 3) % 3 - 1, t / 9 - 1};
            bool ok = true;
            int u[3];
            for (int ax = 0; ax < 3; ax++) {
                if ((cl[ax] == 1 && ot[ax] == -1) || (cl[ax] == 2 && ot[ax] == 1)) ok = false;
                u[ax] = dd[ax] - ot[ax];
                if (u[ax] < -1 || u[ax] > 1) ok = false;
            }
            if (ok) a += K[t * 27 + 9 * (u[2] + 1) + 3 * (u[1] + 1) + u[0] + 1];
        }
        fold[(l - 1) * kLpFoldStride + kLpFold + x] = a;
    }
}
void launch_lp_fold(const LpState& L, cudaStream_t s) {
    L.k5_valid = false;
    int nnet = std::min(kLpNetLevels, L.nlev - 1);
    if (nnet > 0) k_lp_fold<<<nnet, 256, 0, s>>>(L.W, L.lay, L.fold);
}

// =====================================================================================
// flexible CG with the learned preconditioner, FP32 on the correction equation L e = r
//   init : z = B r ; partials z.r
//   K1   : beta = -alpha_prev (z.q_prev) / rz_prev (0 on the first iteration); d' = z + beta d ;
//          q = L d' ; partial d'.q
//   K2   : alpha = rz / d'q ; e += alpha d' ; r -= alpha q ; partial r.r
//   B    : z = B r ; partials z.r, z.q            (beta = z.(r_new - r_old) / rz_prev)
// scal[0..1] rz and scal[2..3] alpha, double-buffered by iteration parity
// =====================================================================================
// d' = z + beta d and q = L d' for the four nodes n0 .. n0 + 3 of a row, from d' at the row (C), at
// its neighbour rows (N: -y, +y, -z, +z), at its x ends (xm, xp) and the node kinds: writes d' and
// q there and adds d'.q to acc (the rules of spmv_group: non-FREE nodes give zero, a flagged
// neighbour is left out of the stencil, on a periodic row node ni-2 takes node 0 as +x neighbour)
__device__ __forceinline__ void cg_row4(const float (&c3)[3], int n0, bool xend, bool wrapx, const float (&C)[4],
                                        const float (&N)[4][4], float xm, float xp, ushort4 k4,
                                        float* __restrict__ d_out, float* __restrict__ q, float& acc) {
    const unsigned short kv[4] = {k4.x, k4.y, k4.z, k4.w};
    float dvo[4], qv[4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        dvo[c] = 0.f;
        qv[c] = 0.f;
        if ((kv[c] & 3) != kFree) continue;
        const float right = c == 3 ? xp : ((c == 2 && xend && wrapx) ? xp : C[c + 1]);
        const float nb[6] = {c == 0 ? xm : C[c - 1], right, N[0][c], N[1][c], N[2][c], N[3][c]};
        float dg = 0.f, o = 0.f;
#pragma unroll
        for (int d = 0; d < 6; d++) {
            if (kv[c] & (1u << (2 + d))) continue;
            dg += c3[d >> 1];
            o += c3[d >> 1] * nb[d];
        }
        dvo[c] = C[c];
        qv[c] = dg * C[c] - o;
        acc += dvo[c] * qv[c];
    }
    *reinterpret_cast<float4*>(d_out + n0) = make_float4(dvo[0], dvo[1], dvo[2], dvo[3]);
    *reinterpret_cast<float4*>(q + n0) = make_float4(qv[0], qv[1], qv[2], qv[3]);
}
// The same for rows j0 and j0 + 1 of a plane at once (rows a multiple of four nodes, the two rows
// adjacent without a periodic seam between them): the centre rows are each other's y neighbours,
// so the pair reads eight rows of z and d instead of ten, all issued before any is used.
__device__ __forceinline__ void cg_pair(const GridDev& g, int i0, int j0, int k, const float* __restrict__ z,
                                        const float* __restrict__ d_in, float* __restrict__ d_out,
                                        float* __restrict__ q, const uint16_t* __restrict__ kind, float fb,
                                        float& acc) {
    const float c3[3] = {g.inv_dx[0] * g.inv_dx[0], g.inv_dx[1] * g.inv_dx[1], g.inv_dx[2] * g.inv_dx[2]};
    const int j1 = j0 + 1;
    const int jm = g.periodic[1] ? wrap_m(j0, g.nj, 1) : max(j0 - 1, 0);
    const int jq = g.periodic[1] ? wrap_p(j1, g.nj, 1) : min(j1 + 1, g.nj - 1);
    const int km = g.periodic[2] ? wrap_m(k, g.nk, 1) : max(k - 1, 0);
    const int kp = g.periodic[2] ? wrap_p(k, g.nk, 1) : min(k + 1, g.nk - 1);
    const int na = (k * g.nj + j0) * g.ni + i0, nb = na + g.ni;
    const int off[8] = {(k * g.nj + jm) * g.ni + i0, na, nb, (k * g.nj + jq) * g.ni + i0,
                        (km * g.nj + j0) * g.ni + i0, (kp * g.nj + j0) * g.ni + i0,
                        (km * g.nj + j1) * g.ni + i0, (kp * g.nj + j1) * g.ni + i0};
    float4 zr[8], dr[8];
#pragma unroll
    for (int m = 0; m < 8; m++) {
        zr[m] = *reinterpret_cast<const float4*>(z + off[m]);
        dr[m] = *reinterpret_cast<const float4*>(d_in + off[m]);
    }
    const bool xend = i0 + 4 == g.ni, wrapx = g.periodic[0] != 0;
    float xe[4];  // x ends: row a -x, +x, row b -x, +x
#pragma unroll
    for (int r = 0; r < 2; r++) {
        const int n0 = r ? nb : na;
        const int ixm = i0 > 0 ? n0 - 1 : (wrapx ? n0 + g.ni - 2 : n0);
        const int ixp = xend ? (wrapx ? n0 - i0 : n0 + 3) : n0 + 4;
        xe[2 * r] = z[ixm] + fb * d_in[ixm];
        xe[2 * r + 1] = z[ixp] + fb * d_in[ixp];
    }
    const ushort4 ka = *reinterpret_cast<const ushort4*>(kind + na);
    const ushort4 kb = *reinterpret_cast<const ushort4*>(kind + nb);
    float v[8][4];
#pragma unroll
    for (int m = 0; m < 8; m++) {
        v[m][0] = zr[m].x + fb * dr[m].x;
        v[m][1] = zr[m].y + fb * dr[m].y;
        v[m][2] = zr[m].z + fb * dr[m].z;
        v[m][3] = zr[m].w + fb * dr[m].w;
    }
    float Na[4][4], Nb[4][4];
#pragma unroll
    for (int c = 0; c < 4; c++) {
        Na[0][c] = v[0][c];  // row a: -y jm, +y row b, -z, +z
        Na[1][c] = v[2][c];
        Na[2][c] = v[4][c];
        Na[3][c] = v[5][c];
        Nb[0][c] = v[1][c];  // row b: -y row a, +y jq, -z, +z
        Nb[1][c] = v[3][c];
        Nb[2][c] = v[6][c];
        Nb[3][c] = v[7][c];
    }
    cg_row4(c3, na, xend, wrapx, v[1], Na, xe[0], xe[1], ka, d_out, q, acc);
    cg_row4(c3, nb, xend, wrapx, v[2], Nb, xe[2], xe[3], kb, d_out, q, acc);
}

__global__ void __launch_bounds__(256) k_lpcg_k1(GridDev g, const float* __restrict__ z,
                                                          const float* __restrict__ d_in, float* __restrict__ d_out,
                                                          float* __restrict__ q, const uint16_t* __restrict__ kind,
                                                          double* gpart, int gstride, unsigned* ticket,
                                                          double* scal, int* flag, int it, double target_rr) {
    // scalars of the previous iteration, evaluated once per block in FP64
    __shared__ float s_beta;
    __shared__ int s_stop;
    if (threadIdx.x == 0) {
        const double rz_new = scal[kS_RZN];
        double beta = 0.0;
        int stop = 0;
        if (it > 0) {
            const double zq = scal[kS_RZO], rr = scal[kS_RR];
            if (rr <= target_rr || flag[0]) {
                stop = 1;
                if (blockIdx.x == 0 && !flag[0]) {
                    flag[1] = it;  // iterations completed
                    flag[0] = 1;
                }
            } else {
                const double rz_old = scal[kS_RZ + ((it - 1) & 1)];
                const double alpha_old = scal[kS_ALPHA + ((it - 1) & 1)];
                beta = rz_old != 0.0 ? -alpha_old * zq / rz_old : 0.0;
            }
        }
        if (blockIdx.x == 0 && !stop) scal[kS_RZ + (it & 1)] = rz_new;
        s_beta = (float)beta;
        s_stop = stop;
    }
    __syncthreads();
    if (s_stop) return;
    float facc = 0.f;
    const float fb = s_beta;
    if ((g.ni & 3) == 0) {
        // pairs of rows (j0 even, j0 + 1) of a plane; an odd last row, or a pair across the seam
        // of a periodic y axis (the +y neighbour of j0 is not j0 + 1), goes row by row
        const int gpr = g.ni >> 2, npair = (g.nj + 1) >> 1;
        const int total = gpr * npair * g.nk;
        for (int pg = blockIdx.x * blockDim.x + threadIdx.x; pg < total; pg += gridDim.x * blockDim.x) {
            const int gx = pg % gpr, t = pg / gpr;
            const int j0 = 2 * (t % npair), k = t / npair;
            const int i0 = 4 * gx;
            const int n0 = (k * g.nj + j0) * g.ni + i0;
            const bool pair = j0 + 1 < g.nj && (g.periodic[1] ? wrap_p(j0, g.nj, 1) : j0 + 1) == j0 + 1;
            if (pair) {
                cg_pair(g, i0, j0, k, z, d_in, d_out, q, kind, fb, facc);
            } else {
                spmv_group(g, n0, z, d_in, d_out, q, kind, fb, facc);
                if (j0 + 1 < g.nj) spmv_group(g, n0 + g.ni, z, d_in, d_out, q, kind, fb, facc);
            }
        }
    } else {
        const int ngroups = (g.nv + 3) >> 2;
        for (int qg = blockIdx.x * blockDim.x + threadIdx.x; qg < ngroups; qg += gridDim.x * blockDim.x)
            spmv_group(g, qg << 2, z, d_in, d_out, q, kind, fb, facc);
    }
    const float v[1] = {facc};
    grid_sum<1>(v, gpart, gstride, ticket, scal + kS_DQ);
}
__global__ void __launch_bounds__(256) k_lpcg_k2(GridDev g, const float* __restrict__ d, const float* __restrict__ q,
                                                 float* __restrict__ e, float* __restrict__ r,
                                                 const uint16_t* __restrict__ kind, double* gpart, int gstride,
                                                 unsigned* ticket, double* scal, int* flag, int it) {
    if (flag[0]) return;
    __shared__ float s_alpha;  // alpha = rz / dq, once per block in FP64
    if (threadIdx.x == 0) {
        const double dq = scal[kS_DQ];
        const double alpha_d = dq != 0.0 ? scal[kS_RZ + (it & 1)] / dq : 0.0;
        if (blockIdx.x == 0) scal[kS_ALPHA + (it & 1)] = alpha_d;
        s_alpha = (float)alpha_d;
    }
    __syncthreads();
    const float alpha = s_alpha;
    float frr = 0.f;
    const int ng = g.nv >> 2;
    for (int qq = blockIdx.x * blockDim.x + threadIdx.x; qq < ng; qq += gridDim.x * blockDim.x) {
        const float4 d4 = reinterpret_cast<const float4*>(d)[qq];
        const float4 q4 = reinterpret_cast<const float4*>(q)[qq];
        const float4 e4 = reinterpret_cast<const float4*>(e)[qq];
        const float4 r4 = reinterpret_cast<const float4*>(r)[qq];
        const float dv[4] = {d4.x, d4.y, d4.z, d4.w}, qv[4] = {q4.x, q4.y, q4.z, q4.w};
        float ev[4] = {e4.x, e4.y, e4.z, e4.w}, rv[4] = {r4.x, r4.y, r4.z, r4.w};
        // no kind read: d and q are zero on non-FREE nodes (k_lpcg_k1 writes them so) and so is r,
        // which leaves e and r unchanged there
#pragma unroll
        for (int c = 0; c < 4; c++) {
            ev[c] += alpha * dv[c];
            rv[c] -= alpha * qv[c];
            frr += rv[c] * rv[c];
        }
        reinterpret_cast<float4*>(e)[qq] = make_float4(ev[0], ev[1], ev[2], ev[3]);
        reinterpret_cast<float4*>(r)[qq] = make_float4(rv[0], rv[1], rv[2], rv[3]);
    }
    if (blockIdx.x == 0 && threadIdx.x < (g.nv & 3)) {
        const int n = (ng << 2) + threadIdx.x;
        e[n] += alpha * d[n];
        const float rn = r[n] - alpha * q[n];
        r[n] = rn;
        frr += rn * rn;
    }
    const float v[1] = {frr};
    grid_sum<1>(v, gpart, gstride, ticket, scal + kS_RR);
}
// |a|^2 over n values into out[0] (deterministic: block partials, then one fixed-order sum)
__global__ void k_lp_sq(const float* __restrict__ a, int n, double* part) {
    float f = 0.f;
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x) f += a[x] * a[x];
    double acc[1] = {f};
    block_partials<1>(acc, part, kParts);
}
__global__ void k_lp_sum1(const double* part, int nblocks, double* out) {
    double t = sum_partials(part, nblocks);
    if (threadIdx.x == 0) out[0] = t;
}
void launch_lp_norm2(const float* a, int n, double* part, double* out, cudaStream_t s, int grid) {
    k_lp_sq<<<grid, 256, 0, s>>>(a, n, part);
    k_lp_sum1<<<1, 256, 0, s>>>(part, grid, out);
}

void launch_lpcg_init(const GridDev& g, SolveWork& w, const LpState& L, cudaStream_t s, int sms) {
    cudaMemsetAsync(w.e, 0, sizeof(float) * g.nv, s);
    cudaMemsetAsync(w.q, 0, sizeof(float) * g.nv, s);
    cudaMemsetAsync(w.d, 0, sizeof(float) * g.nv, s);
    cudaMemsetAsync(w.flag, 0, sizeof(int), s);
    launch_lp_apply(g, L, w.r, w.z, reinterpret_cast<const uint16_t*>(w.kind), w.q, &w, nullptr, s, sms);
}
void launch_lpcg_iter(const GridDev& g, SolveWork& w, const LpState& L, float* d_in, float* d_out, int it,
                      double target_rr, cudaStream_t s, int sms) {
    const uint16_t* kd = reinterpret_cast<const uint16_t*>(w.kind);
    k_lpcg_k1<<<cg_blocks(g), 256, 0, s>>>(g, w.z, d_in, d_out, w.q, kd, w.gpart, w.gstride, w.ticket, w.scal, w.flag,
                                           it, target_rr);
    k_lpcg_k2<<<stream_blocks(g), 256, 0, s>>>(g, d_out, w.q, w.e, w.r, kd, w.gpart, w.gstride, w.ticket, w.scal,
                                                  w.flag, it);
    launch_lp_apply(g, L, w.r, w.z, kd, w.q, &w, w.flag, s, sms);
}
// the first kernel of an iteration alone, at iteration 0 (beta = 0: d = z, q = L z on the scratch
// arrays): what the launch-shape tuner times
void launch_lpcg_k1_probe(const GridDev& g, SolveWork& w, float* d_in, float* d_out, cudaStream_t s) {
    const uint16_t* kd = reinterpret_cast<const uint16_t*>(w.kind);
    k_lpcg_k1<<<cg_blocks(g), 256, 0, s>>>(g, w.z, d_in, d_out, w.q, kd, w.gpart, w.gstride, w.ticket, w.scal, w.flag,
                                           0, 0.0);
}

// =====================================================================================
// training: one step = forward (unfolded network), energy-norm loss, backward, Adam
//   loss = (B r - x)^T L (B r - x) / x^T L x for a pair (r, x) with L x = r
// Network contractions run on the tensor cores as GEMMs over tiles of 128 voxels:
//   lift       h1  = im2col_+(z)  [V x 32] * Wl^T  [32 x C]
//   mix        h2  = h1 [V x C] * Wm^T [C x C]
//   proj bwd   dh2 = im2col_-(g)  [V x 32] * Wp    [32 x C]
//   mix bwd    dh1 = dh2 [V x C] * Wm  [C x C]
//   weight gradients dWp = im2col_-(g)^T h2, dWm = dh2^T h1, dWl^T = im2col_+(z)^T dh1 (K = voxels)
// im2col_+(z)[v][t] = z[v + o_t], im2col_-(g)[v][t] = g[v - o_t] (taps t >= 27 are zero).
// The projection forward (27 taps x C channels per voxel) runs on the CUDA cores.
// =====================================================================================
struct LpTrain {
    __nv_bfloat16* h1[kLpNetLevels + 1] = {};
    __nv_bfloat16* h2[kLpNetLevels + 1] = {};
    __nv_bfloat16* dh2[kLpNetLevels + 1] = {};
    __nv_bfloat16* dh1[kLpNetLevels + 1] = {};
    float* g[kLpMaxLevels] = {};  // restricted loss gradient, levels >= 1
    float *x = nullptr, *r = nullptr, *e0 = nullptr, *ge = nullptr;  // node arrays
    float *grad = nullptr, *m = nullptr, *v = nullptr, *pscale = nullptr;
    float* wprev = nullptr;  // weights before a training round (restored when validation rejects it)
    float* val_r = nullptr;  // right-hand side of the validation solve
    __nv_bfloat16* wbf = nullptr;  // per network level: Wl [C][32], Wm [C][C], Wm^T [C][C], Wp^T [C][32]
    int wbf_off[kLpNetLevels + 1][4] = {};
    double* part = nullptr;  // [32][kParts] partial sums
    double* red = nullptr;   // reduced scalars [64]
    float* wg = nullptr;     // per-CTA weight-gradient tiles [kWgCtas][128][64]
    unsigned* err = nullptr;
    double* h_red = nullptr;  // pinned
    float* pair_r[4] = {};
    float* pair_x[4] = {};
    int npairs = 0, next_pair = 0;
    long step = 0;
};
constexpr int kWgCtas = 152;

enum : int { kAZPos = 0, kAGNeg = 1, kAAct = 2 };

// value of row v (level voxel), column k of the A operand of an activation GEMM
template <int AMODE>
__device__ __forceinline__ float tc_a_value(const LView& src, const __nv_bfloat16* act, int K, int v, const int c[3],
                                            int k) {
    if (AMODE == kAAct) return __bfloat162float(act[(size_t)v * K + k]);
    if (k >= 27) return 0.f;
    const int sgn = AMODE == kAZPos ? 1 : -1;
    int x = lv_nb(c[0], sgn * (k % 3 - 1), src.n[0], src.per[0]);
    int y = lv_nb(c[1], sgn * ((k / 3) % 3 - 1), src.n[1], src.per[1]);
    int z = lv_nb(c[2], sgn * (k / 9 - 1), src.n[2], src.per[2]);
    if (x < 0 || y < 0 || z < 0) return 0.f;
    return src.a[lv_off(src, x, y, z)];
}

// out[v][n] = sum_k A(v, k) Bw[n][k]  (bf16 operands, FP32 accumulation in TMEM, bf16 result)
// 128 threads, one voxel row each; K in {16, 32, 64}, N in {16, 32, 64}
template <int AMODE>
__global__ void __launch_bounds__(128) k_tc_act(LView src, const __nv_bfloat16* __restrict__ act, int K,
                                                const __nv_bfloat16* __restrict__ Bw, int N, int V,
                                                __nv_bfloat16* __restrict__ out, unsigned* err) {
    extern __shared__ __align__(128) unsigned char smem[];
    __nv_bfloat16* sA = reinterpret_cast<__nv_bfloat16*>(smem);
    const int slices = K / 16;
    __nv_bfloat16* sB = sA + slices * 2048;
    __shared__ uint32_t tmem_base;
    __shared__ __align__(8) uint64_t bar;
    __shared__ int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int idx = tid; idx < N * K; idx += 128) {
        int n = idx / K, k = idx - n * K;
        sB[(k >> 4) * (N * 16) + tc_slice_offset(n, k & 15)] = Bw[idx];
    }
    const uint32_t ncols = N < 32 ? 32 : N;
    if (warp == 0) {
        tc_alloc(&tmem_base, ncols);
        tc_relinquish();
    }
    if (tid == 0) {
        tc_mbar_init(&bar, 1);
        s_fail = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tm = tmem_base;
    const uint32_t idesc = tc_idesc_bf16(128, N);
    unsigned phase = 0;
    const int ntiles = (V + 127) / 128;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int v = tile * 128 + tid;
        int c[3] = {0, 0, 0};
        if (v < V && AMODE != kAAct) lv_decode(src, (unsigned)v, c[0], c[1], c[2]);
        for (int k = 0; k < K; k++) {
            float a = v < V ? tc_a_value<AMODE>(src, act, K, v, c, k) : 0.f;
            sA[(k >> 4) * 2048 + tc_slice_offset(tid, k & 15)] = __float2bfloat16(a);
        }
        tc_fence_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            for (int sl = 0; sl < slices; sl++)
                tc_mma_bf16(tm, tc_smem_desc(sA + sl * 2048, 128, 256), tc_smem_desc(sB + sl * N * 16, 128, 256),
                            idesc, sl > 0 ? 1u : 0u);
            tc_commit(&bar);
        }
        if (!tc_mbar_wait(&bar, phase, wait_poll_limit(g_tc_wait_arg, kTcWaitLimit))) atomicExch(&s_fail, 1);
        phase ^= 1u;
        __syncthreads();
        if (s_fail) {
            // the MMAs did not complete in time: record it and wait (bounded) before freeing TMEM
            if (tid == 0) set_error(err, kErrBarrierTimeout);
            tc_mbar_wait(&bar, phase ^ 1u, kTcWaitLimit);
            break;
        }
        tc_fence_after();
        for (int c0 = 0; c0 < N; c0 += 16) {
            float vals[16];
            tc_ld16(tm + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, vals);
            if (v < V) {
                __align__(16) __nv_bfloat16 b[16];
#pragma unroll
                for (int q = 0; q < 16; q++) b[q] = __float2bfloat16(vals[q]);
                uint4* dst = reinterpret_cast<uint4*>(out + (size_t)v * N + c0);
                dst[0] = reinterpret_cast<uint4*>(b)[0];
                dst[1] = reinterpret_cast<uint4*>(b)[1];
            }
        }
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_dealloc(tm, ncols);
}

// D[m][n] = sum_v A(m, v) B(n, v) over all voxels; A(m, v) = im2col(src)[v][m] (m < 27) or
// act[v][m] (m < Mv), B(n, v) = actB[v][n]; M padded to 128 (rows >= Mv zero).  Each CTA writes its
// partial D (rows < Mv, N columns) to wg[blockIdx.x][128][64].
template <int AMODE>
__global__ void __launch_bounds__(128) k_tc_wgrad(LView src, const __nv_bfloat16* __restrict__ actA, int Mv,
                                                  const __nv_bfloat16* __restrict__ actB, int N, int V, float* wg,
                                                  unsigned* err) {
    extern __shared__ __align__(128) unsigned char smem[];
    __nv_bfloat16* sA = reinterpret_cast<__nv_bfloat16*>(smem);  // 8 slices x 128 rows x 16
    __nv_bfloat16* sB = sA + 8 * 2048;                             // 8 slices x N rows x 16
    __shared__ uint32_t tmem_base;
    __shared__ __align__(8) uint64_t bar;
    __shared__ int s_fail;
    const int tid = threadIdx.x, warp = tid >> 5;
    for (int idx = tid; idx < 8 * 2048; idx += 128) sA[idx] = __float2bfloat16(0.f);
    const uint32_t ncols = N < 32 ? 32 : N;
    if (warp == 0) {
        tc_alloc(&tmem_base, ncols);
        tc_relinquish();
    }
    if (tid == 0) {
        tc_mbar_init(&bar, 1);
        s_fail = 0;
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tm = tmem_base;
    const uint32_t idesc = tc_idesc_bf16(128, N);
    unsigned phase = 0;
    bool first = true, ok = true;
    const int ntiles = (V + 127) / 128;
    const int sl = tid >> 4, kk = tid & 15;  // this thread's voxel column inside the tile
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int v = tile * 128 + tid;
        int c[3] = {0, 0, 0};
        if (v < V && AMODE != kAAct) lv_decode(src, (unsigned)v, c[0], c[1], c[2]);
        for (int m = 0; m < Mv; m++) {
            float a = v < V ? tc_a_value<AMODE>(src, actA, Mv, v, c, m) : 0.f;
            sA[sl * 2048 + tc_slice_offset(m, kk)] = __float2bfloat16(a);
        }
        for (int n = 0; n < N; n++) {
            __nv_bfloat16 b = v < V ? actB[(size_t)v * N + n] : __float2bfloat16(0.f);
            sB[sl * (N * 16) + tc_slice_offset(n, kk)] = b;
        }
        tc_fence_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            for (int s8 = 0; s8 < 8; s8++)
                tc_mma_bf16(tm, tc_smem_desc(sA + s8 * 2048, 128, 256), tc_smem_desc(sB + s8 * N * 16, 128, 256),
                            idesc, (first && s8 == 0) ? 0u : 1u);
            tc_commit(&bar);
        }
        first = false;
        if (!tc_mbar_wait(&bar, phase, wait_poll_limit(g_tc_wait_arg, kTcWaitLimit))) atomicExch(&s_fail, 1);
        phase ^= 1u;
        __syncthreads();
        if (s_fail) {
            if (tid == 0) set_error(err, kErrBarrierTimeout);
            tc_mbar_wait(&bar, phase ^ 1u, kTcWaitLimit);
            ok = false;
            break;
        }
        tc_fence_after();
    }
    float* dst = wg + (size_t)blockIdx.x * 128 * 64;
    if (ok) {
        for (int c0 = 0; c0 < N; c0 += 16) {
            float vals[16];
            tc_ld16(tm + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, vals);
            if (tid < Mv)
#pragma unroll
                for (int q = 0; q < 16; q++) dst[tid * 64 + c0 + q] = first ? 0.f : vals[q];
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tc_dealloc(tm, ncols);
}

// sums the per-CTA tiles in a fixed order into the flat gradient: grad[off + m*sm + n*sn]
__global__ void k_lp_wg_reduce(const float* wg, int nctas, int Mv, int N, float* grad, int off, int sm, int sn) {
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < Mv * N; x += gridDim.x * blockDim.x) {
        int m = x / N, n = x - m * N;
        double a = 0.0;
        for (int b = 0; b < nctas; b++) a += wg[((size_t)b * 128 + m) * 64 + n];
        grad[off + m * sm + n * sn] = (float)a;
    }
}

// o = projection(h2) + P e_coarse on a network level
__global__ void k_lp_proj(LView zv, const __nv_bfloat16* __restrict__ h2, int C, const float* __restrict__ Wp, LView cin,
                          LView out) {
    for (unsigned idx = blockIdx.x * blockDim.x + threadIdx.x; idx < (unsigned)out.nvox;
         idx += gridDim.x * blockDim.x) {
        int c[3];
        lv_decode(out, idx, c[0], c[1], c[2]);
        float acc = 0.f;
        for (int t = 0; t < 27; t++) {
            int x = lv_nb(c[0], t % 3 - 1, zv.n[0], zv.per[0]);
            int y = lv_nb(c[1], (t / 3) % 3 - 1, zv.n[1], zv.per[1]);
            int z = lv_nb(c[2], t / 9 - 1, zv.n[2], zv.per[2]);
            if (x < 0 || y < 0 || z < 0) continue;
            const uint4* row = reinterpret_cast<const uint4*>(h2 + (size_t)lv_off(zv, x, y, z) * C);
            const float* w = Wp + t * C;
            for (int c8 = 0; c8 < C / 8; c8++) {
                uint4 u = row[c8];
                const __nv_bfloat16* b = reinterpret_cast<const __nv_bfloat16*>(&u);
#pragma unroll
                for (int q = 0; q < 8; q++) acc += __ldg(&w[c8 * 8 + q]) * __bfloat162float(b[q]);
            }
        }
        if (cin.a) acc += lp_prolong_at(cin, c);
        out.a[lv_off(out, c[0], c[1], c[2])] = acc;
    }
}

// (L v)_p on FREE nodes for v zero off FREE nodes (the operator of the reduced system)
__device__ __forceinline__ float lp_apply_L(const GridDev& g, const float* __restrict__ v, uint16_t kd, int n) {
    int i, j, k;
    node_ijk(g, n, i, j, k);
    Stencil s;
    stencil(g, i, j, k, s);
    float dg = 0.f, off = 0.f;
#pragma unroll
    for (int d = 0; d < 6; d++) {
        if (kd & (1u << (2 + d))) continue;
        dg += s.c[d];
        off += s.c[d] * v[s.q[d]];
    }
    return dg * v[n] - off;
}

// white-noise sample x on FREE nodes (Philox keyed by (seed, step, node)) and r = L x
__global__ void k_lp_noise(GridDev g, const uint16_t* __restrict__ kind, float* x, unsigned long long seed, long step) {
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < g.nv; n += gridDim.x * blockDim.x) {
        if ((kind[n] & 3) != kFree) {
            x[n] = 0.f;
            continue;
        }
        uint4 rr = philox4x32_10(make_uint4((unsigned)n, (unsigned)step, 0x5eedu, 0u),
                                 make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
        float u1 = u01(rr.x), u2 = u01(rr.y);
        x[n] = sqrtf(-2.f * logf(u1)) * cospif(2.f * u2);
    }
}
__global__ void k_lp_L(GridDev g, const uint16_t* __restrict__ kind, const float* __restrict__ x, float* r) {
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < g.nv; n += gridDim.x * blockDim.x) {
        uint16_t kd = kind[n];
        r[n] = (kd & 3) == kFree ? lp_apply_L(g, x, kd, n) : 0.f;
    }
}
// ge = L e - L x on FREE nodes; partials (e - x).ge (slot 0) and x.Lx (slot 1)
__global__ void k_lp_loss(GridDev g, const uint16_t* __restrict__ kind, const float* __restrict__ e,
                          const float* __restrict__ x, float* ge, double* part) {
    float f0 = 0.f, f1 = 0.f;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < g.nv; n += gridDim.x * blockDim.x) {
        uint16_t kd = kind[n];
        if ((kd & 3) != kFree) {
            ge[n] = 0.f;
            continue;
        }
        float le = lp_apply_L(g, e, kd, n), lx = lp_apply_L(g, x, kd, n);
        float d = le - lx;
        ge[n] = d;
        f0 += (e[n] - x[n]) * d;
        f1 += x[n] * lx;
    }
    double a0[1] = {f0}, a1[1] = {f1};
    block_partials<1>(a0, part + 0 * kParts, kParts);
    block_partials<1>(a1, part + 1 * kParts, kParts);
}
// ge *= 2 / x.Lx ; red[0] = loss
__global__ void k_lp_loss_scale(int nv, float* ge, const double* part, double* red) {
    double num = sum_partials(part + 0 * kParts, gridDim.x);
    double q = sum_partials(part + 1 * kParts, gridDim.x);
    const float sc = q > 0 ? (float)(2.0 / q) : 0.f;
    if (blockIdx.x == 0 && threadIdx.x == 0) red[0] = q > 0 ? num / q : 0.0;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nv; n += gridDim.x * blockDim.x) ge[n] *= sc;
}
// dS0[t] partials = sum_v ge[v] r[v + o_t] (level 0, FREE nodes; r is zero elsewhere)
__global__ void k_lp_ds0(GridDev g, LView rin, const uint16_t* __restrict__ kind, const float* __restrict__ ge,
                         double* part) {
    float acc[27];
#pragma unroll
    for (int t = 0; t < 27; t++) acc[t] = 0.f;
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < g.nv; n += gridDim.x * blockDim.x) {
        if ((kind[n] & 3) != kFree) continue;
        int c[3];
        node_ijk(g, n, c[0], c[1], c[2]);
        const float gv = ge[n];
#pragma unroll
        for (int t = 0; t < 27; t++) {
            int x = lv_nb(c[0], t % 3 - 1, rin.n[0], rin.per[0]);
            int y = lv_nb(c[1], (t / 3) % 3 - 1, rin.n[1], rin.per[1]);
            int z = lv_nb(c[2], t / 9 - 1, rin.n[2], rin.per[2]);
            if (x >= 0 && y >= 0 && z >= 0) acc[t] += gv * rin.a[lv_off(rin, x, y, z)];
        }
    }
    __shared__ double s[27][8];
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
    for (int t = 0; t < 27; t++) {
        double x = acc[t];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) s[t][wp] = x;
    }
    __syncthreads();
    if (threadIdx.x < 27) {
        double x = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) x += s[threadIdx.x][w];
        part[threadIdx.x * kParts + blockIdx.x] = x;
    }
}
__global__ void k_lp_ds0_collect(const double* part, int nblocks, float* grad, int off) {
    const int t = blockIdx.x;
    double x = sum_partials(part + t * kParts, nblocks);
    if (threadIdx.x == 0) grad[off + t] = (float)x;
}

// bf16 operand copies of the network weights
__global__ void k_lp_prep_bf16(const float* __restrict__ W, LpLayout lay, __nv_bfloat16* wbf, int o1, int o2, int o3,
                               int o4, int l) {
    const int C = lp_channels(l);
    const float* Wl = W + lay.wl[l];
    const float* Wm = W + lay.wm[l];
    const float* Wp = W + lay.wp[l];
    for (int x = threadIdx.x; x < C * 32; x += blockDim.x) {
        int c = x / 32, t = x % 32;
        wbf[o1 + x] = __float2bfloat16(t < 27 ? Wl[c * 27 + t] : 0.f);  // lift B [C][32]
        wbf[o4 + x] = __float2bfloat16(t < 27 ? Wp[t * C + c] : 0.f);   // proj-backward B [C][32]
    }
    for (int x = threadIdx.x; x < C * C; x += blockDim.x) {
        int a = x / C, b = x % C;
        wbf[o2 + x] = __float2bfloat16(Wm[a * C + b]);  // mix B: [out][in]
        wbf[o3 + x] = __float2bfloat16(Wm[b * C + a]);  // mix-backward B: [in][out]
    }
}

// Adam (beta1 0.9, beta2 0.999), the step of each parameter scaled by its group's magnitude
__global__ void k_lp_adam(float* W, const float* __restrict__ grad, float* m, float* v, const float* __restrict__ pscale,
                          int n, float lr, float bc1, float bc2) {
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x) {
        float gx = grad[x];
        float mm = 0.9f * m[x] + 0.1f * gx;
        float vv = 0.999f * v[x] + 0.001f * gx * gx;
        m[x] = mm;
        v[x] = vv;
        float mh = mm / bc1, vh = vv / bc2;
        W[x] -= lr * pscale[x] * mh / (sqrtf(vh) + 1e-30f);
    }
}

void lp_free_train(LpState& L) {
    LpTrain* T = L.train;
    if (!T) return;
    for (int l = 1; l <= kLpNetLevels; l++)
        for (void* p : {(void*)T->h1[l], (void*)T->h2[l], (void*)T->dh2[l], (void*)T->dh1[l]})
            if (p) cudaFree(p);
    for (int l = 1; l < kLpMaxLevels; l++)
        if (T->g[l]) cudaFree(T->g[l]);
    for (void* p : {(void*)T->x, (void*)T->r, (void*)T->e0, (void*)T->ge, (void*)T->grad, (void*)T->m, (void*)T->v,
                    (void*)T->pscale, (void*)T->wbf, (void*)T->part, (void*)T->red, (void*)T->wg, (void*)T->err,
                    (void*)T->wprev, (void*)T->val_r})
        if (p) cudaFree(p);
    for (int k = 0; k < 4; k++) {
        if (T->pair_r[k]) cudaFree(T->pair_r[k]);
        if (T->pair_x[k]) cudaFree(T->pair_x[k]);
    }
    if (T->h_red) cudaFreeHost(T->h_red);
    delete T;
    L.train = nullptr;
}

#define LP_CU(call)                      \
    do {                                 \
        if ((call) != cudaSuccess) return 2; \
    } while (0)

// allocates the training state; returns 0 or 2 (CUDA error)
int lp_alloc_train(const GridDev& g, LpState& L, const float* init_W) {
    if (L.train) return 0;
    LpTrain* T = new LpTrain();
    L.train = T;
    for (int l = 1; l <= kLpNetLevels && l < L.nlev; l++) {
        size_t V = (size_t)L.dims[l][0] * L.dims[l][1] * L.dims[l][2];
        size_t bytes = V * lp_channels(l) * sizeof(__nv_bfloat16);
        LP_CU(cudaMalloc(&T->h1[l], bytes));
        LP_CU(cudaMalloc(&T->h2[l], bytes));
        LP_CU(cudaMalloc(&T->dh2[l], bytes));
        LP_CU(cudaMalloc(&T->dh1[l], bytes));
    }
    for (int l = 1; l < L.nlev; l++)
        LP_CU(cudaMalloc(&T->g[l], sizeof(float) * (size_t)L.dims[l][0] * L.dims[l][1] * L.dims[l][2]));
    for (float** p : {&T->x, &T->r, &T->e0, &T->ge, &T->val_r}) LP_CU(cudaMalloc(p, sizeof(float) * g.nv));
    const int n = L.lay.total;
    for (float** p : {&T->grad, &T->m, &T->v, &T->pscale, &T->wprev}) LP_CU(cudaMalloc(p, sizeof(float) * n));
    LP_CU(cudaMemset(T->m, 0, sizeof(float) * n));
    LP_CU(cudaMemset(T->v, 0, sizeof(float) * n));
    LP_CU(cudaMemset(T->grad, 0, sizeof(float) * n));
    // step scale of each parameter: the largest starting magnitude of its group
    std::vector<float> ps(n, 1.f);
    auto group = [&](int off, int cnt) {
        float mx = 0.f;
        for (int k = 0; k < cnt; k++) mx = std::max(mx, std::fabs(init_W[off + k]));
        for (int k = 0; k < cnt; k++) ps[off + k] = mx > 0 ? mx : 1.f;
    };
    group(L.lay.s0, 27);
    int wbf = 0;
    for (int l = 1; l <= kLpNetLevels; l++) {
        int C = lp_channels(l);
        group(L.lay.wl[l], C * 27);
        group(L.lay.wm[l], C * C);
        group(L.lay.wp[l], 27 * C);
        T->wbf_off[l][0] = wbf;
        wbf += C * 32;
        T->wbf_off[l][1] = wbf;
        wbf += C * C;
        T->wbf_off[l][2] = wbf;
        wbf += C * C;
        T->wbf_off[l][3] = wbf;
        wbf += C * 32;
    }
    LP_CU(cudaMemcpy(T->pscale, ps.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
    LP_CU(cudaMalloc(&T->wbf, sizeof(__nv_bfloat16) * wbf));
    LP_CU(cudaMalloc(&T->part, sizeof(double) * 32 * kParts));
    LP_CU(cudaMalloc(&T->red, sizeof(double) * 64));
    LP_CU(cudaMalloc(&T->wg, sizeof(float) * (size_t)kWgCtas * 128 * 64));
    LP_CU(cudaMalloc(&T->err, sizeof(unsigned)));
    LP_CU(cudaMemset(T->err, 0, sizeof(unsigned)));
    LP_CU(cudaMallocHost(&T->h_red, sizeof(double) * 64));
    return 0;
}

static size_t tc_act_smem(int K, int N) { return (size_t)(K / 16) * (128 + N) * 16 * sizeof(__nv_bfloat16); }
static size_t tc_wg_smem(int N) { return (size_t)8 * (128 + N) * 16 * sizeof(__nv_bfloat16); }

template <int AMODE>
static void launch_tc_act(LView src, const __nv_bfloat16* act, int K, const __nv_bfloat16* Bw, int N, int V,
                          __nv_bfloat16* out, unsigned* err, cudaStream_t s, int sms) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_tc_act<AMODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_act_smem(64, 64));
        attr = true;
    }
    int tiles = (V + 127) / 128;
    k_tc_act<AMODE><<<std::max(1, std::min(tiles, sms * 4)), 128, tc_act_smem(K, N), s>>>(src, act, K, Bw, N, V, out,
                                                                                          err);
}
template <int AMODE>
static void launch_tc_wgrad(LView src, const __nv_bfloat16* actA, int Mv, const __nv_bfloat16* actB, int N, int V,
                            float* wg, unsigned* err, cudaStream_t s) {
    static bool attr = false;
    if (!attr) {
        cudaFuncSetAttribute(k_tc_wgrad<AMODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tc_wg_smem(64));
        attr = true;
    }
    k_tc_wgrad<AMODE><<<kWgCtas, 128, tc_wg_smem(N), s>>>(src, actA, Mv, actB, N, V, wg, err);
}

void launch_lp_prep(const LpState& L, cudaStream_t s) {
    const LpTrain* T = L.train;
    for (int l = 1; l <= kLpNetLevels; l++)
        k_lp_prep_bf16<<<1, 256, 0, s>>>(L.W, L.lay, T->wbf, T->wbf_off[l][0], T->wbf_off[l][1], T->wbf_off[l][2],
                                         T->wbf_off[l][3], l);
}

// forward + loss + backward for the pair (r, x) on the node array; gradient into T->grad,
// loss into T->red[0].  r and x are zero off FREE nodes.
void launch_lp_loss_grad(const GridDev& g, LpState& L, const uint16_t* kind, const float* r, const float* x,
                         cudaStream_t s, int grid, int sms) {
    LpTrain* T = L.train;
    LView none{};
    none.a = nullptr;
    LView r0 = lp_node_view(g, L, const_cast<float*>(r));
    // forward: restriction chain
    for (int l = 1; l < L.nlev; l++) {
        LView f = l == 1 ? r0 : lp_level_view(L, l - 1, L.z[l - 1]);
        LView c = lp_level_view(L, l, L.z[l]);
        k_lp_restrict<<<lp_blocks(c.nvox, sms), 256, 0, s>>>(f, c, nullptr);
    }
    for (int l = L.nlev - 1; l >= 1; l--) {
        LView zin = lp_level_view(L, l, L.z[l]);
        LView cin = l + 1 < L.nlev ? lp_level_view(L, l + 1, L.e[l + 1]) : none;
        LView out = lp_level_view(L, l, L.e[l]);
        if (l <= kLpNetLevels) {
            const int C = lp_channels(l), V = zin.nvox;
            launch_tc_act<kAZPos>(zin, nullptr, 32, T->wbf + T->wbf_off[l][0], C, V, T->h1[l], T->err, s, sms);
            launch_tc_act<kAAct>(zin, T->h1[l], C, T->wbf + T->wbf_off[l][1], C, V, T->h2[l], T->err, s, sms);
            k_lp_proj<<<lp_blocks(V, sms), 256, 0, s>>>(zin, T->h2[l], C, L.W + L.lay.wp[l], cin, out);
        } else {
            k_lp_up<<<lp_blocks(out.nvox, sms), 256, 0, s>>>(zin, cin, out, 2, nullptr, (float)(1.0 / L.diag[l]),
                                                            nullptr);
        }
    }
    LView cin1 = L.nlev > 1 ? lp_level_view(L, 1, L.e[1]) : none;
    launch_up0(g, r0, cin1, T->e0, kind, L.W + L.lay.s0, nullptr, nullptr, 0, nullptr, nullptr, nullptr, s, sms);
    // loss and its gradient with respect to e
    k_lp_loss<<<grid, 256, 0, s>>>(g, kind, T->e0, x, T->ge, T->part);
    k_lp_loss_scale<<<grid, 256, 0, s>>>(g.nv, T->ge, T->part, T->red);
    // backward: restriction chain of the gradient, then every level's parameters
    LView g0 = lp_node_view(g, L, T->ge);
    for (int l = 1; l < L.nlev; l++) {
        LView f = l == 1 ? g0 : lp_level_view(L, l - 1, T->g[l - 1]);
        LView c = lp_level_view(L, l, T->g[l]);
        k_lp_restrict<<<lp_blocks(c.nvox, sms), 256, 0, s>>>(f, c, nullptr);
    }
    k_lp_ds0<<<grid, 256, 0, s>>>(g, r0, kind, T->ge, T->part);
    k_lp_ds0_collect<<<27, 256, 0, s>>>(T->part, grid, T->grad, L.lay.s0);
    for (int l = 1; l <= kLpNetLevels && l < L.nlev; l++) {
        const int C = lp_channels(l);
        LView zin = lp_level_view(L, l, L.z[l]);
        LView gl = lp_level_view(L, l, T->g[l]);
        const int V = zin.nvox;
        const int rb = std::max(1, std::min(64, (27 * C + 255) / 256));
        launch_tc_act<kAGNeg>(gl, nullptr, 32, T->wbf + T->wbf_off[l][3], C, V, T->dh2[l], T->err, s, sms);
        launch_tc_wgrad<kAGNeg>(gl, nullptr, 27, T->h2[l], C, V, T->wg, T->err, s);
        k_lp_wg_reduce<<<rb, 256, 0, s>>>(T->wg, kWgCtas, 27, C, T->grad, L.lay.wp[l], C, 1);
        launch_tc_act<kAAct>(gl, T->dh2[l], C, T->wbf + T->wbf_off[l][2], C, V, T->dh1[l], T->err, s, sms);
        launch_tc_wgrad<kAAct>(gl, T->dh2[l], C, T->h1[l], C, V, T->wg, T->err, s);
        k_lp_wg_reduce<<<rb, 256, 0, s>>>(T->wg, kWgCtas, C, C, T->grad, L.lay.wm[l], C, 1);
        launch_tc_wgrad<kAZPos>(zin, nullptr, 27, T->dh1[l], C, V, T->wg, T->err, s);
        k_lp_wg_reduce<<<rb, 256, 0, s>>>(T->wg, kWgCtas, 27, C, T->grad, L.lay.wl[l], 1, 27);
    }
}

void launch_lp_noise_pair(const GridDev& g, LpState& L, const uint16_t* kind, unsigned long long seed, cudaStream_t s,
                          int grid) {
    LpTrain* T = L.train;
    k_lp_noise<<<grid, 256, 0, s>>>(g, kind, T->x, seed, T->step);
    k_lp_L<<<grid, 256, 0, s>>>(g, kind, T->x, T->r);
}

__global__ void k_lp_acc(float* dst, const float* __restrict__ src, int n) {
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x) dst[x] += src[x];
}
// training pairs from solves: the first residual r0 of a solve and the sum x of its corrections
int lp_pair_begin(LpState& L, const float* r0, int nv, cudaStream_t s) {
    LpTrain* T = L.train;
    int k = T->next_pair;
    if (!T->pair_r[k]) {
        LP_CU(cudaMalloc(&T->pair_r[k], sizeof(float) * nv));
        LP_CU(cudaMalloc(&T->pair_x[k], sizeof(float) * nv));
    }
    LP_CU(cudaMemcpyAsync(T->pair_r[k], r0, sizeof(float) * nv, cudaMemcpyDeviceToDevice, s));
    LP_CU(cudaMemsetAsync(T->pair_x[k], 0, sizeof(float) * nv, s));
    return 0;
}
void lp_pair_add(LpState& L, const float* e, int nv, cudaStream_t s, int grid) {
    LpTrain* T = L.train;
    k_lp_acc<<<grid, 256, 0, s>>>(T->pair_x[T->next_pair], e, nv);
}
void lp_pair_end(LpState& L) {
    LpTrain* T = L.train;
    T->next_pair = (T->next_pair + 1) % 4;
    T->npairs = std::min(T->npairs + 1, 4);
}
const float* lp_pair_r(const LpState& L, int k) { return L.train->pair_r[k]; }
const float* lp_pair_x(const LpState& L, int k) { return L.train->pair_x[k]; }
int lp_npairs(const LpState& L) { return L.train ? L.train->npairs : 0; }
float* lp_train_x(const LpState& L) { return L.train->x; }
float* lp_train_val(const LpState& L) { return L.train->val_r; }
float* lp_train_wprev(const LpState& L) { return L.train->wprev; }
float* lp_train_r(const LpState& L) { return L.train->r; }
float* lp_train_grad(const LpState& L) { return L.train->grad; }
double* lp_train_red(const LpState& L) { return L.train->red; }
unsigned* lp_train_err(const LpState& L) { return L.train->err; }

// Keeps B symmetric after every optimiser step, so that flexible CG sees a symmetric
// preconditioner (an unconstrained step can make B indefinite, and CG then stalls): the level-0
// stencil is made even (S0[t] = S0[26 - t]); on each network level the projection is tied to the
// scaled adjoint of the lift, Wp[t][c] = s_l Wl[c][26 - t] with s_l = 1 / diag_l (the start weights
// satisfy it), and the channel mix is made symmetric.  Each tied pair is replaced by its mean.
struct LpSymScales {
    float s[kLpNetLevels + 1];
};
__global__ void k_lp_symmetrize(float* W, LpLayout lay, LpSymScales sc) {
    const int tid = threadIdx.x;
    if (tid < 13) {
        const float m = 0.5f * (W[lay.s0 + tid] + W[lay.s0 + 26 - tid]);
        W[lay.s0 + tid] = m;
        W[lay.s0 + 26 - tid] = m;
    }
    for (int l = 1; l <= kLpNetLevels; l++) {
        const int C = lp_channels(l);
        const float s = sc.s[l];
        for (int x = tid; x < C * 27; x += blockDim.x) {
            const int c = x / 27, t = x - c * 27;
            float* a = W + lay.wl[l] + c * 27 + t;
            float* p = W + lay.wp[l] + (26 - t) * C + c;
            const float m = 0.5f * (*a + *p / s);
            *a = m;
            *p = s * m;
        }
        for (int x = tid; x < C * C; x += blockDim.x) {
            const int i = x / C, j = x - i * C;
            if (i >= j) continue;
            float* u = W + lay.wm[l] + i * C + j;
            float* v = W + lay.wm[l] + j * C + i;
            const float m = 0.5f * (*u + *v);
            *u = m;
            *v = m;
        }
    }
}

void launch_lp_adam(LpState& L, float lr, cudaStream_t s) {
    LpTrain* T = L.train;
    T->step++;
    float bc1 = 1.f - powf(0.9f, (float)T->step), bc2 = 1.f - powf(0.999f, (float)T->step);
    k_lp_adam<<<std::max(1, std::min(1024, (L.lay.total + 255) / 256)), 256, 0, s>>>(L.W, T->grad, T->m, T->v,
                                                                                     T->pscale, L.lay.total, lr, bc1, bc2);
    LpSymScales sc{};
    for (int l = 1; l <= kLpNetLevels; l++) sc.s[l] = (float)(1.0 / (l < L.nlev ? L.diag[l] : 1.0));
    k_lp_symmetrize<<<1, 256, 0, s>>>(L.W, L.lay, sc);
    launch_lp_prep(L, s);
    launch_lp_fold(L, s);
}

// =====================================================================================
// host: layout, initial weights, Galerkin diagonals
// =====================================================================================
void lp_layout(LpLayout& lay) {
    int off = 0;
    lay.s0 = off;
    off += 27;
    for (int l = 1; l <= kLpNetLevels; l++) {
        int C = lp_channels(l);
        lay.wl[l] = off;
        off += C * 27;
        lay.wm[l] = off;
        off += C * C;
        lay.wp[l] = off;
        off += 27 * C;
    }
    lay.wl[0] = lay.wm[0] = lay.wp[0] = 0;
    lay.total = off;
}

// BPX start: S0 = delta / diag_0; network level l: lift and projection pick the centre tap of
// channel 0, the mix is the identity, the projection scales by 1 / diag_l
void lp_init_weights(const LpLayout& lay, const double* diag, int nlev, float* W) {
    std::fill(W, W + lay.total, 0.f);
    W[lay.s0 + 13] = (float)(1.0 / diag[0]);
    for (int l = 1; l <= kLpNetLevels; l++) {
        int C = lp_channels(l);
        double d = l < nlev ? diag[l] : 1.0;
        W[lay.wl[l] + 0 * 27 + 13] = 1.f;
        for (int c = 0; c < C; c++) W[lay.wm[l] + c * C + c] = 1.f;
        W[lay.wp[l] + 13 * C + 0] = (float)(1.0 / d);
    }
}

namespace {
std::vector<double> up1(const std::vector<double>& a, size_t nf) {
    std::vector<double> f(nf, 0.0);
    size_t nc = a.size();
    for (size_t i = 0; i < nf; i++) {
        size_t c = i >> 1;
        double v = 0.75 * a[c];
        if (i & 1) {
            if (c + 1 < nc) v += 0.25 * a[c + 1];
        } else if (c > 0) {
            v += 0.25 * a[c - 1];
        }
        f[i] = v;
    }
    return f;
}
std::vector<double> dn1(const std::vector<double>& f) {
    size_t nf = f.size(), nc = (nf + 1) / 2;
    std::vector<double> c(nc, 0.0);
    for (size_t k = 0; k < nc; k++) {
        long raw[4] = {(long)(2 * k) - 1, (long)(2 * k), (long)(2 * k + 1), (long)(2 * k + 2)};
        const double w[4] = {0.25, 0.75, 0.75, 0.25};
        for (int m = 0; m < 4; m++)
            if (raw[m] >= 0 && raw[m] < (long)nf) c[k] += w[m] * f[raw[m]];
    }
    return c;
}
}  // namespace

// diag_l = (cx + cy + cz) t_l m_l^2, with t_l, m_l the interior diagonals of P^T T P and P^T P
// along one axis after l coarsenings (T = tridiag(-1, 2, -1)), probed on a long 1-D array
void lp_galerkin_diag(const double c[3], int nlev, double* diag) {
    size_t n = (size_t)1 << (nlev + 3);
    for (int l = 0; l < nlev; l++) {
        size_t nc = n >> l;
        std::vector<double> f(nc, 0.0);
        f[nc / 2] = 1.0;
        for (int k = 0; k < l; k++) f = up1(f, 2 * f.size());
        std::vector<double> tf(f.size()), mf = f;
        for (size_t i = 0; i < f.size(); i++)
            tf[i] = 2 * f[i] - (i > 0 ? f[i - 1] : 0.0) - (i + 1 < f.size() ? f[i + 1] : 0.0);
        for (int k = 0; k < l; k++) {
            tf = dn1(tf);
            mf = dn1(mf);
        }
        diag[l] = (c[0] + c[1] + c[2]) * tf[nc / 2] * mf[nc / 2] * mf[nc / 2];
    }
}

// the first-wait poll count of the tensor-core kernels on the current device (test hook)
int lp_set_tc_wait_polls(long long arg) {
    return cudaMemcpyToSymbol(g_tc_wait_arg, &arg, sizeof(arg)) == cudaSuccess ? 0 : -1;
}

}  // namespace pic

using namespace pic;

// Multiplies one 128 x N tile on the tensor cores (device pointers, current device); used by the
// tests to check the tcgen05 operand layout.  Returns 0, 1 for bad sizes, 2 for a CUDA error,
// 5 when the MMA completion wait ran out.
extern "C" int pic_tc_gemm_check(const void* A, const void* B, void* D, int N, int K, void* stream) {
    if (!A || !B || !D || K <= 0 || K % 16 || K > 256 || (N != 16 && N != 32 && N != 64 && N != 128)) return 1;
    unsigned* err = nullptr;
    cudaStream_t s = (cudaStream_t)stream;
    if (cudaMallocAsync((void**)&err, sizeof(unsigned), s) != cudaSuccess) return 2;
    cudaMemsetAsync(err, 0, sizeof(unsigned), s);
    size_t smem = (size_t)(K / 16) * (128 + N) * 16 * sizeof(__nv_bfloat16);
    if (smem > 48 * 1024) cudaFuncSetAttribute(k_tc_gemm_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_tc_gemm_tile<<<1, 128, smem, s>>>((const __nv_bfloat16*)A, (const __nv_bfloat16*)B, (float*)D, N, K, err);
    unsigned h = 0;
    cudaMemcpyAsync(&h, err, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    cudaFreeAsync(err, s);
    if (e != cudaSuccess) return 2;
    return h ? 5 : 0;
}
