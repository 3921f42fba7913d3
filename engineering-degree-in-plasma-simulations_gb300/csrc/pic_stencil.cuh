// Node-index decoding, the 7-point stencil of the reduced Poisson system, and deterministic
// block reductions, shared by the field kernels and the learned-preconditioner kernels.
#pragma once
#include "pic_kernels.h"

namespace pic {

constexpr double kEps0 = 8.85418782e-12;  // ch4/v3/src/all.h:16

__device__ __forceinline__ void node_ijk(const GridDev& g, int n, int& i, int& j, int& k) {
    unsigned t = fdiv((unsigned)n, g.fd_ni);
    i = n - (int)t * g.ni;
    unsigned kk = fdiv(t, g.fd_nj);
    j = (int)t - (int)kk * g.nj;
    k = (int)kk;
}
// neighbour index along an axis with periodic wrap (the copy at n-1 folds onto 0)
__device__ __forceinline__ int wrap_m(int c, int n, int per) { return (per && c == 0) ? n - 2 : c - 1; }
__device__ __forceinline__ int wrap_p(int c, int n, int per) { return (per && c + 1 >= n - 1) ? 0 : c + 1; }

struct Stencil {
    int q[6];
    float c[6];
};
__device__ __forceinline__ void stencil(const GridDev& g, int i, int j, int k, Stencil& s) {
    int nij = g.ni * g.nj;
    int im = wrap_m(i, g.ni, g.periodic[0]), ip = wrap_p(i, g.ni, g.periodic[0]);
    int jm = wrap_m(j, g.nj, g.periodic[1]), jp = wrap_p(j, g.nj, g.periodic[1]);
    int km = wrap_m(k, g.nk, g.periodic[2]), kp = wrap_p(k, g.nk, g.periodic[2]);
    int row = k * nij + j * g.ni;
    s.q[0] = row + im;
    s.q[1] = row + ip;
    s.q[2] = k * nij + jm * g.ni + i;
    s.q[3] = k * nij + jp * g.ni + i;
    s.q[4] = km * nij + j * g.ni + i;
    s.q[5] = kp * nij + j * g.ni + i;
    float cx = g.inv_dx[0] * g.inv_dx[0], cy = g.inv_dx[1] * g.inv_dx[1], cz = g.inv_dx[2] * g.inv_dx[2];
    s.c[0] = s.c[1] = cx;
    s.c[2] = s.c[3] = cy;
    s.c[4] = s.c[5] = cz;
}

// ------------------------------------------------------------------------------------
// block reduction of up to four doubles into per-block partial slots
// ------------------------------------------------------------------------------------
template <int N>
__device__ __forceinline__ void block_partials(double (&v)[N], double* part, int nslots_stride) {
    __shared__ double s[N][8];
#pragma unroll
    for (int c = 0; c < N; c++) {
        double x = v[c];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0) s[c][threadIdx.x >> 5] = x;
    }
    __syncthreads();
    if (threadIdx.x < N) {
        double x = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) x += s[threadIdx.x][w];
        part[threadIdx.x * nslots_stride + blockIdx.x] = x;
    }
    __syncthreads();
}
// every block sums the same partials in the same order: identical scalars everywhere
__device__ __forceinline__ double sum_partials(const double* part, int nblocks) {
    __shared__ double s[8];
    double x = 0;
    for (int b = threadIdx.x; b < nblocks; b += blockDim.x) x += part[b];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = x;
    __syncthreads();
    double t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s[w];
    __syncthreads();
    return t;
}

__device__ __forceinline__ float diag_of(uint16_t kd, const Stencil& s) {
    float dg = 0.f;
#pragma unroll
    for (int d = 0; d < 6; d++)
        if (!(kd & (1u << (2 + d)))) dg += s.c[d];
    return dg;
}
}  // namespace pic

namespace pic {

// Deterministic grid-wide sums of N per-thread FP32 values: every block writes its FP64
// partial sums to part[c * stride + block]; the last block to finish (an atomic ticket) adds the
// partials in block order and writes out[c].  The order of the additions never depends on
// timing, so the sums are bit-reproducible from run to run.
template <int N>
__device__ __forceinline__ void grid_sum(const float (&v)[N], double* part, int stride, unsigned* ticket,
                                         double* out) {
    __shared__ double s[N][32];
    __shared__ unsigned s_last;
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    // warp sums in FP32 (FP64 would occupy the narrow FP64 pipe with every thread of the grid),
    // block and grid sums in FP64
#pragma unroll
    for (int c = 0; c < N; c++) {
        float x = v[c];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) s[c][wp] = (double)x;
    }
    __syncthreads();
    if (threadIdx.x < N) {
        double x = 0;
        for (int w = 0; w < nw; w++) x += s[threadIdx.x][w];
        part[threadIdx.x * stride + blockIdx.x] = x;
        __threadfence();  // the writers publish their partials before the ticket is taken
    }
    __syncthreads();
    if (threadIdx.x == 0) s_last = (atomicAdd(ticket, 1u) == gridDim.x - 1) ? 1u : 0u;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
#pragma unroll
    for (int c = 0; c < N; c++) {
        double x = 0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) x += __ldcg(&part[c * stride + b]);
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        __syncthreads();
        if (lane == 0) s[c][wp] = x;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0;
            for (int w = 0; w < nw; w++) t += s[c][w];
            out[c] = t;
        }
    }
    if (threadIdx.x == 0) *ticket = 0u;
}

// d' = z + beta d_in, q = L d' over the nodes n0 .. n0+3 of one row (d'.q summed into acc).  When
// rows are a multiple of four nodes and the group does not touch the row ends, the group and its
// y / z neighbour rows are read with 16-byte loads; other groups go node by node.
__device__ __forceinline__ void spmv_group(const GridDev& g, int n0, const float* __restrict__ z,
                                           const float* __restrict__ d_in, float* __restrict__ d_out,
                                           float* __restrict__ q, const uint16_t* __restrict__ kind, float fb,
                                           float& acc) {
    int i0, j, k;
    node_ijk(g, n0, i0, j, k);
    const float c3[3] = {g.inv_dx[0] * g.inv_dx[0], g.inv_dx[1] * g.inv_dx[1], g.inv_dx[2] * g.inv_dx[2]};
    // rows of a multiple of four nodes: every group, the row ends included (a row-end node is
    // never FREE except the first node of a periodic row, whose -x neighbour is node ni-2; on a
    // periodic row node ni-2 takes node 0, not the copy plane ni-1, as its +x neighbour)
    if ((g.ni & 3) == 0) {
        const int jm = g.periodic[1] ? wrap_m(j, g.nj, 1) : max(j - 1, 0);
        const int jp = g.periodic[1] ? wrap_p(j, g.nj, 1) : min(j + 1, g.nj - 1);
        const int km = g.periodic[2] ? wrap_m(k, g.nk, 1) : max(k - 1, 0);
        const int kp = g.periodic[2] ? wrap_p(k, g.nk, 1) : min(k + 1, g.nk - 1);
        const int off[4] = {(k * g.nj + jm) * g.ni + i0, (k * g.nj + jp) * g.ni + i0, (km * g.nj + j) * g.ni + i0,
                            (kp * g.nj + j) * g.ni + i0};
        // d' at the group, its x ends and its four neighbour rows
        auto dv4 = [&](int o, float (&dst)[4]) {
            const float4 a = *reinterpret_cast<const float4*>(z + o);
            const float4 b = *reinterpret_cast<const float4*>(d_in + o);
            dst[0] = a.x + fb * b.x;
            dst[1] = a.y + fb * b.y;
            dst[2] = a.z + fb * b.z;
            dst[3] = a.w + fb * b.w;
        };
        float C[4], N[4][4];
        dv4(n0, C);
#pragma unroll
        for (int m = 0; m < 4; m++) dv4(off[m], N[m]);
        const bool xend = i0 + 4 == g.ni, wrapx = g.periodic[0] != 0;
        const int ixm = i0 > 0 ? n0 - 1 : (wrapx ? n0 + g.ni - 2 : n0);
        const int ixp = xend ? (wrapx ? n0 - i0 : n0 + 3) : n0 + 4;
        const float xm = z[ixm] + fb * d_in[ixm], xp = z[ixp] + fb * d_in[ixp];
        const ushort4 k4 = *reinterpret_cast<const ushort4*>(kind + n0);
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
                o += c3[d >> 1] * nb[d];  // zero on non-FREE neighbours
            }
            dvo[c] = C[c];
            qv[c] = dg * C[c] - o;
            acc += dvo[c] * qv[c];
        }
        *reinterpret_cast<float4*>(d_out + n0) = make_float4(dvo[0], dvo[1], dvo[2], dvo[3]);
        *reinterpret_cast<float4*>(q + n0) = make_float4(qv[0], qv[1], qv[2], qv[3]);
        return;
    }
    for (int n = n0; n < min(n0 + 4, g.nv); n++) {
        const uint16_t kd = kind[n];
        if ((kd & 3) != kFree) {
            d_out[n] = 0.f;
            q[n] = 0.f;
            continue;
        }
        int i, jj, kk;
        node_ijk(g, n, i, jj, kk);
        Stencil st;
        stencil(g, i, jj, kk, st);
        const float dn = z[n] + fb * d_in[n];
        float dg = 0.f, o = 0.f;
#pragma unroll
        for (int d = 0; d < 6; d++) {
            if (kd & (1u << (2 + d))) continue;
            dg += st.c[d];
            const int qq = st.q[d];
            o += st.c[d] * (z[qq] + fb * d_in[qq]);
        }
        const float qv = dg * dn - o;
        d_out[n] = dn;
        q[n] = qv;
        acc += dn * qv;
    }
}

// inverse diagonal of the reduced operator from the node's mirror mask
__device__ __forceinline__ float inv_diag_of(uint16_t kd, const float c[3]) {
    float dg = 0.f;
#pragma unroll
    for (int d = 0; d < 6; d++)
        if (!(kd & (1u << (2 + d)))) dg += c[d >> 1];
    return 1.f / dg;
}
// the 64 inverse diagonals (one per mirror mask) in shared memory, filled by the block
__device__ __forceinline__ void fill_inv_diag_table(float* tab, const GridDev& g) {
    if (threadIdx.x < 64) {
        const float c[3] = {g.inv_dx[0] * g.inv_dx[0], g.inv_dx[1] * g.inv_dx[1], g.inv_dx[2] * g.inv_dx[2]};
        tab[threadIdx.x] = inv_diag_of((uint16_t)(threadIdx.x << 2), c);
    }
    __syncthreads();
}
__device__ __forceinline__ float inv_diag_lookup(const float* tab, uint16_t kd) { return tab[(kd >> 2) & 63]; }

}  // namespace pic
