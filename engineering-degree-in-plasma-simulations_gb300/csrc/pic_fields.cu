// Node-field kernels: charge density, E = -grad(phi), and the Poisson solvers.
//
// Reference behaviour followed (Misquic/Engineering-degree-in-Plasma-Simulations, ch4/v3/src):
//   node volumes   World::computeNodeVolumes          World.cpp:353-366
//   den, rho       Species::computeNumberDensity      Species.cpp:401-416; World::computeChargeDensity World.cpp:193-200
//   moving average Field::updateMovingAverage         Field.h:245-261
//   E field        PotentialSolver::computeEF         PotentialSolver.cpp:354-408
//   Poisson        PotentialSolver::solveGS / solveNRPCG, PotentialSolver.cpp:69-313
//
// The Poisson equation is solved on the reduced system of FREE nodes: for a FREE node p and a
// face neighbour q (periodic wrap applied), a FIXED q contributes its value to the right-hand
// side, a MIRROR q (a reference Neumann wall, which copies its inner neighbour) equals phi_p and
// drops out of both sides, and a FREE q is an unknown.  L phi = rho/eps0 with
//   (L x)_p = D_p x_p - sum_{q FREE or FIXED} c_q x_q,   D_p = sum_{q not MIRROR} c_q,  c = 1/dx^2.
// kind[n] (uint16): bits 0-1 node kind, bits 2-7 "neighbour d is MIRROR", bits 8-13
// "neighbour d is FIXED"; direction order -x +x -y +y -z +z.
#include <algorithm>
#include "pic_ff.cuh"
#include "pic_stencil.cuh"

namespace pic {

// ------------------------------------------------------------------------------------
// charge density: fixed-point number density -> den_s (per species) and rho
// ------------------------------------------------------------------------------------
// 64-bit integer -> FP32 through 32-bit conversions and one FMA (64-bit conversions run on the
// narrow FP64 pipe of this GPU): hi * 2^32 is exact, the FMA rounds once, the low word's own
// rounding (at most 2^7) lies below half an ulp of the result whenever hi != 0
__device__ __forceinline__ float u64_to_float(unsigned long long x) {
    return __fmaf_rn(__uint2float_rn((unsigned)(x >> 32)), 4294967296.f, __uint2float_rn((unsigned)x));
}
// signed: through the magnitude.  (Splitting a negative value directly gives hi = -1 and a low
// word near 2^32, whose rounding, up to 2^7, is then not small against a small result.)
__device__ __forceinline__ float i64_to_float(long long x) {
    const unsigned long long m = x < 0 ? 0ull - (unsigned long long)x : (unsigned long long)x;
    const float f = u64_to_float(m);
    return x < 0 ? -f : f;
}
__global__ void k_finalize_rho(FinalizeArgs a) {
    const GridDev& g = a.g;
    const float inv_base = g.inv_cell_vol;
    const int nn[3] = {g.ni, g.nj, g.nk}, stride[3] = {1, g.ni, g.ni * g.nj};
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < g.nv; n += gridDim.x * blockDim.x) {
        int ijk[3];
        node_ijk(g, n, ijk[0], ijk[1], ijk[2]);
        bool alias = false;
        unsigned fold = 0;
        float inv_vol = inv_base;  // boundary nodes have half volume per face: exact powers of two
        for (int d = 0; d < 3; d++) {
            if (g.periodic[d]) {
                if (ijk[d] == nn[d] - 1) alias = true;
                if (ijk[d] == 0) fold |= 1u << d;
            } else if (d == 2 && g.zslab) {
                const int lz = slab_local_z(g, ijk[2]);
                if (lz == 0 || lz == g.zslab - 1) inv_vol *= 2.f;  // faces of the instance slab
            } else if (ijk[d] == 0 || ijk[d] == nn[d] - 1) {
                inv_vol *= 2.f;
            }
        }
        if (alias) continue;  // written by the node it copies
        float den_out[kMaxSpecies];
        long long rho_fixed = 0;
        float rho_f = 0.f;
#pragma unroll
        for (int s = 0; s < kMaxSpecies; s++) {
            if (s >= a.ns) break;
            unsigned long long tot = a.acc[s][n];
            if (fold) {
                for (unsigned m = 1; m < 8; m++) {
                    if (m & ~fold) continue;
                    int node = n;
                    for (int d = 0; d < 3; d++)
                        if (m & (1u << d)) node += (nn[d] - 1) * stride[d];
                    tot += a.acc[s][node];
                }
            }
            den_out[s] = u64_to_float(tot) * (a.inv_scale[s] * inv_vol);
            if (a.int_path) rho_fixed += (long long)a.z[s] * (long long)tot;
            else rho_f += a.charge[s] * den_out[s];
        }
        const float rf = a.int_path ? i64_to_float(rho_fixed) * (a.rho_scale * inv_vol) : rho_f;
#pragma unroll
        for (int s = 0; s < kMaxSpecies; s++) {
            if (s >= a.ns) break;
            a.den[s][n] = den_out[s];
        }
        a.rho[n] = rf;
        if (fold) {
            for (unsigned m = 1; m < 8; m++) {
                if (m & ~fold) continue;
                int node = n;
                for (int d = 0; d < 3; d++)
                    if (m & (1u << d)) node += (nn[d] - 1) * stride[d];
#pragma unroll
                for (int s = 0; s < kMaxSpecies; s++) {
                    if (s >= a.ns) break;
                    a.den[s][node] = den_out[s];
                }
                a.rho[node] = rf;
            }
        }
    }
}
void launch_finalize_rho(const FinalizeArgs& a, cudaStream_t s, int grid) { k_finalize_rho<<<grid, 256, 0, s>>>(a); }

// dst += src over n floats, four per thread with 16-byte accesses where n allows
__global__ void k_add_f32(float* __restrict__ dst, const float* __restrict__ src, int n) {
    const int n4 = n >> 2;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n4; q += gridDim.x * blockDim.x) {
        float4 a = reinterpret_cast<float4*>(dst)[q];
        const float4 b = reinterpret_cast<const float4*>(src)[q];
        a.x += b.x;
        a.y += b.y;
        a.z += b.z;
        a.w += b.w;
        reinterpret_cast<float4*>(dst)[q] = a;
    }
    if (blockIdx.x == 0 && threadIdx.x < (n & 3)) dst[(n4 << 2) + threadIdx.x] += src[(n4 << 2) + threadIdx.x];
}
void launch_add(float* dst, const float* src, int n, cudaStream_t s, int grid) {
    k_add_f32<<<grid, 256, 0, s>>>(dst, src, n);
}

// avg = a*avg + b*den  (Field::updateMovingAverage with the sample count handled on the host)
__global__ void k_den_avg(float* avg, const float* den, int nv, float a, float b) {
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < nv; n += gridDim.x * blockDim.x)
        avg[n] = a * avg[n] + b * den[n];
}
void launch_den_avg(float* avg, const float* den, int nv, float a, float b, cudaStream_t s, int grid) {
    k_den_avg<<<grid, 256, 0, s>>>(avg, den, nv, a, b);
}

// ------------------------------------------------------------------------------------
// E = -grad(phi): central inside, second-order one-sided on non-periodic faces.  Potential
// differences are taken on the float-float values (exact high parts), the scaling in FP32.
// ------------------------------------------------------------------------------------
__device__ __forceinline__ float ffd(float2 a, float2 b) {
    FF d = ff_diff(a, b);
    return d.hi + d.lo;
}
__global__ void k_efield(GridDev g, const float2* __restrict__ phi, float4* __restrict__ ef) {
    const int stride[3] = {1, g.ni, g.ni * g.nj}, nn[3] = {g.ni, g.nj, g.nk};
    const float inv2[3] = {g.inv2dx[0], g.inv2dx[1], g.inv2dx[2]};
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < g.nv; n += gridDim.x * blockDim.x) {
        int ijk[3];
        node_ijk(g, n, ijk[0], ijk[1], ijk[2]);
        float e[3];
        for (int d = 0; d < 3; d++) {
            // along z, a stacked instance's slab is its own domain
            const int c = d == 2 ? slab_local_z(g, ijk[2]) : ijk[d];
            const int st = stride[d], N = (d == 2 && g.zslab) ? g.zslab : nn[d];
            float v;
            if (g.periodic[d]) {
                int cc = (c == N - 1) ? 0 : c;
                int base = n - (c - cc) * st;
                int im = base + (((cc == 0) ? N - 2 : cc - 1) - cc) * st;
                int ip = base + (((cc + 1 == N - 1) ? 0 : cc + 1) - cc) * st;
                v = ffd(phi[im], phi[ip]);
            } else if (N == 2) {
                v = c == 0 ? 2.f * ffd(phi[n], phi[n + st]) : 2.f * ffd(phi[n - st], phi[n]);  // first order
            } else if (c == 0) {
                // 3 phi_0 - 4 phi_1 + phi_2 = 3 (phi_0 - phi_1) - (phi_1 - phi_2)
                v = 3.f * ffd(phi[n], phi[n + st]) - ffd(phi[n + st], phi[n + 2 * st]);
            } else if (c == N - 1) {
                // -phi_{-2} + 4 phi_{-1} - 3 phi_0 = 3 (phi_{-1} - phi_0) - (phi_{-2} - phi_{-1})
                v = 3.f * ffd(phi[n - st], phi[n]) - ffd(phi[n - 2 * st], phi[n - st]);
            } else {
                v = ffd(phi[n - st], phi[n + st]);
            }
            e[d] = v * inv2[d];
        }
        ef[n] = make_float4(e[0], e[1], e[2], 0.f);
    }
}
void launch_efield(const GridDev& g, const float2* phi, float4* ef, cudaStream_t s, int grid) {
    k_efield<<<grid, 256, 0, s>>>(g, phi, ef);
}

// ------------------------------------------------------------------------------------
// field energy sum |E|^2 V_node / V_cell (World::getPE, World.cpp:108-119): node volumes halve
// on every non-periodic face (slab faces for stacked instances); the duplicate last plane of a
// periodic axis is skipped.  Per-thread sums in float-float, FP64 from the warp sums on; the
// host adds the block partials and scales by eps0/2 * V_cell.
// ------------------------------------------------------------------------------------
__global__ void k_field_energy(GridDev g, const float4* __restrict__ ef, double* part) {
    FF a{0.f, 0.f};
    for (int n = blockIdx.x * blockDim.x + threadIdx.x; n < g.nv; n += gridDim.x * blockDim.x) {
        int ijk[3];
        node_ijk(g, n, ijk[0], ijk[1], ijk[2]);
        const int nn[3] = {g.ni, g.nj, g.zslab ? g.zslab : g.nk};
        ijk[2] = slab_local_z(g, ijk[2]);
        float f = 1.f;
        bool alias = false;
        for (int d = 0; d < 3; d++) {
            const bool face = ijk[d] == 0 || ijk[d] == nn[d] - 1;
            if (g.periodic[d]) alias |= ijk[d] == nn[d] - 1;
            else if (face) f *= 0.5f;
        }
        if (alias) continue;
        const float4 e = __ldg(&ef[n]);
        FF e2 = ff_add(ff_add(two_prod(e.x, e.x), two_prod(e.y, e.y)), two_prod(e.z, e.z));
        a = ff_add(a, FF{e2.hi * f, e2.lo * f});  // f is a power of two: exact
    }
    __shared__ double s[32];
    double x = (double)a.hi + (double)a.lo;
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s[w];
        part[blockIdx.x] = t;
    }
}
void launch_field_energy(const GridDev& g, const float4* ef, double* part, cudaStream_t s, int grid) {
    k_field_energy<<<grid, 256, 0, s>>>(g, ef, part);
}

// ------------------------------------------------------------------------------------
// Residual of the reduced system in float-float, optionally after phi += e (ping-pong buffers)
//   r = b - L phi,  b = rho/eps0 + sum_{FIXED q} c_q phi_q ; partials: |r|^2, |b|^2
// (L phi)_p = sum_ax c_ax ((phi_p - phi_minus) + (phi_p - phi_plus)), a mirror neighbour taking
// phi_p: the differences are error-free in their high parts, the products by c and the sums are
// float-float, so r carries about 48 bits like an FP64 residual, on the FP32 pipe.  The
// correction's part L e is FP32 (e is small against phi).  The kernel also records rho and the
// FP32 boundary part of b, from which the next solve updates r without a full pass.
// ------------------------------------------------------------------------------------
// the residual at one FREE node from its potential pp, its six face neighbours pn[d] and, with
// apply_e, its correction ep and the neighbours' corrections en[d] (direction order -x +x -y +y
// -z +z); a MIRROR neighbour takes the node's own values
struct ResConst {
    FF cf[3];
    float c3[3];
    FF ie;
};
__device__ __forceinline__ void residual_node(const ResConst& K, uint16_t kd, float2 pp, const float2 (&pn)[6], float ep,
                                              const float (&en)[6], float rh, bool apply_e, float& rf, float& b,
                                              float& bfix, float2& np) {
    FF lphi{0.f, 0.f};
    float le = 0.f;
    bfix = 0.f;
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
        const int dm = 2 * ax, dp = 2 * ax + 1;
        const bool mm = kd & (1u << (2 + dm)), mp = kd & (1u << (2 + dp));
        const float2 pm = mm ? pp : pn[dm];
        const float2 pq = mp ? pp : pn[dp];
        const FF d1 = ff_diff(pp, pm), d2 = ff_diff(pp, pq);
        FF sd = two_sum(d1.hi, d2.hi);
        sd.lo += d1.lo + d2.lo;
        lphi = ff_add(lphi, ff_mul(K.cf[ax], sd));
        if (apply_e) le += K.c3[ax] * ((2.f * ep - (mm ? ep : en[dm])) - (mp ? ep : en[dp]));
        if (kd & (1u << (8 + dm))) bfix += K.c3[ax] * pm.x;
        if (kd & (1u << (8 + dp))) bfix += K.c3[ax] * pq.x;
    }
    if (apply_e) lphi = ff_add_f(lphi, le);
    FF src = two_prod(rh, K.ie.hi);
    src.lo += rh * K.ie.lo;
    const FF res = ff_add(src, ff_neg(lphi));
    np = pp;
    if (apply_e) {
        const FF v = ff_add_f(FF{pp.x, pp.y}, ep);
        np = make_float2(v.hi, v.lo);
    }
    rf = res.hi + res.lo;
    b = src.hi + bfix;
}

// neighbour rows of a group of nodes in row (j, k): y and z neighbours with the periodic wrap,
// clamped on non-periodic walls (a wall row holds no FREE node, its values go unused)
__device__ __forceinline__ void row_neighbours(const GridDev& g, int j, int k, int& jm, int& jp, int& km, int& kp) {
    jm = g.periodic[1] ? wrap_m(j, g.nj, 1) : max(j - 1, 0);
    jp = g.periodic[1] ? wrap_p(j, g.nj, 1) : min(j + 1, g.nj - 1);
    km = g.periodic[2] ? wrap_m(k, g.nk, 1) : max(k - 1, 0);
    kp = g.periodic[2] ? wrap_p(k, g.nk, 1) : min(k + 1, g.nk - 1);
}

// Four consecutive nodes of one row per thread and iteration.  When rows are a multiple of four
// nodes and the group does not touch the row ends, the group and its y / z neighbour rows are read
// with 16-byte loads and the two x neighbours with scalar loads; other groups go node by node.
// Capped at 80 registers (three CTAs per SM; a few bytes spill): measured faster than two CTAs at
// 116 registers or four at 64.
__global__ void __launch_bounds__(256, 3) k_residual(GridDev g, const float2* __restrict__ phi_in,
                                                  float2* __restrict__ phi_out, const float* __restrict__ e,
                                                  const float* __restrict__ rho, const uint16_t* __restrict__ kind,
                                                  float* __restrict__ r, double* gpart, int gstride, unsigned* ticket,
                                                  double* out, int apply_e, float* __restrict__ rho_prev,
                                                  float* __restrict__ bfix_out) {
    // float-float constants from the host: no FP64 arithmetic in the kernel
    constexpr float kIeHi = (float)(1.0 / kEps0);
    constexpr float kIeLo = (float)(1.0 / kEps0 - (double)kIeHi);
    ResConst K;
    for (int ax = 0; ax < 3; ax++) {
        K.cf[ax] = FF{g.c_hi[ax], g.c_lo[ax]};
        K.c3[ax] = g.inv_dx[ax] * g.inv_dx[ax];
    }
    K.ie = FF{kIeHi, kIeLo};
    const bool ae = apply_e != 0;
    const bool rows4 = (g.ni & 3) == 0;
    const int nij = g.ni * g.nj;
    const float ie_f = kIeHi;
    float acc_r = 0.f, acc_b = 0.f, acc_s = 0.f;  // per-thread sums in FP32, block and grid sums in FP64
    const int ngroups = (g.nv + 3) >> 2;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < ngroups; q += gridDim.x * blockDim.x) {
        const int n0 = q << 2;
        int i0, j, k;
        node_ijk(g, n0, i0, j, k);
        if (rows4) {
            // every group of a row, its ends included: see spmv_group for the x neighbours at the ends
            const bool xend = i0 + 4 == g.ni, wrapx = g.periodic[0] != 0;
            const int ixm = i0 > 0 ? n0 - 1 : (wrapx ? n0 + g.ni - 2 : n0);
            const int ixp = xend ? (wrapx ? n0 - i0 : n0 + 3) : n0 + 4;
            int jm, jp, km, kp;
            row_neighbours(g, j, k, jm, jp, km, kp);
            const int rowm = (k * g.nj + jm) * g.ni + i0, rowp = (k * g.nj + jp) * g.ni + i0;
            const int plm = (km * g.nj + j) * g.ni + i0, plp = (kp * g.nj + j) * g.ni + i0;
            const ushort4 k4 = *reinterpret_cast<const ushort4*>(kind + n0);
            const unsigned short kv[4] = {k4.x, k4.y, k4.z, k4.w};
            float2 P[4], Ym[4], Yp[4], Zm[4], Zp[4];
            auto load4 = [&](const float2* src, float2 (&dst)[4]) {
                const float4 a0 = *reinterpret_cast<const float4*>(src);
                const float4 a1 = *reinterpret_cast<const float4*>(src + 2);
                dst[0] = make_float2(a0.x, a0.y);
                dst[1] = make_float2(a0.z, a0.w);
                dst[2] = make_float2(a1.x, a1.y);
                dst[3] = make_float2(a1.z, a1.w);
            };
            load4(phi_in + n0, P);
            load4(phi_in + rowm, Ym);
            load4(phi_in + rowp, Yp);
            load4(phi_in + plm, Zm);
            load4(phi_in + plp, Zp);
            const float2 xm = phi_in[ixm], xp = phi_in[ixp];
            float E[4] = {0.f, 0.f, 0.f, 0.f}, EYm[4] = {0.f, 0.f, 0.f, 0.f}, EYp[4] = {0.f, 0.f, 0.f, 0.f},
                  EZm[4] = {0.f, 0.f, 0.f, 0.f}, EZp[4] = {0.f, 0.f, 0.f, 0.f}, exm = 0.f, exp_ = 0.f;
            if (ae) {
                auto ld = [&](const float* src, float (&dst)[4]) {
                    const float4 a0 = *reinterpret_cast<const float4*>(src);
                    dst[0] = a0.x;
                    dst[1] = a0.y;
                    dst[2] = a0.z;
                    dst[3] = a0.w;
                };
                ld(e + n0, E);
                ld(e + rowm, EYm);
                ld(e + rowp, EYp);
                ld(e + plm, EZm);
                ld(e + plp, EZp);
                exm = e[ixm];
                exp_ = e[ixp];
            }
            const float4 h4 = *reinterpret_cast<const float4*>(rho + n0);
            const float hv[4] = {h4.x, h4.y, h4.z, h4.w};
            float rv[4], bf[4];
            float2 pv[4];
#pragma unroll
            for (int c = 0; c < 4; c++) {
                rv[c] = 0.f;
                bf[c] = 0.f;
                pv[c] = P[c];
                if ((kv[c] & 3) != kFree) continue;
                const bool wr = c == 3 || (c == 2 && xend && wrapx);
                const float2 pn[6] = {c == 0 ? xm : P[c - 1], wr ? xp : P[c + 1], Ym[c], Yp[c], Zm[c], Zp[c]};
                const float en[6] = {c == 0 ? exm : E[c - 1], wr ? exp_ : E[c + 1], EYm[c], EYp[c], EZm[c], EZp[c]};
                float b;
                residual_node(K, kv[c], P[c], pn, E[c], en, hv[c], ae, rv[c], b, bf[c], pv[c]);
                acc_r += rv[c] * rv[c];
                acc_b += b * b;
                const float sc = hv[c] * ie_f;
                acc_s += sc * sc;
            }
            *reinterpret_cast<float4*>(r + n0) = make_float4(rv[0], rv[1], rv[2], rv[3]);
            if (ae) {
                *reinterpret_cast<float4*>(phi_out + n0) = make_float4(pv[0].x, pv[0].y, pv[1].x, pv[1].y);
                *reinterpret_cast<float4*>(phi_out + n0 + 2) = make_float4(pv[2].x, pv[2].y, pv[3].x, pv[3].y);
            }
            if (rho_prev) *reinterpret_cast<float4*>(rho_prev + n0) = h4;
            if (bfix_out) *reinterpret_cast<float4*>(bfix_out + n0) = make_float4(bf[0], bf[1], bf[2], bf[3]);
            continue;
        }
        // node by node
        for (int n = n0; n < min(n0 + 4, g.nv); n++) {
            const uint16_t kd = kind[n];
            if ((kd & 3) != kFree) {
                if (ae) phi_out[n] = phi_in[n];
                r[n] = 0.f;
                continue;
            }
            int i, jj, kk;
            node_ijk(g, n, i, jj, kk);
            Stencil st;
            stencil(g, i, jj, kk, st);
            float2 pn[6];
            float en[6];
#pragma unroll
            for (int d = 0; d < 6; d++) {
                pn[d] = phi_in[st.q[d]];
                en[d] = ae ? e[st.q[d]] : 0.f;
            }
            const float rh = rho[n];
            float rf, b, bfix;
            float2 np;
            residual_node(K, kd, phi_in[n], pn, ae ? e[n] : 0.f, en, rh, ae, rf, b, bfix, np);
            r[n] = rf;
            if (ae) phi_out[n] = np;
            acc_r += rf * rf;
            acc_b += b * b;
            const float sc = rh * ie_f;
            acc_s += sc * sc;
            if (rho_prev) rho_prev[n] = rh;
            if (bfix_out) bfix_out[n] = bfix;
        }
    }
    const float v[4] = {acc_r, acc_b, 0.f, acc_s};
    grid_sum<4>(v, gpart, gstride, ticket, out);
}
void launch_residual(const GridDev& g, SolveWork& w, int apply_e, cudaStream_t s, float* rho_prev, float* bfix_out) {
    const float2* in = w.phi;
    float2* out = apply_e ? w.phi_alt : w.phi;
    k_residual<<<stream_blocks(g), 256, 0, s>>>(g, in, out, w.e, w.rho,
                                                          reinterpret_cast<const uint16_t*>(w.kind), w.r, w.gpart,
                                                          w.gstride, w.ticket, w.scal + kS_R2, apply_e, rho_prev,
                                                          bfix_out);
    if (apply_e) {
        float2* t = w.phi;
        w.phi = w.phi_alt;
        w.phi_alt = t;
    }
}
// residual of the next solve without a full pass: r += (rho - rho_prev) / eps0 on FREE nodes
// (r holds the residual of the current phi, rounded to FP32); |r|^2, |b|^2, the squared norm
// of the update t = (rho - rho_prev) / eps0 and |rho / eps0|^2 into out[0..3] (the host bounds
// the rounding error of r from |t| and |r|).
// Four consecutive nodes per thread and iteration with 16-byte loads.
__global__ void __launch_bounds__(256) k_rhs_update(GridDev g, float* __restrict__ r, const float* __restrict__ rho,
                                                    float* __restrict__ rho_prev, const float* __restrict__ bfix,
                                                    const uint16_t* __restrict__ kind, double* gpart, int gstride,
                                                    unsigned* ticket, double* out) {
    const float inv_eps0_f = (float)(1.0 / kEps0);
    float acc_r = 0.f, acc_b = 0.f, acc_t = 0.f, acc_s = 0.f;
    const int ng = g.nv >> 2;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < ng; q += gridDim.x * blockDim.x) {
        const float4 r4 = reinterpret_cast<const float4*>(r)[q];
        const float4 h4 = reinterpret_cast<const float4*>(rho)[q];
        const float4 p4 = reinterpret_cast<const float4*>(rho_prev)[q];
        const float4 f4 = reinterpret_cast<const float4*>(bfix)[q];
        const ushort4 k4 = reinterpret_cast<const ushort4*>(kind)[q];
        float rv[4] = {r4.x, r4.y, r4.z, r4.w}, hv[4] = {h4.x, h4.y, h4.z, h4.w};
        const float pv[4] = {p4.x, p4.y, p4.z, p4.w}, fv[4] = {f4.x, f4.y, f4.z, f4.w};
        const unsigned short kv[4] = {k4.x, k4.y, k4.z, k4.w};
#pragma unroll
        for (int c = 0; c < 4; c++) {
            if ((kv[c] & 3) != kFree) continue;
            const float t = (hv[c] - pv[c]) * inv_eps0_f;
            rv[c] += t;
            const float sc = hv[c] * inv_eps0_f;
            const float b = sc + fv[c];
            acc_r += rv[c] * rv[c];
            acc_b += b * b;
            acc_t += t * t;
            acc_s += sc * sc;
        }
        reinterpret_cast<float4*>(r)[q] = make_float4(rv[0], rv[1], rv[2], rv[3]);
        reinterpret_cast<float4*>(rho_prev)[q] = h4;
    }
    // the last nv % 4 nodes
    if (blockIdx.x == 0 && threadIdx.x < (g.nv & 3)) {
        const int n = (ng << 2) + threadIdx.x;
        if ((kind[n] & 3) == kFree) {
            const float rh = rho[n];
            const float t = (rh - rho_prev[n]) * inv_eps0_f;
            const float rn = r[n] + t;
            r[n] = rn;
            const float sc = rh * inv_eps0_f;
            const float b = sc + bfix[n];
            acc_r += rn * rn;
            acc_b += b * b;
            acc_t += t * t;
            acc_s += sc * sc;
        }
        rho_prev[n] = rho[n];
    }
    const float v[4] = {acc_r, acc_b, acc_t, acc_s};
    grid_sum<4>(v, gpart, gstride, ticket, out);
}
void launch_rhs_update(const GridDev& g, SolveWork& w, float* rho_prev, const float* bfix, cudaStream_t s) {
    k_rhs_update<<<stream_blocks(g), 256, 0, s>>>(g, w.r, w.rho, rho_prev, bfix,
                                                            reinterpret_cast<const uint16_t*>(w.kind), w.gpart,
                                                            w.gstride, w.ticket, w.scal + kS_R2);
}
// sums nslots consecutive partial rows (grid-sized) into out[0..nslots)
__global__ void k_reduce_partials(const double* part, int nblocks, double* out) {
    double t = sum_partials(part + blockIdx.x * kParts, nblocks);
    if (threadIdx.x == 0) out[blockIdx.x] = t;
}
void launch_reduce_partials(const double* part, int nslots, int nblocks, double* out, cudaStream_t s) {
    // slot rows are kParts apart; the producing kernel wrote its first nblocks entries
    k_reduce_partials<<<nslots, 256, 0, s>>>(part, nblocks, out);
}

// ------------------------------------------------------------------------------------
// FP32 red-black SOR on the correction equation L e = r (e = 0 on non-FREE nodes)
// ------------------------------------------------------------------------------------
// A periodic axis with an odd number of distinct nodes (n-1 odd) closes an odd cycle, so the
// last distinct index n-2 ("seam") has a same-colour neighbour across the wrap.  Seam nodes are
// left out of the red and black passes and relaxed (omega = 1) in a third pass.
__device__ __forceinline__ bool on_seam(const GridDev& g, int i, int j, int k) {
    return (g.periodic[0] && ((g.ni - 1) & 1) && i == g.ni - 2) ||
           (g.periodic[1] && ((g.nj - 1) & 1) && j == g.nj - 2) ||
           (g.periodic[2] && ((g.nk - 1) & 1) && k == g.nk - 2);
}
__device__ __forceinline__ void sor_update(const GridDev& g, float* __restrict__ e, const float* __restrict__ r,
                                           const uint16_t* __restrict__ kind, float omega, int i, int j, int k) {
    const int n = (k * g.nj + j) * g.ni + i;
    const uint16_t kd = kind[n];
    if ((kd & 3) != kFree) return;
    Stencil s;
    stencil(g, i, j, k, s);
    float diag = 0.f, off = 0.f;
#pragma unroll
    for (int d = 0; d < 6; d++) {
        if (kd & (1u << (2 + d))) continue;
        diag += s.c[d];
        off += s.c[d] * e[s.q[d]];  // zero on FIXED neighbours
    }
    const float en = e[n];
    e[n] = en + omega * ((r[n] + off) / diag - en);
}
__global__ void k_rbsor(GridDev g, float* __restrict__ e, const float* __restrict__ r,
                        const uint16_t* __restrict__ kind, float omega, int color) {
    // thread t -> (m, j, k) with i = 2m + parity of the requested colour
    const int half = (g.ni + 1) / 2;
    const int total = half * g.nj * g.nk;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < total; t += gridDim.x * blockDim.x) {
        int m = t % half, jk = t / half;
        int j = jk % g.nj, k = jk / g.nj;
        int i = 2 * m + ((color + j + k) & 1);
        if (i >= g.ni || on_seam(g, i, j, k)) continue;
        sor_update(g, e, r, kind, omega, i, j, k);
    }
}
__global__ void k_rbsor_seam(GridDev g, float* __restrict__ e, const float* __restrict__ r,
                             const uint16_t* __restrict__ kind) {
    const int nx = (g.periodic[0] && ((g.ni - 1) & 1)) ? g.nj * g.nk : 0;
    const int ny = (g.periodic[1] && ((g.nj - 1) & 1)) ? g.ni * g.nk : 0;
    const int nz = (g.periodic[2] && ((g.nk - 1) & 1)) ? g.ni * g.nj : 0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nx + ny + nz; t += gridDim.x * blockDim.x) {
        int i, j, k;
        if (t < nx) {
            i = g.ni - 2;
            j = t % g.nj;
            k = t / g.nj;
        } else if (t < nx + ny) {
            int u = t - nx;
            j = g.nj - 2;
            i = u % g.ni;
            k = u / g.ni;
        } else {
            int u = t - nx - ny;
            k = g.nk - 2;
            i = u % g.ni;
            j = u / g.ni;
        }
        sor_update(g, e, r, kind, 1.0f, i, j, k);
    }
}
void launch_rbsor_sweeps(const GridDev& g, SolveWork& w, float omega, int sweeps, cudaStream_t s) {
    const uint16_t* kd = reinterpret_cast<const uint16_t*>(w.kind);
    const int grid = ((g.ni + 1) / 2 * g.nj * g.nk + 255) / 256;  // one thread per node of a colour
    const bool seam = (g.periodic[0] && ((g.ni - 1) & 1)) || (g.periodic[1] && ((g.nj - 1) & 1)) ||
                      (g.periodic[2] && ((g.nk - 1) & 1));
    for (int it = 0; it < sweeps; it++) {
        k_rbsor<<<grid, 256, 0, s>>>(g, w.e, w.r, kd, omega, 0);
        k_rbsor<<<grid, 256, 0, s>>>(g, w.e, w.r, kd, omega, 1);
        if (seam) k_rbsor_seam<<<256, 256, 0, s>>>(g, w.e, w.r, kd);
    }
}

// ------------------------------------------------------------------------------------
// FP32 flexible (Polak-Ribiere) Jacobi-preconditioned CG on L e = r, e0 = 0.
// Two kernels per iteration; d is ping-ponged so the direction update fuses into the SpMV:
//   K1: d' = z + beta d ; q = L0 d' ; partial d'.q          (beta = 0 on the first iteration)
//   K2: alpha = rz/dq ; e += alpha d' ; r -= alpha q ; z' = r/D ; partials r.z', r.z, r.r
// scalars: scal[0..1] rz (double-buffered by iteration parity); flag[0] set when r.r <= target
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_pcg_init(GridDev g, const float* __restrict__ r, float* __restrict__ z,
                                                  float* __restrict__ e, float* __restrict__ d,
                                                  const uint16_t* __restrict__ kind, double* gpart, int gstride,
                                                  unsigned* ticket, double* scal, int* flag) {
    if (blockIdx.x == 0 && threadIdx.x == 0) flag[0] = 0;
    const float c3[3] = {g.inv_dx[0] * g.inv_dx[0], g.inv_dx[1] * g.inv_dx[1], g.inv_dx[2] * g.inv_dx[2]};
    float acc = 0.f;
    const int ng = g.nv >> 2;
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < ng; q += gridDim.x * blockDim.x) {
        const float4 r4 = reinterpret_cast<const float4*>(r)[q];
        const ushort4 k4 = reinterpret_cast<const ushort4*>(kind)[q];
        const float rv[4] = {r4.x, r4.y, r4.z, r4.w};
        const unsigned short kv[4] = {k4.x, k4.y, k4.z, k4.w};
        float zv[4];
#pragma unroll
        for (int c = 0; c < 4; c++) {
            zv[c] = (kv[c] & 3) == kFree ? rv[c] * inv_diag_of(kv[c], c3) : 0.f;
            acc += rv[c] * zv[c];
        }
        reinterpret_cast<float4*>(z)[q] = make_float4(zv[0], zv[1], zv[2], zv[3]);
        reinterpret_cast<float4*>(e)[q] = zero4;
        reinterpret_cast<float4*>(d)[q] = zero4;
    }
    if (blockIdx.x == 0 && threadIdx.x < (g.nv & 3)) {
        const int n = (ng << 2) + threadIdx.x;
        const uint16_t kd = kind[n];
        const float zz = (kd & 3) == kFree ? r[n] * inv_diag_of(kd, c3) : 0.f;
        z[n] = zz;
        e[n] = 0.f;
        d[n] = 0.f;
        acc += r[n] * zz;
    }
    const float v[1] = {acc};
    grid_sum<1>(v, gpart, gstride, ticket, scal + kS_RZN);  // r.z
}
__global__ void __launch_bounds__(256) k_pcg_k1(GridDev g, const float* __restrict__ z,
                                                         const float* __restrict__ d_in, float* __restrict__ d_out,
                                                         float* __restrict__ q, const uint16_t* __restrict__ kind,
                                                         double* gpart, int gstride, unsigned* ticket, double* scal,
                                                         int* flag, int it, double target_rr) {
    // scalars of the previous iteration (r.z', r.z, r.r), evaluated once per block in FP64
    __shared__ float s_beta;
    __shared__ int s_stop;
    if (threadIdx.x == 0) {
        const double rz_new = scal[kS_RZN];
        double beta = 0.0;
        int stop = 0;
        if (it > 0) {
            const double rzo = scal[kS_RZO], rr = scal[kS_RR];
            if (rr <= target_rr || flag[0]) {
                stop = 1;
                if (blockIdx.x == 0 && !flag[0]) {
                    flag[1] = it;  // iterations completed
                    flag[0] = 1;
                }
            } else {
                beta = (rz_new - rzo) / scal[kS_RZ + ((it - 1) & 1)];
            }
        }
        if (blockIdx.x == 0 && !stop) scal[kS_RZ + (it & 1)] = rz_new;
        s_beta = (float)beta;
        s_stop = stop;
    }
    __syncthreads();
    if (s_stop) return;
    const float fb = s_beta;
    float facc = 0.f;
    const int ngroups = (g.nv + 3) >> 2;
    for (int qg = blockIdx.x * blockDim.x + threadIdx.x; qg < ngroups; qg += gridDim.x * blockDim.x)
        spmv_group(g, qg << 2, z, d_in, d_out, q, kind, fb, facc);
    const float v[1] = {facc};
    grid_sum<1>(v, gpart, gstride, ticket, scal + kS_DQ);
}
__global__ void __launch_bounds__(256) k_pcg_k2(GridDev g, const float* __restrict__ d, const float* __restrict__ q,
                                                float* __restrict__ e, float* __restrict__ r, float* __restrict__ z,
                                                const uint16_t* __restrict__ kind, double* gpart, int gstride,
                                                unsigned* ticket, double* scal, int* flag, int it) {
    if (flag[0]) return;
    __shared__ float s_alpha;  // alpha = rz / dq, once per block in FP64
    if (threadIdx.x == 0) {
        const double dq = scal[kS_DQ];
        s_alpha = dq != 0.0 ? (float)(scal[kS_RZ + (it & 1)] / dq) : 0.f;
    }
    __syncthreads();
    const float alpha = s_alpha;
    const float c3[3] = {g.inv_dx[0] * g.inv_dx[0], g.inv_dx[1] * g.inv_dx[1], g.inv_dx[2] * g.inv_dx[2]};
    float f0 = 0.f, f1 = 0.f, f2 = 0.f;
    const int ng = g.nv >> 2;
    for (int qq = blockIdx.x * blockDim.x + threadIdx.x; qq < ng; qq += gridDim.x * blockDim.x) {
        const float4 d4 = reinterpret_cast<const float4*>(d)[qq];
        const float4 q4 = reinterpret_cast<const float4*>(q)[qq];
        const float4 e4 = reinterpret_cast<const float4*>(e)[qq];
        const float4 r4 = reinterpret_cast<const float4*>(r)[qq];
        const float4 z4 = reinterpret_cast<const float4*>(z)[qq];
        const ushort4 k4 = reinterpret_cast<const ushort4*>(kind)[qq];
        const float dv[4] = {d4.x, d4.y, d4.z, d4.w}, qv[4] = {q4.x, q4.y, q4.z, q4.w};
        float ev[4] = {e4.x, e4.y, e4.z, e4.w}, rv[4] = {r4.x, r4.y, r4.z, r4.w}, zv[4] = {z4.x, z4.y, z4.z, z4.w};
        const unsigned short kv[4] = {k4.x, k4.y, k4.z, k4.w};
#pragma unroll
        for (int c = 0; c < 4; c++) {
            if ((kv[c] & 3) != kFree) continue;
            ev[c] += alpha * dv[c];
            const float rn = rv[c] - alpha * qv[c];
            const float zn = rn * inv_diag_of(kv[c], c3);
            f0 += rn * zn;
            f1 += rn * zv[c];
            f2 += rn * rn;
            rv[c] = rn;
            zv[c] = zn;
        }
        reinterpret_cast<float4*>(e)[qq] = make_float4(ev[0], ev[1], ev[2], ev[3]);
        reinterpret_cast<float4*>(r)[qq] = make_float4(rv[0], rv[1], rv[2], rv[3]);
        reinterpret_cast<float4*>(z)[qq] = make_float4(zv[0], zv[1], zv[2], zv[3]);
    }
    if (blockIdx.x == 0 && threadIdx.x < (g.nv & 3)) {
        const int n = (ng << 2) + threadIdx.x;
        const uint16_t kd = kind[n];
        if ((kd & 3) == kFree) {
            e[n] += alpha * d[n];
            const float rn = r[n] - alpha * q[n];
            const float zn = rn * inv_diag_of(kd, c3);
            f0 += rn * zn;
            f1 += rn * z[n];
            f2 += rn * rn;
            r[n] = rn;
            z[n] = zn;
        }
    }
    const float v[3] = {f0, f1, f2};
    grid_sum<3>(v, gpart, gstride, ticket, scal + kS_RZN);  // r.z', r.z, r.r
}
void launch_pcg_init(const GridDev& g, SolveWork& w, cudaStream_t s) {
    k_pcg_init<<<stream_blocks(g), 256, 0, s>>>(g, w.r, w.z, w.e, w.d,
                                                          reinterpret_cast<const uint16_t*>(w.kind), w.gpart,
                                                          w.gstride, w.ticket, w.scal, w.flag);
}
// one iteration; d ping-pongs between two buffers
void launch_pcg_iter_impl(const GridDev& g, SolveWork& w, float* d_in, float* d_out, int it, double target_rr,
                          cudaStream_t s) {
    const uint16_t* kd = reinterpret_cast<const uint16_t*>(w.kind);
    k_pcg_k1<<<cg_blocks(g), 256, 0, s>>>(g, w.z, d_in, d_out, w.q, kd, w.gpart, w.gstride, w.ticket, w.scal, w.flag,
                                         it, target_rr);
    k_pcg_k2<<<stream_blocks(g), 256, 0, s>>>(g, d_out, w.q, w.e, w.r, w.z, kd, w.gpart, w.gstride, w.ticket,
                                                 w.scal, w.flag, it);
}

// ------------------------------------------------------------------------------------
// MIRROR nodes take the clamped interior value, then ALIAS nodes their periodic source
// ------------------------------------------------------------------------------------
// phi[dst] = phi[src] over a list of node pairs: the MIRROR nodes first (their clamped interior
// node), then the ALIAS nodes (their periodic source, which may be a MIRROR node)
__global__ void k_fill_pairs(const int2* __restrict__ pairs, int n, float2* phi) {
    for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < n; x += gridDim.x * blockDim.x) {
        const int2 p = pairs[x];
        phi[p.x] = phi[p.y];
    }
}
void launch_fill_aux(const int2* pairs, int n_mirror, int n_alias, float2* phi, cudaStream_t s) {
    if (n_mirror > 0) k_fill_pairs<<<std::min(1216, (n_mirror + 255) / 256), 256, 0, s>>>(pairs, n_mirror, phi);
    if (n_alias > 0)
        k_fill_pairs<<<std::min(1216, (n_alias + 255) / 256), 256, 0, s>>>(pairs + n_mirror, n_alias, phi);
}

}  // namespace pic
