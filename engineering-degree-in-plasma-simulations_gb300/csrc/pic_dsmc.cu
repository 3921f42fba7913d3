// DSMC_MEX: VHS particle-particle collisions within cells (ch4/v3/src/Interactions.cpp:143-284).
//
// The reference walks the cells in order and, per cell, draws
//   n_groups = (int)(0.5 np1 np2 mpw0 (sigma v)_max dt / dV + 0.5)
// candidate pairs; a pair collides with probability sigma(v_rel) v_rel / (sigma v)_max and is
// scattered isotropically in its centre-of-mass frame.  Cells are independent, so the GPU form
// gives every cell one thread that runs that cell's groups in order on the species' sorted
// velocities (cell c owns [start[c], start[c+1])).  Draws come from one Philox-4x32-10 block keyed
// by (cell, call, tag, group) instead of one global MT19937 stream, and the one-species second
// partner is drawn directly from the np-1 other particles (the reference redraws until it
// differs: the same distribution).  (sigma v)_max follows the reference's rule: after a call
// with at least one collision it becomes the largest sigma v of that call's candidates; the
// update runs on the device, so a call needs no host round trip.
#include "pic_kernels.h"

namespace pic {
namespace {
__device__ __forceinline__ float warp_max_f(float v) {
#pragma unroll
    for (int o = 16; o; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__global__ void __launch_bounds__(128) k_dsmc(DsmcArgs a) {
    const float svmax = *a.svmax;
    const double coef = a.half_coef * (double)svmax;
    const int n1 = *a.n1, n2 = *a.n2;
    unsigned ncoll = 0, npairs = 0;
    float mx = 0.f;
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < a.nc) {
        const int s1 = a.start1[c];
        const int na = (c + 1 < a.nc ? a.start1[c + 1] : n1) - s1;
        int s2 = s1, nb = na;
        if (!a.one) {
            s2 = a.start2[c];
            nb = (c + 1 < a.nc ? a.start2[c + 1] : n2) - s2;
        }
        const bool active = a.one ? na >= 2 : (na >= 1 && nb >= 1);
        const int ng = active ? (int)((double)na * (double)nb * coef + 0.5) : 0;
        float4* v1p = a.vel1 + s1;
        float4* v2p = a.vel2 + s2;
        const unsigned range2 = a.one ? (unsigned)(na - 1) : (unsigned)nb;
        for (int gi = 0; gi < ng; gi++) {
            const uint4 r = philox4x32_10(make_uint4((unsigned)c, a.call, a.tag, (unsigned)gi), a.key);
            const unsigned i1 = mulhi32(r.x, (unsigned)na);
            unsigned i2 = mulhi32(r.y, range2);
            if (a.one && i2 >= i1) i2++;
            float4 v1 = v1p[i1], v2 = v2p[i2];
            const float dx = v1.x - v2.x, dy = v1.y - v2.y, dz = v1.z - v2.z;
            const float g2 = dx * dx + dy * dy + dz * dz;
            // K (g^2)^ex through the hardware base-2 logarithm and exponential (g2 = 0 gives 0)
            const float sv = a.K * exp2f(a.ex * __log2f(g2));
            mx = fmaxf(mx, sv);
            npairs++;
            if (!(sv > u01(r.z) * svmax)) continue;
            ncoll++;
            // the azimuth's uniform from the nine low bits of r.x, r.y, r.z (their high 23 bits
            // drew the pair and the acceptance), so a collision needs no second block
            const unsigned low27 = (r.x & 511u) | ((r.y & 511u) << 9) | ((r.z & 511u) << 18);
            const float ck = 2.f * u01(r.w) - 1.f;
            const float sk = sqrtf(fmaxf(1.f - ck * ck, 0.f));
            float se, ce;
            sincospif(2.f * ((float)low27 + 0.5f) * (1.0f / 134217728.0f), &se, &ce);
            const float gm = sqrtf(g2);
            const float r0 = gm * ck, r1 = gm * sk * ce, r2 = gm * sk * se;
            const float cx = a.f1 * v1.x + a.f2 * v2.x;
            const float cy = a.f1 * v1.y + a.f2 * v2.y;
            const float cz = a.f1 * v1.z + a.f2 * v2.z;
            v1.x = cx + a.f2 * r0;
            v1.y = cy + a.f2 * r1;
            v1.z = cz + a.f2 * r2;
            v2.x = cx - a.f1 * r0;
            v2.y = cy - a.f1 * r1;
            v2.z = cz - a.f1 * r2;
            v1p[i1] = v1;
            v2p[i2] = v2;
        }
    }
    // one atomic per warp for each counter
    const unsigned fc = __reduce_add_sync(0xffffffffu, ncoll), fp = __reduce_add_sync(0xffffffffu, npairs);
    mx = warp_max_f(mx);
    if ((threadIdx.x & 31) == 0 && fp > 0u) {
        atomicAdd(&a.stats[0], (unsigned long long)fc);
        atomicAdd(&a.stats[1], (unsigned long long)fp);
        atomicAdd(&a.stats[2], (unsigned long long)fc);
        atomicMax(a.svmax_step, __float_as_uint(mx));  // non-negative floats order as their bits
    }
}

// (sigma v)_max <- the call's largest candidate sigma v when the call collided (Interactions.cpp:214-217)
__global__ void k_dsmc_finish(DsmcArgs a) {
    if (a.stats[2] > 0) *a.svmax = __uint_as_float(*a.svmax_step);
    a.stats[2] = 0;
    *a.svmax_step = 0u;
}
}  // namespace

void launch_dsmc(const DsmcArgs& a, cudaStream_t s) {
    if (a.nc > 0) k_dsmc<<<(a.nc + 127) / 128, 128, 0, s>>>(a);
    k_dsmc_finish<<<1, 1, 0, s>>>(a);
}
}  // namespace pic
