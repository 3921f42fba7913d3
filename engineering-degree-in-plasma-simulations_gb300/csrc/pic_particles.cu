// Particle kernels: fused collide + push + deposit, compaction, counting sort by cell,
// host <-> device conversion and the synthetic loaders.
//
// Reference behaviour followed (Misquic/Engineering-degree-in-Plasma-Simulations, ch4/v3/src):
//   push           Species::advanceElectronsSerial      Species.cpp:356-399
//   gather         Field<Vec3>::gather                  Field.h:200-232
//   deposit        Species::computeNumberDensity        Species.cpp:401-416 (Field::scatter, Field.h:156-199)
//   bounds         World::inBounds / inObject           World.cpp:201-205, 293-301
//   collisions     MC_MEX_Ionization::collide, IONIZE_1 Interactions.cpp:845-947
//   creation       Species::addParticle                 Species.cpp:420-434
//   cell lists     Species::sortIndexes                 Species.cpp:905-915
#include <climits>
#include "pic_ff.cuh"
#include "pic_kernels.h"

namespace pic {

constexpr int kThreads = 256;
constexpr int kPPT = 4;                     // particles per thread per chunk
constexpr int kChunk = kThreads * kPPT;     // particles per chunk
constexpr int kSeg = 256;                   // nodes per staged row segment
constexpr int kMargin = 2;                  // deposit window starts this many nodes below the gather window
constexpr int kHalfWin = (kSeg - kMargin - 2) / 2;  // staged base nodes either side of the chunk's anchor
constexpr int kPushBlocksPerSM = 3;         // resident push CTAs per SM (80 registers, 56 KB shared)
// shared memory of the push: the next chunk's particles (pos, vel), the E rows (float4) and the
// fixed-point deposit tile (a low-word and a high-word plane of 32-bit counters), four rows of
// kSeg nodes each
constexpr size_t kPbufBytes = (size_t)kChunk * 2 * sizeof(float4);
constexpr size_t kPushSmem = kPbufBytes + 4 * kSeg * sizeof(float4) + 2 * 4 * kSeg * sizeof(unsigned);
constexpr long long kWaitLimit = kMbarWaitPolls;  // mbarrier polls of a drain before giving up

// ------------------------------------------------------------------------------------
// mbarrier + bulk-copy (TMA) helpers
// ------------------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// global -> shared bulk copy completing on an mbarrier; both addresses 16-byte aligned,
// size a multiple of 16 bytes (node rows of float4)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
// bounded wait: returns false if the copies did not land within `limit` polls
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity,
                                                  long long limit = kWaitLimit) {
    for (long long it = 0; it < limit; it++)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// ------------------------------------------------------------------------------------
// cross sections (MC_MEX_Ionization::evaluateSigmaColl / evaluateSigmaIon,
// Interactions.cpp:541-566) in FP32
// ------------------------------------------------------------------------------------
__device__ float sigma_coll(const CollDev& c, float E) {
    int lo = 0, hi = c.tn;  // first index with tE >= E (std::map::lower_bound)
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (__ldg(&c.tE[mid]) < E) lo = mid + 1;
        else hi = mid;
    }
    if (lo == 0) return __ldg(&c.tS[0]);
    if (lo == c.tn) return __ldg(&c.tS[c.tn - 1]);
    float x1 = __ldg(&c.tE[lo - 1]), x2 = __ldg(&c.tE[lo]), y1 = __ldg(&c.tS[lo - 1]), y2 = __ldg(&c.tS[lo]);
    return y1 + (E - x1) * (y2 - y1) / (x2 - x1);
}
__device__ float sigma_ion(const CollDev& c, float E) {
    if (E <= c.E_ion_eV) return 0.f;
    if (c.sig_kind == 0) return c.sig_a * logf(E / c.sig_b) / E * expf(-c.sig_c / E);
    float I = c.E_ion_eV, x = E / I;
    return c.sig_A * logf(x) / (E * I) * (1.f - c.sig_b * expf(-c.sig_c * (x - 1.f)));
}

// draw stream after the candidate test: blocks 2, 3, ... of (id_lo, id_hi, step, block)
struct Draws {
    uint4 ctr;
    uint2 key;
    uint4 buf;
    int pos;
    __device__ float next() {
        if (pos >= 4) {
            ctr.w += 1;
            buf = philox4x32_10(ctr, key);
            pos = 0;
        }
        unsigned v = pos == 0 ? buf.x : pos == 1 ? buf.y : pos == 2 ? buf.z : buf.w;
        pos++;
        return u01(v);
    }
};

// MC_MEX_Ionization::newVelocityElecton, LAB form (Interactions.cpp:845-870), keeping the
// reference's unnormalised perpendicular basis (i x u and u x (i x u)).
__device__ float3 new_vel_electron(const CollDev& c, float E, float3 u, float r_pow, float r_phi) {
    const float kPiRef = 3.141592653f;
    float cos_ksi = (2.f + E - 2.f * powf(1.f + E, r_pow)) / E;
    float sin_ksi = sqrtf(fmaxf(1.f - cos_ksi * cos_ksi, 0.f));
    float sp, cp;
    sincosf(2.f * kPiRef * r_phi, &sp, &cp);
    float v_mag = sqrtf(E * c.two_q_over_me);
    float3 a = make_float3(0.f, -u.z, u.y);  // (1,0,0) x u
    float3 b = make_float3(u.y * a.z - u.z * a.y, u.z * a.x - u.x * a.z, u.x * a.y - u.y * a.x);
    return make_float3((cos_ksi * u.x + a.x * sin_ksi * sp + b.x * sin_ksi * cp) * v_mag,
                       (cos_ksi * u.y + a.y * sin_ksi * sp + b.y * sin_ksi * cp) * v_mag,
                       (cos_ksi * u.z + a.z * sin_ksi * sp + b.z * sin_ksi * cp) * v_mag);
}

// ------------------------------------------------------------------------------------
// push helpers
// ------------------------------------------------------------------------------------
struct Tile {
    const float4* etile;  // staged E rows (row m at etile + m*kSeg), or nullptr
    unsigned* dtile;      // deposit tile: low words of row m at dtile + m*kSeg, high words 4*kSeg on, or nullptr
    int lo;               // first base node of the staged window
    int span;             // base nodes lo .. lo + span are staged
    int off[4];           // node offsets of the four rows: 0, ni, ni*nj, ni*nj+ni
};

// E at the eight corners of the cell whose base node is b (Field::gather order)
__device__ __forceinline__ float3 gather_e(const PushArgs& a, const Tile& t, int b, float3 o) {
    const float4* e0;
    int r1, r2, r3;
    if (t.etile && (unsigned)(b - t.lo) <= (unsigned)t.span) {
        e0 = t.etile + (b - t.lo);
        r1 = kSeg;
        r2 = 2 * kSeg;
        r3 = 3 * kSeg;
    } else {
        e0 = a.ef + b;
        r1 = t.off[1];
        r2 = t.off[2];
        r3 = t.off[3];
    }
    float4 e000 = e0[0], e100 = e0[1], e010 = e0[r1], e110 = e0[r1 + 1];
    float4 e001 = e0[r2], e101 = e0[r2 + 1], e011 = e0[r3], e111 = e0[r3 + 1];
    // trilinear weights as three nested linear interpolations (x, then y, then z)
    auto lx = [&](const float4& p, const float4& q) {
        return make_float3(fmaf(o.x, q.x - p.x, p.x), fmaf(o.x, q.y - p.y, p.y), fmaf(o.x, q.z - p.z, p.z));
    };
    const float3 c00 = lx(e000, e100), c10 = lx(e010, e110), c01 = lx(e001, e101), c11 = lx(e011, e111);
    const float3 c0 = make_float3(fmaf(o.y, c10.x - c00.x, c00.x), fmaf(o.y, c10.y - c00.y, c00.y),
                                  fmaf(o.y, c10.z - c00.z, c00.z));
    const float3 c1 = make_float3(fmaf(o.y, c11.x - c01.x, c01.x), fmaf(o.y, c11.y - c01.y, c01.y),
                                  fmaf(o.y, c11.z - c01.z, c01.z));
    return make_float3(fmaf(o.z, c1.x - c0.x, c0.x), fmaf(o.z, c1.y - c0.y, c0.y), fmaf(o.z, c1.z - c0.z, c0.z));
}

// advance offsets by v dt/dx, move across cells, wrap periodic axes; returns the new packed
// cell, -1 when the particle leaves the domain, or the packed cell with kHitFlag set (also
// negative, so the particle counts as removed) when it enters an object: k_object_hits then
// applies the reference's object interaction to it, and without one the object absorbs it
__device__ __forceinline__ int move_particle(const PushArgs& a, int i, int j, int k, float3& o, float3 v) {
    const GridDev& g = a.g;
    const float kBelowOne = 0x1.fffffep-1f;
    float ox = o.x + v.x * a.dtdx[0], oy = o.y + v.y * a.dtdx[1], oz = o.z + v.z * a.dtdx[2];
    float fx = floorf(ox), fy = floorf(oy), fz = floorf(oz);
    i += (int)fx;
    j += (int)fy;
    k += (int)fz;
    o.x = fminf(ox - fx, kBelowOne);
    o.y = fminf(oy - fy, kBelowOne);
    o.z = fminf(oz - fz, kBelowOne);
    // periodic wrap: one unsigned compare per axis, the modulo only for a particle outside
    if (g.periodic[0] && (unsigned)i >= (unsigned)g.ci) i = ((i % g.ci) + g.ci) % g.ci;
    if (g.periodic[1] && (unsigned)j >= (unsigned)g.cj) j = ((j % g.cj) + g.cj) % g.cj;
    if (g.periodic[2] && (unsigned)k >= (unsigned)g.ck) k = ((k % g.ck) + g.ck) % g.ck;
    if ((unsigned)i >= (unsigned)g.ci || (unsigned)j >= (unsigned)g.cj || (unsigned)k >= (unsigned)g.ck) return -1;
    if (g.zslab && slab_local_z(g, k) == g.zslab - 1) return -1;  // the cell between two instance slabs
    if (g.n_boxes) {
        float X = ((float)i + o.x) * g.dx[0], Y = ((float)j + o.y) * g.dx[1], Z = ((float)k + o.z) * g.dx[2];
        for (int bx = 0; bx < g.n_boxes; bx++)
            if (X >= g.box_lo[bx][0] && X <= g.box_hi[bx][0] && Y >= g.box_lo[bx][1] && Y <= g.box_hi[bx][1] &&
                Z >= g.box_lo[bx][2] && Z <= g.box_hi[bx][2])
                return pack_cell(i, j, k) | kHitFlag;
    }
    return pack_cell(i, j, k);
}

// round-to-nearest conversion of a non-negative float below 2^64 to a 64-bit integer through two
// 32-bit conversions, bit-identical to __float2ull_rn: hi = floor(x / 2^32) and lo = x - hi 2^32
// are exact in FP32 (lo < 2^32 keeps at most 24 significant bits of x), and x is an integer
// whenever hi > 0.  64-bit conversions are slow on this GPU; 32-bit ones run on the integer and
// conversion units at full rate.
__device__ __forceinline__ unsigned long long f2u64_rn(float x) {
    if (x < 0x1p32f) return __float2uint_rn(x);  // the common case: one 32-bit conversion
    const float hi = floorf(x * 0x1p-32f);
    const float lo = fmaf(hi, -0x1p32f, x);
    return ((unsigned long long)__float2uint_rz(hi) << 32) + __float2uint_rn(lo);
}

// the eight corner contributions of weight w at offsets o as 64-bit fixed point
struct Corners {
    unsigned long long q[8];  // order 000 100 010 110 001 101 011 111 (x fastest)
};
__device__ __forceinline__ void corner_values(float w, float3 o, float scale, Corners& c, bool add) {
    float wx1 = o.x, wx0 = 1.f - o.x, wy1 = o.y, wy0 = 1.f - o.y, wz1 = o.z, wz0 = 1.f - o.z;
    float s = w * scale;
    float s00 = s * wx0 * wy0, s10 = s * wx1 * wy0, s01 = s * wx0 * wy1, s11 = s * wx1 * wy1;
    unsigned long long v[8] = {f2u64_rn(s00 * wz0), f2u64_rn(s10 * wz0), f2u64_rn(s01 * wz0), f2u64_rn(s11 * wz0),
                               f2u64_rn(s00 * wz1), f2u64_rn(s10 * wz1), f2u64_rn(s01 * wz1), f2u64_rn(s11 * wz1)};
#pragma unroll
    for (int c8 = 0; c8 < 8; c8++) c.q[c8] = add ? c.q[c8] + v[c8] : v[c8];
}

// Deposit tile.  Each node slot keeps its 64-bit fixed-point sum as a low and a high 32-bit word
// (native 32-bit shared atomics; 64-bit shared adds are compare-and-swap loops, four times slower
// when measured here).  A value's low word is added with an atomic that returns the old word;
// when the add wraps past 2^32 the carry goes to the high word together with the value's own
// high word.  With the values light (below), the high word is touched only on a wrap, so a
// corner costs one shared atomic.  A slot's sum over a chunk stays below 2^63 (the species'
// fixed-point scale bounds its total weight), so the high word cannot overflow.  The tile is
// committed to HBM with one 64-bit atomic per touched node; integer sums do not depend on the
// order of the additions, so rho is bit-reproducible.
__device__ __forceinline__ void tile_add(unsigned* dt, int x, unsigned long long v) {
    const unsigned lo = (unsigned)v;
    const unsigned old = atomicAdd(&dt[x], lo);
    const unsigned hi = (unsigned)(v >> 32) + (old + lo < lo ? 1u : 0u);
    if (hi) atomicAdd(&dt[4 * kSeg + x], hi);
}
// commits the corner sums of one cell (base node b): into the tile when the cell lies in the
// deposit window, else one 64-bit atomic per corner in HBM
__device__ __forceinline__ void commit_corners(const PushArgs& a, const Tile& t, int b, const Corners& c) {
    int loc = b - (t.lo - kMargin);
    if (t.dtile && loc >= 0 && loc < kSeg - 1) {
#pragma unroll
        for (int c8 = 0; c8 < 8; c8++) tile_add(t.dtile, ((c8 >> 1) * kSeg) + loc + (c8 & 1), c.q[c8]);
    } else {
#pragma unroll
        for (int c8 = 0; c8 < 8; c8++)
            if (c.q[c8]) atomicAdd(&a.sp.acc[b + t.off[c8 >> 1] + (c8 & 1)], c.q[c8]);
    }
}
// A light particle (w * scale below kLightMax, just under 2^30: the species scale puts a particle
// of the mean weight at 2^26 at most) has corner values below 2^30, so the run of a thread's four
// particles sums below 2^32 and the run is kept in 32-bit registers.  The values are the same
// integers as the 64-bit path gives (both round x < 2^32 with one 32-bit conversion).
constexpr float kLightMax = 1.07e9f;
struct Corners32 {
    unsigned q[8];
};
__device__ __forceinline__ void corner_values32(float s, float3 o, Corners32& c, bool add) {
    float wx1 = o.x, wx0 = 1.f - o.x, wy1 = o.y, wy0 = 1.f - o.y, wz1 = o.z, wz0 = 1.f - o.z;
    float s00 = s * wx0 * wy0, s10 = s * wx1 * wy0, s01 = s * wx0 * wy1, s11 = s * wx1 * wy1;
    const unsigned v[8] = {__float2uint_rn(s00 * wz0), __float2uint_rn(s10 * wz0), __float2uint_rn(s01 * wz0),
                           __float2uint_rn(s11 * wz0), __float2uint_rn(s00 * wz1), __float2uint_rn(s10 * wz1),
                           __float2uint_rn(s01 * wz1), __float2uint_rn(s11 * wz1)};
#pragma unroll
    for (int c8 = 0; c8 < 8; c8++) c.q[c8] = add ? c.q[c8] + v[c8] : v[c8];
}
// commits a light run: the eight adds are issued before any returned word is examined
__device__ __forceinline__ void commit_run32(const PushArgs& a, const Tile& t, int b, const Corners32& c) {
    int loc = b - (t.lo - kMargin);
    if (t.dtile && loc >= 0 && loc < kSeg - 1) {
        unsigned old[8];
#pragma unroll
        for (int c8 = 0; c8 < 8; c8++) old[c8] = atomicAdd(&t.dtile[((c8 >> 1) * kSeg) + loc + (c8 & 1)], c.q[c8]);
#pragma unroll
        for (int c8 = 0; c8 < 8; c8++)
            if (old[c8] + c.q[c8] < c.q[c8]) atomicAdd(&t.dtile[4 * kSeg + ((c8 >> 1) * kSeg) + loc + (c8 & 1)], 1u);
    } else {
#pragma unroll
        for (int c8 = 0; c8 < 8; c8++)
            if (c.q[c8]) atomicAdd(&a.sp.acc[b + t.off[c8 >> 1] + (c8 & 1)], (unsigned long long)c.q[c8]);
    }
}

// append one particle to a species at (committed count + pending slot)
__device__ __forceinline__ bool append_particle(const SpeciesDev& sp, int n_committed, float4 p, float4 v,
                                                unsigned long long id, unsigned* err) {
    int slot = atomicAdd(&sp.counts[1], 1);
    int dst = n_committed + slot;
    if (dst >= sp.capacity) {
        set_error(err, kErrCapacity);
        return false;
    }
    sp.pos[dst] = p;
    sp.vel[dst] = v;
    sp.id[dst] = id;
    return true;
}

// Result of one accepted collision: the electron's new velocity, and for an ionisation the
// ejected electron (velocity, offsets in the parent's cell) and the ion (neutral velocity).
struct Collision {
    int kind;  // 0 none, 1 elastic or failed ionisation, 2 ionisation
    float3 v, pv, nv, po;
};

// MC_MEX_Ionization::collide with IONIZE_1 (Interactions.cpp:885-947), background-gas form.
// Kept out of line: only the rare candidates (probability p_null) reach it.
__device__ __noinline__ Collision collide_candidate(const CollDev& cd, unsigned long long id, float3 v, uint4 r0) {
    Collision out;
    out.kind = 0;
    out.v = v;
    uint4 ctr = make_uint4((unsigned)id, (unsigned)(id >> 32), cd.step, 1u);
    uint4 r1 = philox4x32_10(ctr, cd.key);
    const float kTwoPi = 6.283185307179586f;
    float rr1 = sqrtf(-2.f * logf(u01(r0.y))), rr2 = sqrtf(-2.f * logf(u01(r1.x)));
    float s1, c1, s2, c2;
    sincosf(kTwoPi * u01(r0.z), &s1, &c1);
    sincosf(kTwoPi * u01(r1.y), &s2, &c2);
    float3 nv = make_float3(cd.sig_n * rr1 * c1, cd.sig_n * rr1 * s1, cd.sig_n * rr2 * c2);
    float3 vr = make_float3(nv.x - v.x, nv.y - v.y, nv.z - v.z);
    float v_rel = sqrtf(vr.x * vr.x + vr.y * vr.y + vr.z * vr.z);
    float E_rel = cd.E_precalc_rel_eV * v_rel * v_rel;
    float sig = sigma_coll(cd, E_rel);
    if (!(u01(r0.w) * cd.sigv_max < sig * v_rel)) return out;
    out.kind = 1;
    out.nv = nv;
    Draws dr;
    dr.ctr = ctr;
    dr.ctr.w = 2u;
    dr.key = cd.key;
    dr.buf = philox4x32_10(dr.ctr, cd.key);
    dr.pos = 0;
    float E_rel_J = cd.half_mred * v_rel * v_rel;
    float P_ion = sigma_ion(cd, E_rel_J / 1.602176565e-19f) / sig;
    if (dr.next() <= P_ion) {
        float vmag = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
        float E_inc = vmag * vmag * cd.E_precalc_ele_eV;
        if (E_inc < cd.E_ion_eV) return out;  // Interactions.cpp:901-905: no change
        float E_ej = 10.0f * tanf(dr.next() * atanf((E_inc - cd.E_ion_eV) / (2.f * cd.B_inc)));
        float E_sc = E_inc - cd.E_ion_eV - E_ej;
        if (E_sc < 0.f) E_sc = 0.000001f;
        float inv = 1.f / vmag;
        float3 u = make_float3(v.x * inv, v.y * inv, v.z * inv);
        float a1 = dr.next(), a2 = dr.next();
        out.v = new_vel_electron(cd, E_sc, u, a1, a2);
        float a3 = dr.next(), a4 = dr.next();
        out.pv = new_vel_electron(cd, E_ej, u, a3, a4);
        ctr.w = 4u;
        uint4 r4 = philox4x32_10(ctr, cd.key);
        out.po = make_float3(u01(r1.z), u01(r1.w), u01(r4.x));
        out.kind = 2;
    } else {
        float inv_sum = 1.f / (cd.m_n + cd.m_e);
        float3 cm = make_float3((cd.m_n * nv.x + cd.m_e * v.x) * inv_sum, (cd.m_n * nv.y + cd.m_e * v.y) * inv_sum,
                                (cd.m_n * nv.z + cd.m_e * v.z) * inv_sum);
        float cos_ksi = 2.f * dr.next() - 1.f;
        float sin_ksi = sqrtf(fmaxf(1.f - cos_ksi * cos_ksi, 0.f));
        float se, ce;
        sincosf(2.f * 3.141592653f * dr.next(), &se, &ce);
        float3 vr2 = make_float3(v_rel * cos_ksi, v_rel * sin_ksi * ce, v_rel * sin_ksi * se);
        float f = cd.m_n * inv_sum;
        out.v = make_float3(cm.x - f * vr2.x, cm.y - f * vr2.y, cm.z - f * vr2.z);
    }
    return out;
}

// ------------------------------------------------------------------------------------
// push + deposit (collisions run before it, k_mcc_candidates / k_mcc_collide)
//   A CTA takes chunks of 1024 particles (4 consecutive per thread), software-pipelined: the
//   next chunk's particle arrays are bulk-copied (TMA) into shared memory while the current
//   chunk is processed.  For each chunk the four node rows around the base node of its middle
//   particle, [lo + off_m, lo + off_m + L), are bulk-copied into shared memory; the gather reads
//   them there, and the deposit accumulates into a shared 64-bit fixed-point tile (two 32-bit
//   word planes) committed to HBM with one atomic per touched node.  Particles outside the window
//   use HBM directly.
// ------------------------------------------------------------------------------------
// bulk copy of one full chunk's particle arrays into the staging buffer
__device__ __forceinline__ void issue_chunk(const SpeciesDev& sp, int base, float4* ppos, float4* pvel,
                                            unsigned long long* bar) {
    const unsigned b16 = kChunk * sizeof(float4);
    fence_proxy_async();
    mbar_expect_tx(bar, 2 * b16);
    bulk_g2s(ppos, sp.pos + base, b16, bar);
    bulk_g2s(pvel, sp.vel + base, b16, bar);
}

__global__ void __launch_bounds__(kThreads, kPushBlocksPerSM) k_push(PushArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    float4* ppos = reinterpret_cast<float4*>(smem);
    float4* pvel = ppos + kChunk;
    float4* etile = reinterpret_cast<float4*>(smem + kPbufBytes);
    unsigned* dtile = reinterpret_cast<unsigned*>(etile + 4 * kSeg);
    __shared__ __align__(8) unsigned long long bar_p, bar_e;
    __shared__ int s_fail;

    const GridDev& g = a.g;
    const int tid = threadIdx.x, lane = tid & 31;
    const int n = a.sp.counts[0];
    const int nchunks = (n + kChunk - 1) / kChunk;
    const int nij = g.ni * g.nj;

    if (tid == 0) {
        mbar_init(&bar_p, 1);
        mbar_init(&bar_e, 1);
        fence_mbar_init();
        s_fail = 0;
    }
    __syncthreads();
    unsigned phase_p = 0, phase_e = 0;
    const long long wait_lim = wait_poll_limit(a.wait_polls, kWaitLimit);
    Tile t;
    t.off[0] = 0;
    t.off[1] = g.ni;
    t.off[2] = nij;
    t.off[3] = nij + g.ni;
    // last base node whose eight corners exist: the window must not copy past the node array
    const int max_base = g.nv - 2 - t.off[3];

    int moved = 0;  // particles of this thread that changed cell or left, over all its chunks
    int ch = blockIdx.x;
    bool pending = false;  // a particle bulk copy into the staging buffer is in flight
    if (ch < nchunks && (ch + 1) * kChunk <= n && tid == 0) issue_chunk(a.sp, ch * kChunk, ppos, pvel, &bar_p);
    pending = ch < nchunks && (ch + 1) * kChunk <= n;

    for (; ch < nchunks; ch += gridDim.x) {
        const int base = ch * kChunk;
        const int nin = min(kChunk, n - base);
        // ---- this chunk's particles into registers (staged by TMA, or loaded here for the last,
        // partial chunk)
        if (pending) {
            if (!mbar_wait_bounded(&bar_p, phase_p, wait_lim)) atomicExch(&s_fail, 1);
            phase_p ^= 1u;
            pending = false;
            __syncthreads();
            if (s_fail) {
                if (tid == 0) set_error(a.err, kErrBarrierTimeout);
                mbar_wait_bounded(&bar_p, phase_p ^ 1u);  // the copy in flight, bounded
                return;
            }
        } else {
            for (int x = tid; x < nin; x += kThreads) {
                ppos[x] = a.sp.pos[base + x];
                pvel[x] = a.sp.vel[base + x];
            }
            __syncthreads();
        }
        // A thread owns particles tid*4 .. tid*4+3.  Read in place, the eight threads of a
        // quarter-warp would hit the same banks four times over (64-byte stride); reading them in
        // an order rotated by (lane/2) mod 4 spreads the reads over all 32 banks, and two
        // conditional register rotations restore the order.
        float4 P[kPPT], V[kPPT];
        {
            const int rot = (lane >> 1) & 3;
#pragma unroll
            for (int q = 0; q < kPPT; q++) {
                const int x = tid * kPPT + ((q + rot) & 3);
                P[q] = ppos[x];
                V[q] = pvel[x];
            }
            if (rot & 1) {  // U[k] = T[k - 1]
                const float4 p3 = P[3], v3 = V[3];
                P[3] = P[2], P[2] = P[1], P[1] = P[0], P[0] = p3;
                V[3] = V[2], V[2] = V[1], V[1] = V[0], V[0] = v3;
            }
            if (rot & 2) {  // P[k] = U[k - 2]
                float4 t0 = P[0], t1 = P[1];
                P[0] = P[2], P[1] = P[3], P[2] = t0, P[3] = t1;
                t0 = V[0], t1 = V[1];
                V[0] = V[2], V[1] = V[3], V[2] = t0, V[3] = t1;
            }
        }
        // particles past the end of a partial chunk are marked absent
#pragma unroll
        for (int q = 0; q < kPPT; q++)
            if (tid * kPPT + q >= nin) P[q].w = __int_as_float(-1);
        // ---- window: +-kHalfWin base nodes around the base node of the chunk's middle particle
        int lo = 0, hi = -1;
        {
            const int c = __float_as_int(ppos[nin >> 1].w);
            if (c >= 0) {
                const int anchor = cell_base(g, c);
                lo = max(0, anchor - kHalfWin);
                hi = min(anchor + kHalfWin, max_base);
            }
        }
        const bool use_tile = a.staged && hi >= lo;
        __syncthreads();  // every thread has read the staging buffer
        if (tid == 0) {
            if (use_tile) {
                const unsigned bytes = (unsigned)(hi - lo + 2) * (unsigned)sizeof(float4);
                fence_proxy_async();
                mbar_expect_tx(&bar_e, 4 * bytes);
#pragma unroll
                for (int m = 0; m < 4; m++) bulk_g2s(etile + m * kSeg, a.ef + lo + t.off[m], bytes, &bar_e);
            }
            const int nx = ch + gridDim.x;
            if (nx < nchunks && (nx + 1) * kChunk <= n) issue_chunk(a.sp, nx * kChunk, ppos, pvel, &bar_p);
        }
        {
            const int nx = ch + gridDim.x;
            pending = nx < nchunks && (nx + 1) * kChunk <= n;
        }
        t.lo = lo;
        t.span = hi - lo;
        t.etile = nullptr;
        t.dtile = nullptr;
        if (use_tile) {
            if (a.deposit)
                for (int x = tid; x < 8 * kSeg; x += kThreads) dtile[x] = 0u;
            if (!mbar_wait_bounded(&bar_e, phase_e, wait_lim)) atomicExch(&s_fail, 1);
            phase_e ^= 1u;
            __syncthreads();
            if (s_fail) {
                // a copy did not complete in time: record it, wait once more (bounded) for the
                // copies in flight, and leave without touching the tile
                if (tid == 0) set_error(a.err, kErrBarrierTimeout);
                mbar_wait_bounded(&bar_e, phase_e ^ 1u);
                if (pending) mbar_wait_bounded(&bar_p, phase_p);
                return;
            }
            t.etile = etile;
            if (a.deposit) t.dtile = dtile;
        }

        unsigned dead_mask[kPPT];
        Corners32 run;      // deposit sums of the current run of light particles
        int run_cell = -1;  // packed cell of the run, -1: none
#pragma unroll
        for (int q = 0; q < kPPT; q++) {
            const int p = base + tid * kPPT + q;
            dead_mask[q] = 0;
            int c = __float_as_int(P[q].w);
            if (c < 0) continue;
            int i, j, k;
            cell_ijk(g, c, i, j, k);
            float3 o = make_float3(P[q].x, P[q].y, P[q].z);
            float3 v = make_float3(V[q].x, V[q].y, V[q].z);
            const float w = V[q].w;
            // leapfrog push (Species.cpp:369-373)
            float3 E = gather_e(a, t, cell_base(g, c), o);
            v.x += a.qm_dt * E.x;
            v.y += a.qm_dt * E.y;
            v.z += a.qm_dt * E.z;
            const int newc = move_particle(a, i, j, k, o, v);
            moved += newc != c;
            a.sp.pos[p] = make_float4(o.x, o.y, o.z, __int_as_float(newc));
            a.sp.vel[p] = make_float4(v.x, v.y, v.z, w);
            if (newc >= 0) {
                if (a.deposit) {
                    const float s = w * a.dep_scale;
                    if (s < kLightMax) {
                        if (newc != run_cell && run_cell >= 0)
                            commit_run32(a, t, cell_base(g, run_cell), run);
                        corner_values32(s, o, run, newc == run_cell);
                        run_cell = newc;
                    } else {
                        Corners hc;
                        corner_values(w, o, a.dep_scale, hc, false);
                        commit_corners(a, t, cell_base(g, newc), hc);
                    }
                }
            } else {
                dead_mask[q] = 1;
            }
        }
        if (run_cell >= 0)
            commit_run32(a, t, cell_base(g, run_cell), run);
        // warp-aggregated record of the particles that left the domain
#pragma unroll
        for (int q = 0; q < kPPT; q++) {
            unsigned dm = __ballot_sync(0xffffffffu, dead_mask[q] != 0);
            if (dm) {
                int b0 = 0;
                if (lane == __ffs(dm) - 1) b0 = atomicAdd(&a.sp.counts[2], __popc(dm));
                b0 = __shfl_sync(0xffffffffu, b0, __ffs(dm) - 1);
                if (dead_mask[q]) a.sp.dead[b0 + __popc(dm & ((1u << lane) - 1u))] = base + tid * kPPT + q;
            }
        }
        __syncthreads();
        if (use_tile && a.deposit) {
            // commit the tile: slot o of row m is node lo - kMargin + off_m + o (only slots that
            // received a deposit are nonzero, and those are nodes of the grid)
            const int wlo = lo - kMargin;
            for (int x = tid; x < 4 * kSeg; x += kThreads) {
                unsigned long long v = (unsigned long long)dtile[x] + ((unsigned long long)dtile[4 * kSeg + x] << 32);
                if (v) atomicAdd(&a.sp.acc[wlo + t.off[x / kSeg] + (x % kSeg)], v);
            }
        }
        __syncthreads();
    }
    // cell-order bookkeeping for the sort policy: one global atomic per CTA (a per-warp atomic on
    // one address serialises hundreds of thousands of updates per launch)
    __shared__ int s_moved;
    if (tid == 0) s_moved = 0;
    __syncthreads();
    const int wm = __reduce_add_sync(0xffffffffu, moved);
    if (lane == 0 && wm) atomicAdd(&s_moved, wm);
    __syncthreads();
    if (tid == 0 && s_moved) atomicAdd(&a.sp.counts[5], s_moved);
}

// ------------------------------------------------------------------------------------
// collisions as separate passes ahead of a collision-free push:
//   candidates: cand_draw(id) < 2^32 P_null per electron, a list of candidates (with instance
//               slabs the list holds the draws below the largest slab threshold; the collide pass
//               applies the particle's own slab threshold)
//   collide   : the collisions of the candidates (Philox draws keyed by (seed, step, id)); the
//               ejected electron is pushed and deposited there, the ion product appended
// The split keeps the push kernel free of the collision registers and code, and the candidate
// pass reads only the ids.
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_mcc_candidates(PushArgs a, int* cand, int* ncand) {
    const CollDev& cd = a.coll;
    const int n = a.sp.counts[0];
    const int lane = threadIdx.x & 31;
    const int ng = (n + 3) >> 2;  // four consecutive ids per thread, two 16-byte loads
    for (int base = blockIdx.x * blockDim.x; base < ng; base += gridDim.x * blockDim.x) {
        const int gq = base + threadIdx.x;
        const int p0 = gq << 2;
        unsigned long long id[4] = {0ull, 0ull, 0ull, 0ull};
        if (p0 + 4 <= n) {
            const ulonglong2 x = reinterpret_cast<const ulonglong2*>(a.sp.id)[2 * gq];
            const ulonglong2 y = reinterpret_cast<const ulonglong2*>(a.sp.id)[2 * gq + 1];
            id[0] = x.x, id[1] = x.y, id[2] = y.x, id[3] = y.y;
        } else {
#pragma unroll
            for (int q = 0; q < 4; q++)
                if (p0 + q < n) id[q] = a.sp.id[p0 + q];
        }
#pragma unroll
        for (int q = 0; q < 4; q++) {
            const bool is_cand = p0 + q < n && cand_draw(id[q], cd.step, cd.key) < cd.cand_max;
            const unsigned m = __ballot_sync(0xffffffffu, is_cand);
            if (m) {
                int b0 = 0;
                if (lane == __ffs(m) - 1) b0 = atomicAdd(ncand, __popc(m));
                b0 = __shfl_sync(0xffffffffu, b0, __ffs(m) - 1);
                if (is_cand) cand[b0 + __popc(m & ((1u << lane) - 1u))] = p0 + q;
            }
        }
    }
}

__global__ void __launch_bounds__(128) k_mcc_collide(PushArgs a, const int* cand, const int* ncand) {
    const CollDev& cd = a.coll;
    const GridDev& g = a.g;
    const int n = a.sp.counts[0];
    const int ion_n = cd.ion.counts[0];
    const int nc = *ncand;
    unsigned st_cand = 0, st_coll = 0, st_ion = 0, st_lost = 0;
    Tile t;  // no staged rows: gathers and deposits go to HBM
    t.etile = nullptr;
    t.dtile = nullptr;
    t.lo = 0;
    t.span = -1;
    t.off[0] = 0;
    t.off[1] = g.ni;
    t.off[2] = g.ni * g.nj;
    t.off[3] = g.ni * g.nj + g.ni;
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nc; q += gridDim.x * blockDim.x) {
        const int p = cand[q];
        const float4 P = a.sp.pos[p];
        const float4 V = a.sp.vel[p];
        const int c = __float_as_int(P.w);
        if (c < 0) continue;
        const unsigned long long id = a.sp.id[p];
        if (cd.cand_slab && cand_draw(id, cd.step, cd.key) >= __ldg(&cd.cand_slab[fdiv((unsigned)(c >> 18), g.fd_zslab)]))
            continue;  // below the largest slab threshold, not below its own
        st_cand++;
        int i, j, k;
        cell_ijk(g, c, i, j, k);
        const uint4 r0 = philox4x32_10(make_uint4((unsigned)id, (unsigned)(id >> 32), cd.step, 0u), cd.key);
        const float w = V.w;
        Collision col = collide_candidate(cd, id, make_float3(V.x, V.y, V.z), r0);
        if (!col.kind) continue;
        st_coll++;
        a.sp.vel[p] = make_float4(col.v.x, col.v.y, col.v.z, w);
        if (col.kind != 2) continue;
        st_ion++;
        // the ejected electron and the ion are created at a uniform point of the parent's cell
        // without velocity rewind; the electron is pushed and deposited now
        if (!append_particle(cd.ion, ion_n, make_float4(col.po.x, col.po.y, col.po.z, __int_as_float(c)),
                             make_float4(col.nv.x, col.nv.y, col.nv.z, w), child_id(id, cd.step, 2), a.err))
            st_lost++;
        float3 po = col.po, pv = col.pv;
        const float3 Ep = gather_e(a, t, cell_base(g, c), po);
        pv.x += a.qm_dt * Ep.x;
        pv.y += a.qm_dt * Ep.y;
        pv.z += a.qm_dt * Ep.z;
        const int pc = move_particle(a, i, j, k, po, pv);
        if (pc < 0) continue;
        if (append_particle(a.sp, n, make_float4(po.x, po.y, po.z, __int_as_float(pc)),
                            make_float4(pv.x, pv.y, pv.z, w), child_id(id, cd.step, 1), a.err)) {
            if (a.deposit) {
                Corners pcn;
                corner_values(w, po, a.dep_scale, pcn, false);
                commit_corners(a, t, cell_base(g, pc), pcn);
            }
        } else {
            st_lost++;
        }
    }
    const unsigned v[4] = {st_cand, st_coll, st_ion, st_lost};
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int x = 0; x < 4; x++) {
        const unsigned s = __reduce_add_sync(0xffffffffu, v[x]);
        if (lane == 0 && s) atomicAdd(&cd.stats[x], (unsigned long long)s);
    }
}

void launch_mcc(const PushArgs& a, int* cand, int* ncand, cudaStream_t s, int sms) {
    cudaMemsetAsync(ncand, 0, sizeof(int), s);
    k_mcc_candidates<<<sms * 8, 256, 0, s>>>(a, cand, ncand);
    k_mcc_collide<<<sms * 4, 128, 0, s>>>(a, cand, ncand);
}

int push_blocks_per_sm() {
    static int nb = 0;
    if (!nb) {
        cudaFuncSetAttribute(k_push, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPushSmem);
        cudaFuncSetAttribute(k_push, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_push, kThreads, kPushSmem) != cudaSuccess || nb < 1)
            nb = 1;
    }
    return nb;
}
void launch_push(const PushArgs& a, cudaStream_t s, int grid) {
    push_blocks_per_sm();
    k_push<<<grid, kThreads, kPushSmem, s>>>(a);
}

// ------------------------------------------------------------------------------------
// appends and compaction
// ------------------------------------------------------------------------------------
__global__ void k_commit_appends(SpeciesDev sp, unsigned* err) {
    int n = sp.counts[0], pend = sp.counts[1];
    int nn = n + pend;
    if (nn > sp.capacity) {
        nn = sp.capacity;
        set_error(err, kErrCapacity);
    }
    sp.counts[0] = nn;
    sp.counts[1] = 0;
    sp.counts[5] += nn - n;  // appended particles are out of cell order
}
void launch_commit_appends(SpeciesDev sp, unsigned* err, cudaStream_t s) { k_commit_appends<<<1, 1, 0, s>>>(sp, err); }

// dead particles below the new end become holes
__global__ void k_compact_holes(SpeciesDev sp) {
    int n = sp.counts[0], nd = sp.counts[2], nnew = n - nd;
    for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < nd; d += gridDim.x * blockDim.x) {
        int idx = sp.dead[d];
        if (idx < nnew) sp.holes[atomicAdd(&sp.counts[3], 1)] = idx;
    }
}
// live particles above the new end fill the holes
__global__ void k_compact_move(SpeciesDev sp) {
    int n = sp.counts[0], nd = sp.counts[2], nnew = n - nd;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nd; t += gridDim.x * blockDim.x) {
        int idx = nnew + t;
        float4 p = sp.pos[idx];
        if (__float_as_int(p.w) < 0) continue;
        int h = sp.holes[atomicAdd(&sp.counts[4], 1)];
        sp.pos[h] = p;
        sp.vel[h] = sp.vel[idx];
        sp.id[h] = sp.id[idx];
    }
}
__global__ void k_compact_finish(SpeciesDev sp) {
    sp.counts[0] -= sp.counts[2];
    sp.counts[2] = 0;
    sp.counts[3] = 0;
    sp.counts[4] = 0;
}
void launch_compact(SpeciesDev sp, cudaStream_t s, int grid) {
    k_compact_holes<<<grid, 256, 0, s>>>(sp);
    k_compact_move<<<grid, 256, 0, s>>>(sp);
    k_compact_finish<<<1, 1, 0, s>>>(sp);
}

// ------------------------------------------------------------------------------------
// counting sort by cell (Species::sortIndexes keeps index lists; here the particles
// themselves are reordered so that each cell is a contiguous run)
// ------------------------------------------------------------------------------------
__global__ void k_sort_hist(GridDev g, SpeciesDev sp, int* cnt) {
    int n = sp.counts[0];
    int stride = gridDim.x * blockDim.x;
    int lim = ((n + 31) / 32) * 32;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < lim; p += stride) {
        int c = p < n ? __float_as_int(sp.pos[p].w) : -1;
        unsigned m = __match_any_sync(0xffffffffu, c);
        if (c >= 0 && (threadIdx.x & 31) == __ffs(m) - 1) atomicAdd(&cnt[cell_linear(g, c)], __popc(m));
    }
}
// exclusive scan in three passes over tiles of 2048 counts
constexpr int kScanTile = 2048;
__global__ void k_scan_tiles(const int* in, int* out, int* aux, int n) {
    __shared__ int s[kScanTile];
    __shared__ int wsum[8];
    int tile = blockIdx.x, t = threadIdx.x;  // 256 threads, 8 values each
    int base = tile * kScanTile;
    for (int x = t; x < kScanTile; x += 256) s[x] = base + x < n ? in[base + x] : 0;
    __syncthreads();
    int v[8], run = 0;
    for (int q = 0; q < 8; q++) {
        v[q] = run;
        run += s[t * 8 + q];
    }
    // inclusive scan of per-thread totals
    int lane = t & 31, w = t >> 5, x = run;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    int woff = 0;
    for (int q = 0; q < w; q++) woff += wsum[q];
    int excl = woff + x - run;
    for (int q = 0; q < 8; q++)
        if (base + t * 8 + q < n) out[base + t * 8 + q] = excl + v[q];
    if (t == 255) aux[tile] = woff + x;
}
__global__ void k_scan_aux(int* aux, int ntiles) {
    // single block of 1024 threads, sequential chunks
    __shared__ int carry;
    __shared__ int wsum[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b0 = 0; b0 < ntiles; b0 += 1024) {
        int idx = b0 + threadIdx.x;
        int val = idx < ntiles ? aux[idx] : 0;
        int lane = threadIdx.x & 31, w = threadIdx.x >> 5, x = val;
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wsum[w] = x;
        __syncthreads();
        int woff = 0;
        for (int q = 0; q < w; q++) woff += wsum[q];
        int c0 = carry;
        if (idx < ntiles) aux[idx] = c0 + woff + x - val;
        __syncthreads();
        if (threadIdx.x == 1023) carry = c0 + woff + x;
        __syncthreads();
    }
}
__global__ void k_scan_add(int* out, const int* aux, int n) {
    int base = blockIdx.x * kScanTile;
    int add = aux[blockIdx.x];
    for (int x = threadIdx.x; x < kScanTile; x += 256)
        if (base + x < n) out[base + x] += add;
}
__global__ void k_sort_scatter(GridDev g, SpeciesDev sp, const int* start, int* cursor, float4* pos2,
                               float4* vel2, unsigned long long* id2) {
    int n = sp.counts[0];
    int stride = gridDim.x * blockDim.x;
    int lim = ((n + 31) / 32) * 32;
    int lane = threadIdx.x & 31;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < lim; p += stride) {
        float4 ps = p < n ? sp.pos[p] : make_float4(0, 0, 0, __int_as_float(-1));
        int c = __float_as_int(ps.w);
        unsigned m = __match_any_sync(0xffffffffu, c);
        int leader = __ffs(m) - 1;
        int lc = c >= 0 ? cell_linear(g, c) : 0;
        int b = 0;
        if (c >= 0 && lane == leader) b = atomicAdd(&cursor[lc], __popc(m));
        b = __shfl_sync(m, b, leader);
        if (c >= 0) {
            int dst = start[lc] + b + __popc(m & ((1u << lane) - 1u));
            pos2[dst] = ps;
            vel2[dst] = sp.vel[p];
            id2[dst] = sp.id[p];
        }
    }
}
void launch_sort(const GridDev& g, SpeciesDev sp, float4* pos_alt, float4* vel_alt, unsigned long long* id_alt,
                 int* cell_count, int* cell_start, int* scan_aux, cudaStream_t s, int grid) {
    int nc = g.nc;
    cudaMemsetAsync(cell_count, 0, sizeof(int) * nc, s);
    k_sort_hist<<<grid, 256, 0, s>>>(g, sp, cell_count);
    int ntiles = (nc + kScanTile - 1) / kScanTile;
    k_scan_tiles<<<ntiles, 256, 0, s>>>(cell_count, cell_start, scan_aux, nc);
    k_scan_aux<<<1, 1024, 0, s>>>(scan_aux, ntiles);
    k_scan_add<<<ntiles, 256, 0, s>>>(cell_start, scan_aux, nc);
    cudaMemsetAsync(cell_count, 0, sizeof(int) * nc, s);
    k_sort_scatter<<<grid, 256, 0, s>>>(g, sp, cell_start, cell_count, pos_alt, vel_alt, id_alt);
}

// ------------------------------------------------------------------------------------
// host <-> device conversion (Species::addParticle semantics when rewind is set)
// ------------------------------------------------------------------------------------
// id == nullptr: particle p gets id id0 + p
// one particle of an upload: Species::addParticle semantics when rewind is set
__device__ __forceinline__ void from_abs_one(const GridDev& g, const SpeciesDev& sp, int n0, int p, const double* xp,
                                             const double* vp, const double* w, const unsigned long long* id,
                                             unsigned long long id0, int rewind, float qm_half_dt, const float4* ef) {
    int dst = n0 + p;
    if (dst >= sp.capacity) return;
    double x[3] = {xp[0], xp[1], xp[2]};
    float3 v = make_float3((float)vp[0], (float)vp[1], (float)vp[2]);
    bool ok = !(isnan(x[0]) || isnan(x[1]) || isnan(x[2]) || isnan(v.x) || isnan(v.y) || isnan(v.z));
    int ijk[3];
    float o[3];
    int nc3[3] = {g.ci, g.cj, g.ck};
    for (int d = 0; d < 3 && ok; d++) {
        if (g.periodic[d]) {
            double L = g.xm[d] - g.x0[d];
            if (x[d] < g.x0[d]) x[d] += L;
            else if (x[d] >= g.xm[d]) x[d] -= L;
        }
        if (x[d] < g.x0[d] || x[d] >= g.xm[d]) ok = false;
        double lc = (x[d] - g.x0[d]) / g.dxd[d];
        int c = (int)lc;
        if (c >= nc3[d]) c = nc3[d] - 1;
        double f = lc - c;
        ijk[d] = c;
        o[d] = fminf((float)f, 0x1.fffffep-1f);
    }
    int cell = -1;
    if (ok) {
        cell = pack_cell(ijk[0], ijk[1], ijk[2]);
        if (g.n_boxes) {
            float X = ((float)ijk[0] + o[0]) * g.dx[0], Y = ((float)ijk[1] + o[1]) * g.dx[1],
                  Z = ((float)ijk[2] + o[2]) * g.dx[2];
            for (int b = 0; b < g.n_boxes; b++)
                if (X >= g.box_lo[b][0] && X <= g.box_hi[b][0] && Y >= g.box_lo[b][1] && Y <= g.box_hi[b][1] &&
                    Z >= g.box_lo[b][2] && Z <= g.box_hi[b][2])
                    cell = -1;
        }
    }
    if (cell >= 0 && rewind && ef) {
        // vel -= q/m E dt/2 (Species.cpp:431)
        PushArgs dummy;
        dummy.ef = ef;
        Tile t;
        t.etile = nullptr;
        t.dtile = nullptr;
        t.lo = 0;
        t.span = -1;
        t.off[0] = 0;
        t.off[1] = g.ni;
        t.off[2] = g.ni * g.nj;
        t.off[3] = g.ni * g.nj + g.ni;
        float3 E = gather_e(dummy, t, cell_base_node(g, ijk[0], ijk[1], ijk[2]), make_float3(o[0], o[1], o[2]));
        v.x -= qm_half_dt * E.x;
        v.y -= qm_half_dt * E.y;
        v.z -= qm_half_dt * E.z;
    }
    sp.pos[dst] = make_float4(o[0], o[1], o[2], __int_as_float(cell));
    sp.vel[dst] = make_float4(v.x, v.y, v.z, (float)w[p]);
    sp.id[dst] = id ? id[p] : id0 + (unsigned long long)p;
    if (cell < 0) sp.dead[atomicAdd(&sp.counts[2], 1)] = dst;
}
// Block-cooperative: a block stages the FP64 positions and velocities of its 256 particles in
// shared memory with contiguous reads (each source sector is read once, which matters when the
// arrays are pinned host memory read over the host link), then converts one particle per thread.
__global__ void __launch_bounds__(256) k_from_abs(GridDev g, SpeciesDev sp, const double* pos, const double* vel,
                                                  const double* w, const unsigned long long* id,
                                                  unsigned long long id0, int n, int rewind, float qm_half_dt,
                                                  const float4* ef) {
    __shared__ double s_pos[3 * 256], s_vel[3 * 256];
    const int n0 = sp.counts[0];
    for (long long base = (long long)blockIdx.x * 256; base < n; base += (long long)gridDim.x * 256) {
        const int m = (int)min(256ll, n - base);
        for (int e = threadIdx.x; e < 3 * m; e += 256) {
            s_pos[e] = pos[3 * base + e];
            s_vel[e] = vel[3 * base + e];
        }
        __syncthreads();
        if ((int)threadIdx.x < m)
            from_abs_one(g, sp, n0, (int)base + (int)threadIdx.x, s_pos + 3 * threadIdx.x, s_vel + 3 * threadIdx.x, w,
                         id, id0, rewind, qm_half_dt, ef);
        __syncthreads();
    }
}
__global__ void k_from_abs_count(SpeciesDev sp, int n, unsigned* err) {
    int nn = sp.counts[0] + n;
    if (nn > sp.capacity) {
        nn = sp.capacity;
        set_error(err, kErrCapacity);
    }
    sp.counts[0] = nn;
}
void launch_from_abs(const GridDev& g, SpeciesDev sp, const double* pos, const double* vel, const double* w,
                     const unsigned long long* id, unsigned long long id0, int n, int rewind, float qm_half_dt,
                     const float4* ef, cudaStream_t s, int max_grid) {
    int grid = (n + 255) / 256;
    if (grid > max_grid) grid = max_grid;
    if (grid < 1) grid = 1;
    k_from_abs<<<grid, 256, 0, s>>>(g, sp, pos, vel, w, id, id0, n, rewind, qm_half_dt, ef);
    k_from_abs_count<<<1, 1, 0, s>>>(sp, n, nullptr);
    launch_compact(sp, s, 256);
}

// export of particles first, first + stride, ... (n of them) to absolute FP64 positions
__global__ void k_to_abs(GridDev g, SpeciesDev sp, double* pos, double* vel, double* w, unsigned long long* id,
                         int n, long long first, long long stride) {
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const long long q = first + (long long)p * stride;
        float4 ps = sp.pos[q], vs = sp.vel[q];
        int i, j, k;
        cell_ijk(g, __float_as_int(ps.w), i, j, k);
        if (pos) {
            pos[3 * p] = g.x0[0] + ((double)i + (double)ps.x) * g.dxd[0];
            pos[3 * p + 1] = g.x0[1] + ((double)j + (double)ps.y) * g.dxd[1];
            pos[3 * p + 2] = g.x0[2] + ((double)k + (double)ps.z) * g.dxd[2];
        }
        if (vel) {
            vel[3 * p] = vs.x;
            vel[3 * p + 1] = vs.y;
            vel[3 * p + 2] = vs.z;
        }
        if (w) w[p] = vs.w;
        if (id) id[p] = sp.id[q];
    }
}
void launch_to_abs(const GridDev& g, SpeciesDev sp, double* pos, double* vel, double* w, unsigned long long* id,
                   int n, cudaStream_t s, long long first, long long stride) {
    int grid = (n + 255) / 256;
    if (grid > 4096) grid = 4096;
    if (grid < 1) grid = 1;
    k_to_abs<<<grid, 256, 0, s>>>(g, sp, pos, vel, w, id, n, first, stride);
}

// ------------------------------------------------------------------------------------
// synthetic loader: uniform box, Maxwellian velocities, lognormal weights (Philox)
// ------------------------------------------------------------------------------------
__global__ void k_load_uniform(GridDev g, SpeciesDev sp, LoadArgs la) {
    int n0 = sp.counts[0];
    const float kTwoPi = 6.283185307179586f;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < la.n; p += gridDim.x * blockDim.x) {
        int dst = n0 + p;
        if (dst >= sp.capacity) continue;
        unsigned long long id = la.id0 + (unsigned long long)p;
        uint4 r0 = philox4x32_10(make_uint4((unsigned)id, (unsigned)(id >> 32), 0xA5A5A5A5u, 0u), la.key);
        uint4 r1 = philox4x32_10(make_uint4((unsigned)id, (unsigned)(id >> 32), 0xA5A5A5A5u, 1u), la.key);
        double x[3] = {la.lo[0] + (la.hi[0] - la.lo[0]) * (double)u01(r0.x),
                       la.lo[1] + (la.hi[1] - la.lo[1]) * (double)u01(r0.y),
                       la.lo[2] + (la.hi[2] - la.lo[2]) * (double)u01(r0.z)};
        int ijk[3];
        float o[3];
        int nc3[3] = {g.ci, g.cj, g.ck};
        for (int d = 0; d < 3; d++) {
            double lc = (x[d] - g.x0[d]) / g.dxd[d];
            int c = (int)lc;
            c = c < 0 ? 0 : (c >= nc3[d] ? nc3[d] - 1 : c);
            ijk[d] = c;
            o[d] = fminf(fmaxf((float)(lc - c), 0.f), 0x1.fffffep-1f);
        }
        float s1, c1, s2, c2;
        float ra = sqrtf(-2.f * logf(u01(r0.w))), rb = sqrtf(-2.f * logf(u01(r1.y)));
        sincosf(kTwoPi * u01(r1.x), &s1, &c1);
        sincosf(kTwoPi * u01(r1.z), &s2, &c2);
        float3 v = make_float3(la.vth * ra * c1, la.vth * ra * s1, la.vth * rb * c2);
        if (la.ref_thermal) {
            // Species::sampleVth: speed = |v_th (u1+u2+u3-1.5) per axis|; sampleV3th: isotropic
            // direction from theta = 2 pi u, r = 2u - 1 (Species.cpp:855-869)
            uint4 r2 = philox4x32_10(make_uint4((unsigned)id, (unsigned)(id >> 32), 0xA5A5A5A5u, 2u), la.key);
            uint4 r3 = philox4x32_10(make_uint4((unsigned)id, (unsigned)(id >> 32), 0xA5A5A5A5u, 3u), la.key);
            float v1 = la.vth * (u01(r1.x) + u01(r1.y) + u01(r1.z) - 1.5f);
            float v2 = la.vth * (u01(r1.w) + u01(r2.x) + u01(r2.y) - 1.5f);
            float v3 = la.vth * (u01(r2.z) + u01(r2.w) + u01(r3.x) - 1.5f);
            float sp_ = sqrtf(v1 * v1 + v2 * v2 + v3 * v3);
            float st, ct;
            sincosf(2.f * 3.141592653f * u01(r3.y), &st, &ct);
            float rr = -1.f + 2.f * u01(r3.z), aa = sqrtf(fmaxf(1.f - rr * rr, 0.f));
            v = make_float3(sp_ * rr, sp_ * (ct * aa), sp_ * (st * aa));
        }
        float wgt = la.w_mean;
        if (la.w_sigma > 0.f) {
            // lognormal with mean w_mean: mu = ln(w_mean) - sigma^2/2; the normal is rb*s2
            float zn = rb * s2;
            wgt = expf(logf(la.w_mean) - 0.5f * la.w_sigma * la.w_sigma + la.w_sigma * zn);
        }
        int cell = pack_cell(ijk[0], ijk[1], ijk[2]);
        sp.pos[dst] = make_float4(o[0], o[1], o[2], __int_as_float(cell));
        sp.vel[dst] = make_float4(v.x, v.y, v.z, wgt);
        sp.id[dst] = id;
    }
}
// Beam source particles.  Particle p of a step draws Philox blocks (p, step, 0x5C000000 + src, b):
//   b = 0: in-face coordinates a, b (u01 of words x, y); speed draws t0, t1 (z, w)
//   b = 1: t2 .. t5;  b = 2: t6, t7, t8, theta;  b = 3: r (word x)
// Position: the face plane (the + faces one cell in, as Source.cpp offsets L by -dx), the two
// other coordinates uniform over the face.  Velocity: drift along the inward normal, plus for a
// warm beam Species::sampleV3th (speed from three per-axis sums of three uniforms, isotropic
// direction from theta = 2 pi u and r = 2u - 1), in FP64.
__global__ void k_source(SourceArgs sa, double* pos, double* vel, double* w) {
    const double kTwoPi = 6.283185307179586;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < sa.n; p += gridDim.x * blockDim.x) {
        const unsigned tag = 0x5C000000u + sa.src;
        const unsigned pp = (unsigned)(sa.first + p);
        const uint4 r0 = philox4x32_10(make_uint4(pp, sa.step, tag, 0u), sa.key);
        const int ax = sa.face >> 1;  // normal axis
        const int e1 = ax == 0 ? 1 : 0, e2 = ax == 2 ? 1 : 2;
        double x[3];
        x[ax] = sa.x0[ax] + ((sa.face & 1) ? sa.L[ax] : 0.0);
        x[e1] = sa.x0[e1] + (double)u01(r0.x) * sa.L[e1];
        x[e2] = sa.x0[e2] + (double)u01(r0.y) * sa.L[e2];
        double v[3] = {0.0, 0.0, 0.0};
        if (sa.vth > 0.0) {
            const uint4 r1 = philox4x32_10(make_uint4(pp, sa.step, tag, 1u), sa.key);
            const uint4 r2 = philox4x32_10(make_uint4(pp, sa.step, tag, 2u), sa.key);
            const uint4 r3 = philox4x32_10(make_uint4(pp, sa.step, tag, 3u), sa.key);
            const double v1 = sa.vth * ((double)u01(r0.z) + (double)u01(r0.w) + (double)u01(r1.x) - 1.5);
            const double v2 = sa.vth * ((double)u01(r1.y) + (double)u01(r1.z) + (double)u01(r1.w) - 1.5);
            const double v3 = sa.vth * ((double)u01(r2.x) + (double)u01(r2.y) + (double)u01(r2.z) - 1.5);
            const double sp_ = sqrt(v1 * v1 + v2 * v2 + v3 * v3);
            const double th = kTwoPi * (double)u01(r2.w);
            const double r = -1.0 + 2.0 * (double)u01(r3.x), aa = sqrt(fmax(1.0 - r * r, 0.0));
            v[0] = sp_ * r;
            v[1] = sp_ * (cos(th) * aa);
            v[2] = sp_ * (sin(th) * aa);
        }
        v[ax] += (sa.face & 1) ? -sa.v_drift : sa.v_drift;
        for (int d = 0; d < 3; d++) {
            pos[3 * p + d] = x[d];
            vel[3 * p + d] = v[d];
        }
        w[p] = sa.mpw0;
    }
}
void launch_source(const SourceArgs& sa, double* pos, double* vel, double* w, cudaStream_t s) {
    int grid = (sa.n + 255) / 256;
    if (grid > 1024) grid = 1024;
    if (grid < 1) grid = 1;
    k_source<<<grid, 256, 0, s>>>(sa, pos, vel, w);
}

// ------------------------------------------------------------------------------------
// Object interaction (Species.cpp:79-256, Object.cpp:231-275, Species.cpp:835-861), FP64.
// A particle's draws come from one Philox-4x32-10 stream keyed by (id, step, 0x0B000000 + block),
// taken in the order of the reference's rnd() calls.
// ------------------------------------------------------------------------------------
namespace {
constexpr double kKbRef = 1.380648e-23;  // Const::k, ch4/v3/src/all.h:19
constexpr double kPiRef = 3.141592653;   // Const::pi, ch4/v3/src/all.h:20
struct DrawStream {
    uint4 ctr;
    uint2 key;
    uint4 buf;
    int pos;
    __device__ DrawStream(unsigned long long id, unsigned step, uint2 k)
        : ctr(make_uint4((unsigned)id, (unsigned)(id >> 32), step, 0x0B000000u)), key(k), pos(4) {}
    __device__ double next() {
        if (pos == 4) {
            buf = philox4x32_10(ctr, key);
            ctr.w++;
            pos = 0;
        }
        const unsigned x = pos == 0 ? buf.x : pos == 1 ? buf.y : pos == 2 ? buf.z : buf.w;
        pos++;
        return (double)u01(x);
    }
};
// World::inObject over Rectangle::inObject (World.cpp:293-301, Object.cpp:231-238): object index + 1
__device__ int in_object_d(const ObjArgs& o, const double x[3]) {
    for (int b = 0; b < o.n_boxes; b++) {
        bool in = true;
        for (int d = 0; d < 3; d++)
            if (fabs(x[d] - o.box_c[b][d]) > o.box_half[b][d]) in = false;
        if (in) return b + 1;
    }
    return 0;
}
__device__ void add_side_normal(int side, double n[3]) {  // Rectangle::find_n (Object.cpp:277-302)
    n[side % 3] += side < 3 ? -1.0 : 1.0;
}
// Rectangle::lineIntersect (Object.cpp:239-275): entry time along x1 -> x2, entry point, normal
__device__ void line_intersect_d(const ObjArgs& o, int b, const double x1[3], const double x2[3], double& t_entry,
                                 double xi[3], double n[3]) {
    double tmin[3], tmax[3];
    int ps[3] = {0, 1, 2};
    for (int d = 0; d < 3; d++) {
        const double A = x2[d] - x1[d];
        tmin[d] = (o.box_c[b][d] - o.box_half[b][d] - x1[d]) / A;
        tmax[d] = (o.box_c[b][d] + o.box_half[b][d] - x1[d]) / A;
        if (tmin[d] > tmax[d]) {
            const double t = tmin[d];
            tmin[d] = tmax[d];
            tmax[d] = t;
            ps[d] += 3;
        }
    }
    t_entry = tmin[0];
    int j = 0, k = 0, t = 0;
    for (int i = 0; i < 2; i++) {
        if (t_entry < tmin[i + 1]) {
            t_entry = tmin[i + 1];
            j = i + 1;
            k = 0;
        } else if (fabs(t_entry - tmin[i + 1]) < 1e-6) {
            k++;
            t = i + 1;
        }
    }
    n[0] = n[1] = n[2] = 0.0;
    add_side_normal(ps[j], n);
    if (k != 0) {  // an edge or a vertex: the sum of the faces' normals, normalised
        if (k < 2) {
            add_side_normal(ps[t], n);
        } else {
            add_side_normal(ps[2], n);
            add_side_normal(ps[1], n);
        }
        const double inv = 1.0 / sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int d = 0; d < 3; d++) n[d] *= inv;
    }
    for (int d = 0; d < 3; d++) xi[d] = x1[d] + (x2[d] - x1[d]) * t_entry;
}
// Species::sampleReflectedVelocity (Species.cpp:835-853) with sampleVth(300) (855-861): full
// thermal accommodation at 300 K, direction from the reference's diffuse vector (whose t2 term
// carries no sin(theta) factor, kept as it is)
__device__ void reflect_d(double mass, double v_mag1, const double n[3], DrawStream& r, double out[3]) {
    const double v_th0 = sqrt(2 * kKbRef * 300.0 / mass);
    double s3[3];
    for (int d = 0; d < 3; d++) {
        const double u1 = r.next(), u2 = r.next(), u3 = r.next();
        s3[d] = v_th0 * (u1 + u2 + u3 - 1.5);
    }
    const double v_th = sqrt(s3[0] * s3[0] + s3[1] * s3[1] + s3[2] * s3[2]);
    const double v_mag2 = v_mag1 + 1.0 * (v_th - v_mag1);
    const double sin_theta = r.next();
    const double cos_theta = sqrt(1 - sin_theta * sin_theta);
    const double psi = 2 * kPiRef * r.next();
    double t1[3];
    if (n[0] != 0) {  // n x (1,0,0)
        t1[0] = 0.0;
        t1[1] = n[2];
        t1[2] = -n[1];
    } else {  // n x (0,1,0)
        t1[0] = -n[2];
        t1[1] = 0.0;
        t1[2] = n[0];
    }
    const double t2[3] = {n[1] * t1[2] - n[2] * t1[1], n[2] * t1[0] - n[0] * t1[2], n[0] * t1[1] - n[1] * t1[0]};
    const double a = sin_theta * cos(psi), b = sin(psi);
    for (int d = 0; d < 3; d++) out[d] = (t1[d] * a + t2[d] * b + n[d] * cos_theta) * v_mag2;
}
__device__ bool in_bounds_d(const GridDev& g, const double x[3]) {  // World::inBounds (World.cpp:201-205)
    for (int d = 0; d < 3; d++)
        if (x[d] < g.x0[d] || x[d] >= g.xm[d]) return false;
    return true;
}
// an absolute position as (offsets, packed cell), as the upload path converts it
__device__ float4 to_cell(const GridDev& g, const double x[3]) {
    const int nc3[3] = {g.ci, g.cj, g.ck};
    int ijk[3];
    float o[3];
    for (int d = 0; d < 3; d++) {
        const double lc = (x[d] - g.x0[d]) / g.dxd[d];
        int c = (int)lc;
        if (c >= nc3[d]) c = nc3[d] - 1;
        ijk[d] = c;
        o[d] = fminf((float)(lc - c), 0x1.fffffep-1f);
    }
    return make_float4(o[0], o[1], o[2], __int_as_float(pack_cell(ijk[0], ijk[1], ijk[2])));
}
// ids of the particles an impact creates: distinct from the parent's and from the merge's
__device__ unsigned long long obj_child_id(unsigned long long parent, unsigned step, unsigned k) {
    return mix64(child_id(parent, step, 3) + (unsigned long long)(k + 1) * 0xD1B54A32D192ED03ull);
}
// Field::gather of E at an absolute position in FP64 (Field.h:200-232, World::XtoL)
__device__ void gather_e_d(const GridDev& g, const float4* ef, const double x[3], double e[3]) {
    double f[3];
    int c[3];
    const int nc3[3] = {g.ci, g.cj, g.ck};
    for (int d = 0; d < 3; d++) {
        const double lc = (x[d] - g.x0[d]) * (1.0 / g.dxd[d]);
        c[d] = min((int)lc, nc3[d] - 1);
        f[d] = lc - c[d];
    }
    e[0] = e[1] = e[2] = 0.0;
    for (int c8 = 0; c8 < 8; c8++) {
        const int a = c8 & 1, b = (c8 >> 1) & 1, k = c8 >> 2;
        const double wt = (a ? f[0] : 1 - f[0]) * (b ? f[1] : 1 - f[1]) * (k ? f[2] : 1 - f[2]);
        const float4 E = ef[cell_base_node(g, c[0] + a, c[1] + b, c[2] + k)];
        e[0] += wt * E.x;
        e[1] += wt * E.y;
        e[2] += wt * E.z;
    }
}
// Species::addParticle(pos, vel) (Species.cpp:420-434): NaN, bounds and objects rejected (a
// point on an object's surface counts as inside, Object.cpp:235), then v -= q/m E dt/2
__device__ bool add_neutral(const ObjArgs& o, const SpeciesDev& sp, double qm, int n0, const double x[3],
                            const double v[3], double w, unsigned long long id) {
    for (int d = 0; d < 3; d++)
        if (isnan(x[d]) || isnan(v[d])) return false;
    if (!in_bounds_d(o.a.g, x) || in_object_d(o, x)) return false;
    double vr[3] = {v[0], v[1], v[2]};
    if (qm != 0.0) {
        double e[3];
        gather_e_d(o.a.g, o.a.ef, x, e);
        for (int d = 0; d < 3; d++) vr[d] -= e[d] * qm * o.half_dt_global;
    }
    return append_particle(sp, n0, to_cell(o.a.g, x), make_float4((float)vr[0], (float)vr[1], (float)vr[2], (float)w),
                           id, o.a.err);
}

__global__ void __launch_bounds__(128) k_object_hits(ObjArgs o) {
    const GridDev& g = o.a.g;
    const SpeciesDev& sp = o.a.sp;
    const int nd = sp.counts[2], n_self = sp.counts[0];
    const int n_neu = o.charged ? o.neu.counts[0] : 0, n_spu = o.charged && o.sputtering ? o.spu.counts[0] : 0;
    unsigned long long st[4] = {0, 0, 0, 0};
    for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < nd; d += gridDim.x * blockDim.x) {
        const int p = sp.dead[d];
        const float4 P = sp.pos[p];
        const int c = __float_as_int(P.w);
        if (c >= 0 || c == -1) continue;  // alive, or left the domain
        int ijk[3];
        cell_ijk(g, c & ~kHitFlag, ijk[0], ijk[1], ijk[2]);
        const float4 V = sp.vel[p];
        const unsigned long long id = sp.id[p];
        const double w = V.w;
        const float off[3] = {P.x, P.y, P.z};
        double v[3] = {V.x, V.y, V.z}, x1[3], x2[3];
        for (int k = 0; k < 3; k++) {
            x2[k] = g.x0[k] + ((double)ijk[k] + (double)off[k]) * g.dxd[k];
            x1[k] = x2[k] - v[k] * o.dt;  // the start of the push's move
        }
        st[0]++;
        DrawStream r(id, o.step, o.key);
        double t_rem = 1.0;
        int n_bounces = 1;  // the push made the first move
        bool alive = true;
        while (true) {
            const int obj = in_object_d(o, x2);
            if (!obj) break;  // FP32 said inside, FP64 says outside: the move stands
            double tp, xi[3], nrm[3];
            line_intersect_d(o, obj - 1, x1, x2, tp, xi, nrm);
            const double vmag = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            if (!o.charged) {  // neutrals bounce (Species.cpp:221-223)
                reflect_d(o.mass, vmag, nrm, r, v);
                st[1]++;
                t_rem *= (1 - tp);
                if (++n_bounces > 20) {
                    alive = false;
                    break;
                }
                for (int k = 0; k < 3; k++) {
                    x1[k] = xi[k];
                    x2[k] = xi[k] + v[k] * t_rem * o.dt;
                    if (g.periodic[k]) {
                        const double L = g.xm[k] - g.x0[k];
                        if (x2[k] < g.x0[k]) x2[k] += L;
                        else if (x2[k] >= g.xm[k]) x2[k] -= L;
                    }
                }
                if (!in_bounds_d(g, x2)) {
                    alive = false;
                    break;
                }
                continue;
            }
            // ions: neutrals of the neutral species' weight at the impact point (Species.cpp:225-235)
            const int m = (int)(w / o.neu_mpw0 + r.next());
            for (int q = 0; q < m; q++) {
                double vn[3];
                reflect_d(o.mass, vmag, nrm, r, vn);
                st[2] += add_neutral(o, o.neu, o.neu_qm, n_neu, xi, vn, o.neu_mpw0, obj_child_id(id, o.step, (unsigned)q));
            }
            if (o.sputtering) {  // simple yield model (Species.cpp:136-144)
                const double yield = vmag > 5e3 ? 0.1 : 0.0;
                const int ms = (int)(yield * w / o.spu_mpw0 + r.next());
                for (int q = 0; q < ms; q++) {
                    double vn[3];
                    reflect_d(o.mass, vmag, nrm, r, vn);
                    st[3] += add_neutral(o, o.spu, o.spu_qm, n_spu, xi, vn, o.spu_mpw0,
                                         obj_child_id(id, o.step, 0x10000000u + (unsigned)q));
                }
            }
            alive = false;
            break;
        }
        if (!alive) continue;
        // the particle lives on: re-created at its final position with its id, and deposited
        const float4 np = to_cell(g, x2);
        if (!append_particle(sp, n_self, np, make_float4((float)v[0], (float)v[1], (float)v[2], V.w), id, o.a.err))
            continue;
        if (o.a.deposit) {
            Corners hc;
            corner_values(V.w, make_float3(np.x, np.y, np.z), o.a.dep_scale, hc, false);
            const int b = cell_base(g, __float_as_int(np.w));
            const int offs[4] = {0, g.ni, g.ni * g.nj, g.ni * g.nj + g.ni};
            for (int c8 = 0; c8 < 8; c8++)
                if (hc.q[c8]) atomicAdd(&sp.acc[b + offs[c8 >> 1] + (c8 & 1)], hc.q[c8]);
        }
    }
    for (int k = 0; k < 4; k++)
        if (st[k]) atomicAdd(&o.stats[k], st[k]);
}
}  // namespace

void launch_object_hits(const ObjArgs& o, cudaStream_t s, int grid) { k_object_hits<<<grid, 128, 0, s>>>(o); }

__global__ void k_load_count(SpeciesDev sp, int n) {
    int nn = sp.counts[0] + n;
    sp.counts[0] = nn > sp.capacity ? sp.capacity : nn;
}
void launch_load_uniform(const GridDev& g, SpeciesDev sp, const LoadArgs& la, cudaStream_t s) {
    int grid = (la.n + 255) / 256;
    if (grid > 8192) grid = 8192;
    if (grid < 1) grid = 1;
    k_load_uniform<<<grid, 256, 0, s>>>(g, sp, la);
    k_load_count<<<1, 1, 0, s>>>(sp, la.n);
}

// ------------------------------------------------------------------------------------
// FP64 conservation sums (Species::getMicroCount / getMomentum / getKE, Species.cpp:732-752)
// out[0] sum w, out[1..3] sum w v, out[4] sum w v.v   (per-block partials reduced on host side)
// ------------------------------------------------------------------------------------
// compensated FP32 accumulation: hi += x by TwoSum, its rounding error and the exact error ex of
// the term collected in lo
__device__ __forceinline__ void comp_add(float& hi, float& lo, float x, float ex) {
    const FF s = two_sum(hi, x);
    hi = s.hi;
    lo += s.lo + ex;
}
__global__ void k_sums(SpeciesDev sp, double* part) {
    int n = sp.counts[0];
    // per-thread compensated sums of w, w v (exact products) and w |v|^2 (|v|^2 rounded once, as
    // the FP32 velocities it comes from; the exact product with w), FP64 only for the per-thread
    // totals and the block sums: the totals do not depend on the particle order beyond ~1e-14
    float h[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, l[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll 4
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        const float4 v = sp.vel[p];
        comp_add(h[0], l[0], v.w, 0.f);
        const FF px = two_prod(v.w, v.x), py = two_prod(v.w, v.y), pz = two_prod(v.w, v.z);
        comp_add(h[1], l[1], px.hi, px.lo);
        comp_add(h[2], l[2], py.hi, py.lo);
        comp_add(h[3], l[3], pz.hi, pz.lo);
        const FF ke = two_prod(v.w, fmaf(v.z, v.z, fmaf(v.y, v.y, v.x * v.x)));
        comp_add(h[4], l[4], ke.hi, ke.lo);
    }
    __shared__ double s[5][8];
    for (int c = 0; c < 5; c++) {
        double x = (double)h[c] + (double)l[c];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0) s[c][threadIdx.x >> 5] = x;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        double x = 0;
        for (int w = 0; w < 8; w++) x += s[threadIdx.x][w];
        part[blockIdx.x * 5 + threadIdx.x] = x;
    }
}
void launch_sums(SpeciesDev sp, double* out, cudaStream_t s, int grid) { k_sums<<<grid, 256, 0, s>>>(sp, out); }

// ------------------------------------------------------------------------------------
// velocity-binned merge (Species::merge + sortVelocitiesInCell, Species.cpp:981-1145)
// GPU form: per cell a CTA bins velocities on a 15^3 grid between the cell's min and max,
// orders the cell by (bin, Philox hash of the id), and every bin with more than two particles
// becomes two particles of half the bin weight at mean +- per-axis rms velocity, placed at the
// two members with the smallest hashes (the reference picks two random members).  Sums are
// FP64 in that order, so the result does not depend on the order of the particles in memory.
// ------------------------------------------------------------------------------------
constexpr int kMergeThreads = 128;
constexpr int kMergeMax = 1024;  // particles of one cell handled per merge
constexpr int kVelGrid = 15;     // Species.h:129

__global__ void k_merge_candidates(SpeciesDev sp, const int* start, int nc, int min_count, int* list, int* nlist) {
    int n = sp.counts[0];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        int cnt = (c + 1 < nc ? start[c + 1] : n) - start[c];
        if (cnt >= min_count) list[atomicAdd(nlist, 1)] = c;
    }
}

__device__ __forceinline__ int vel_bin(float v, float vmin, float dv) {
    if (!(dv > 0.f)) return 0;
    int b = (int)__fdiv_rn(__fsub_rn(v, vmin), dv);
    return b < 0 ? 0 : (b > kVelGrid - 1 ? kVelGrid - 1 : b);
}

struct MergeArgs {
    GridDev g;
    SpeciesDev sp;
    const float4* ef;
    const int* start;
    const int* list;
    const int* nlist;
    float qm_half_dt;  // rewind of addParticle (Species.cpp:431), global dt
    uint2 key;
    unsigned step;
    unsigned* err;
    unsigned long long* stats;  // [0] bins merged, [1] particles removed, [2] products dropped (NaN)
};

__global__ void __launch_bounds__(kMergeThreads) k_merge(MergeArgs a) {
    __shared__ unsigned long long keys[kMergeMax];
    __shared__ float4 vs[kMergeMax];
    __shared__ float s_red[6][kMergeThreads / 32];
    __shared__ float s_min[3], s_dv[3];
    const int n = a.sp.counts[0];
    const int nl = *a.nlist;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    for (int li = blockIdx.x; li < nl; li += gridDim.x) {
        const int c = a.list[li];
        const int s0 = a.start[c];
        int m = (c + 1 < a.g.nc ? a.start[c + 1] : n) - s0;
        if (m > kMergeMax) {
            if (tid == 0) set_error(a.err, kErrMergeTruncated);
            m = kMergeMax;
        }
        float mn[3] = {INFINITY, INFINITY, INFINITY}, mx[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int q = tid; q < m; q += kMergeThreads) {
            float4 v = a.sp.vel[s0 + q];
            vs[q] = v;
            mn[0] = fminf(mn[0], v.x); mn[1] = fminf(mn[1], v.y); mn[2] = fminf(mn[2], v.z);
            mx[0] = fmaxf(mx[0], v.x); mx[1] = fmaxf(mx[1], v.y); mx[2] = fmaxf(mx[2], v.z);
        }
        for (int d = 0; d < 3; d++) {
            for (int o = 16; o > 0; o >>= 1) {
                mn[d] = fminf(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
                mx[d] = fmaxf(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
            }
            if (lane == 0) {
                s_red[d][warp] = mn[d];
                s_red[3 + d][warp] = mx[d];
            }
        }
        __syncthreads();
        if (tid < 3) {
            float lo = s_red[tid][0], hi = s_red[3 + tid][0];
            for (int w = 1; w < kMergeThreads / 32; w++) {
                lo = fminf(lo, s_red[tid][w]);
                hi = fmaxf(hi, s_red[3 + tid][w]);
            }
            hi = hi > 0.f ? __fmul_rn(hi, 1.001f) : __fmul_rn(hi, 0.999f);  // Species.cpp:1007-1013
            s_min[tid] = lo;
            s_dv[tid] = __fdiv_rn(__fsub_rn(hi, lo), (float)kVelGrid);
        }
        __syncthreads();
        // keys: bin (12 bits) | hash (42 bits) | local index (10 bits)
        int P = 1;
        while (P < m) P <<= 1;
        for (int q = tid; q < P; q += kMergeThreads) {
            if (q < m) {
                float4 v = vs[q];
                int b = (vel_bin(v.x, s_min[0], s_dv[0]) * kVelGrid + vel_bin(v.y, s_min[1], s_dv[1])) * kVelGrid +
                        vel_bin(v.z, s_min[2], s_dv[2]);
                unsigned long long id = a.sp.id[s0 + q];
                uint4 h = philox4x32_10(make_uint4((unsigned)id, (unsigned)(id >> 32), a.step, 0x4D455247u), a.key);
                unsigned long long hh = ((unsigned long long)h.y << 32 | h.x) & ((1ull << 42) - 1);
                keys[q] = ((unsigned long long)b << 52) | (hh << 10) | (unsigned long long)q;
            } else {
                keys[q] = ~0ull;
            }
        }
        __syncthreads();
        // bitonic sort of P keys
        for (int k = 2; k <= P; k <<= 1)
            for (int j = k >> 1; j > 0; j >>= 1) {
                for (int q = tid; q < P; q += kMergeThreads) {
                    int r = q ^ j;
                    if (r > q) {
                        unsigned long long x = keys[q], y = keys[r];
                        bool up = (q & k) == 0;
                        if ((x > y) == up) {
                            keys[q] = y;
                            keys[r] = x;
                        }
                    }
                }
                __syncthreads();
            }
        // one thread per run of equal bins
        for (int q = tid; q < m; q += kMergeThreads) {
            unsigned bq = (unsigned)(keys[q] >> 52);
            if (q > 0 && (unsigned)(keys[q - 1] >> 52) == bq) continue;
            int e = q + 1;
            while (e < m && (unsigned)(keys[e] >> 52) == bq) e++;
            if (e - q <= 2) continue;  // Species.cpp:1058: merge bins with more than two particles
            double W = 0, M[3] = {0, 0, 0}, E[3] = {0, 0, 0};
            for (int r = q; r < e; r++) {
                float4 v = vs[keys[r] & 1023];
                double w = v.w, vx = v.x, vy = v.y, vz = v.z;
                W += w;
                M[0] += w * vx; M[1] += w * vy; M[2] += w * vz;
                E[0] += w * (vx * vx); E[1] += w * (vy * vy); E[2] += w * (vz * vz);
            }
            double inv = 1.0 / W;
            for (int d = 0; d < 3; d++) {
                M[d] *= inv;
                E[d] = E[d] * inv - M[d] * M[d];
            }
            for (int d = 0; d < 3; d++)  // Species.cpp:1074-1082
                if (E[d] < 0) {
                    if (E[d] < -10e-5) break;
                    E[d] = 0;
                }
            double sq[3] = {sqrt(E[0]), sqrt(E[1]), sqrt(E[2])};
            int la = (int)(keys[q] & 1023), lb = (int)(keys[q + 1] & 1023);
            for (int r = q; r < e; r++) {
                int p = s0 + (int)(keys[r] & 1023);
                float4 ps = a.sp.pos[p];
                a.sp.pos[p] = make_float4(ps.x, ps.y, ps.z, __int_as_float(-1));
            }
            int base = atomicAdd(&a.sp.counts[2], e - q);
            for (int r = q; r < e; r++) a.sp.dead[base + (r - q)] = s0 + (int)(keys[r] & 1023);
            atomicAdd(&a.stats[0], 1ull);
            atomicAdd(&a.stats[1], (unsigned long long)(e - q));
            int i, j, k;
            linear_ijk(a.g, c, i, j, k);
            int bnode = cell_base_node(a.g, i, j, k);
            const int cpk = pack_cell(i, j, k);
            Tile t;
            t.etile = nullptr;
            t.dtile = nullptr;
            t.lo = 0;
            t.span = -1;
            t.off[0] = 0;
            t.off[1] = a.g.ni;
            t.off[2] = a.g.ni * a.g.nj;
            t.off[3] = a.g.ni * a.g.nj + a.g.ni;
            PushArgs pa;
            pa.ef = a.ef;
            for (int side = 0; side < 2; side++) {
                int l = side == 0 ? la : lb;
                float4 ps = a.sp.pos[s0 + l];
                float3 o = make_float3(ps.x, ps.y, ps.z);
                double sgn = side == 0 ? 1.0 : -1.0;
                float3 v = make_float3((float)(M[0] + sgn * sq[0]), (float)(M[1] + sgn * sq[1]),
                                       (float)(M[2] + sgn * sq[2]));
                if (isnan(v.x) || isnan(v.y) || isnan(v.z)) {  // addParticle drops NaN (Species.cpp:421-423)
                    atomicAdd(&a.stats[2], 1ull);
                    continue;
                }
                float3 Ev = gather_e(pa, t, bnode, o);
                v.x -= a.qm_half_dt * Ev.x;
                v.y -= a.qm_half_dt * Ev.y;
                v.z -= a.qm_half_dt * Ev.z;
                unsigned long long pid = child_id(a.sp.id[s0 + l], a.step, 3);
                append_particle(a.sp, n, make_float4(o.x, o.y, o.z, __int_as_float(cpk)),
                                make_float4(v.x, v.y, v.z, (float)(W * 0.5)), pid, a.err);
            }
        }
        __syncthreads();
    }
}

void launch_merge(const GridDev& g, SpeciesDev sp, const float4* ef, const int* cell_start, int* list, int* nlist,
                  int min_count, float qm_half_dt, uint2 key, unsigned step, unsigned* err,
                  unsigned long long* stats, cudaStream_t s, int grid) {
    cudaMemsetAsync(nlist, 0, sizeof(int), s);
    k_merge_candidates<<<1024, 256, 0, s>>>(sp, cell_start, g.nc, min_count, list, nlist);
    MergeArgs a;
    a.g = g;
    a.sp = sp;
    a.ef = ef;
    a.start = cell_start;
    a.list = list;
    a.nlist = nlist;
    a.qm_half_dt = qm_half_dt;
    a.key = key;
    a.step = step;
    a.err = err;
    a.stats = stats;
    k_merge<<<grid, kMergeThreads, 0, s>>>(a);
}

}  // namespace pic

namespace pic {
// ------------------------------------------------------------------------------------
// velocity moments (Species::sampleMoments, Species.cpp:767-776): n, n v, n u^2, n v^2, n w^2
// scattered with the CIC weights and accumulated across calls until cleared (the reference
// never clears them inside the loop).  FP32 atomics: a diagnostic, not bit-reproducible.
// mom layout: 7 planes of nv floats: n, nvx, nvy, nvz, nuu, nvv, nww
// ------------------------------------------------------------------------------------
__global__ void k_sample_moments(GridDev g, SpeciesDev sp, float* __restrict__ mom) {
    const int n = sp.counts[0];
    const int nij = g.ni * g.nj;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        float4 ps = sp.pos[p], vs = sp.vel[p];
        int c = __float_as_int(ps.w);
        if (c < 0) continue;
        int i, j, k;
        cell_ijk(g, c, i, j, k);
        int b = cell_base_node(g, i, j, k);
        float wx1 = ps.x, wx0 = 1.f - ps.x, wy1 = ps.y, wy0 = 1.f - ps.y, wz1 = ps.z, wz0 = 1.f - ps.z;
        float wc[8] = {wx0 * wy0 * wz0, wx1 * wy0 * wz0, wx0 * wy1 * wz0, wx1 * wy1 * wz0,
                       wx0 * wy0 * wz1, wx1 * wy0 * wz1, wx0 * wy1 * wz1, wx1 * wy1 * wz1};
        int nd[8] = {b, b + 1, b + g.ni, b + g.ni + 1, b + nij, b + nij + 1, b + nij + g.ni, b + nij + g.ni + 1};
        float val[7] = {vs.w, vs.w * vs.x, vs.w * vs.y, vs.w * vs.z, vs.w * vs.x * vs.x, vs.w * vs.y * vs.y,
                        vs.w * vs.z * vs.z};
#pragma unroll
        for (int m = 0; m < 7; m++)
#pragma unroll
            for (int c8 = 0; c8 < 8; c8++) atomicAdd(&mom[(size_t)m * g.nv + nd[c8]], val[m] * wc[c8]);
    }
}
void launch_sample_moments(const GridDev& g, SpeciesDev sp, float* mom, cudaStream_t s, int grid) {
    k_sample_moments<<<grid, 256, 0, s>>>(g, sp, mom);
}
}  // namespace pic
