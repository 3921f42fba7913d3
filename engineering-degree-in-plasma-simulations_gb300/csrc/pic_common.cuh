// Shared device-side definitions of the GB300 PIC + DSMC library (sm_103a).
//
// Data layout in HBM (one World):
//   nodes  n = (k*nj + j)*ni + i            (reference Field::U, ch4/v3/src/Field.h:262-265)
//   cells  c = (k*(nj-1) + j)*(ni-1) + i    (reference World::XtoC, ch4/v3/src/World.cpp:134-137)
//   E      float4 per node {Ex, Ey, Ez, 0}  (16 B aligned: TMA bulk copies of node rows)
//   phi    double per node (master copy; FP32 inner solves refine it)
//   rho    float per node
//   kind   uint8 per node: bits 0-1 node kind, bits 2-7 "neighbour d is a mirror wall"
// Particles of a species, structure of arrays:
//   pos    float4 {ox, oy, oz, cell-as-int}   offsets in [0,1) inside the cell
//   vel    float4 {vx, vy, vz, w}             m/s and macroweight
//   id     uint64                             keys the Philox streams
// Charge deposition accumulates 64-bit fixed-point integers per node and species, so the
// node sums do not depend on the order of the atomic updates.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace pic {

constexpr int kMaxSpecies = 4;
constexpr int kMaxBoxes = 8;

enum NodeKind : uint8_t { kFree = 0, kFixed = 1, kMirror = 2, kAlias = 3 };

// device error word bits (read back by pic_last_error)
enum DevError : unsigned {
    kErrCapacity = 1u << 0,    // an append would exceed the species capacity
    kErrBarrierTimeout = 1u << 1,  // an mbarrier wait ran out of iterations
    kErrMergeTruncated = 1u << 2,  // a merge cell held more particles than the per-cell cap
    kErrNaN = 1u << 3,
};

// division by a runtime constant with a multiply-high (Granlund & Montgomery 1994), exact for
// every 32-bit dividend; d >= 2
struct FastDiv {
    unsigned d, m, l;
};
__host__ __device__ inline FastDiv make_fastdiv(unsigned d) {
    unsigned l = 0;
    while ((1ull << l) < d) l++;
    unsigned long long m = ((1ull << 32) * ((1ull << l) - d)) / d + 1;
    return FastDiv{d, (unsigned)m, l};
}
__device__ __forceinline__ unsigned fdiv(unsigned n, const FastDiv& f) {
    unsigned t = __umulhi(f.m, n);
    return (t + ((n - t) >> 1)) >> (f.l - 1);
}

struct GridDev {
    FastDiv fd_ni, fd_nj;  // node index decoding
    int ni, nj, nk;       // nodes
    int ci, cj, ck;       // cells per axis (n-1)
    int nv, nc;           // node and cell totals
    int periodic[3];
    float dx[3], inv_dx[3];
    float c_hi[3], c_lo[3];  // 1/dx^2 per axis as float-float (hi + lo), set on the host
    float inv2dx[3];         // 1/(2 dx) per axis
    float inv_cell_vol;      // 1/(dx dy dz)
    double x0[3], xm[3], dxd[3];
    int n_boxes;
    float box_lo[kMaxBoxes][3], box_hi[kMaxBoxes][3];  // absorbing objects, absolute coordinates
    // independent instances stacked along z: zslab nodes per instance (0: one instance); the
    // first and last node plane of every slab are Dirichlet electrodes, the cell between two
    // slabs is outside every instance
    int zslab;
    FastDiv fd_zslab;
    int node_grid;  // CTAs of the streaming node kernels chosen by the autotuner (0: default)
    int cg_grid;    // CTAs of the CG stencil kernels (d = z + beta d, q = L d) chosen likewise (0: node_grid)
    // one bit per node, set on FREE nodes: row (j, k) of x bits starts at word (k nj + j) free_wpr
    const unsigned* free_bits;
    int free_wpr;
};
// z index of a node or cell inside its instance slab (the global index without slabs)
__device__ __forceinline__ int slab_local_z(const GridDev& g, int k) {
    return g.zslab ? k - (int)fdiv((unsigned)k, g.fd_zslab) * g.zslab : k;
}

struct SpeciesDev {
    float4* pos;
    float4* vel;
    unsigned long long* id;
    int* counts;  // [0] n, [1] pending appends, [2] dead, [3] holes, [4] movers,
                  // [5] particles moved to another cell or appended since the last sort
    int* dead;    // dead particle indices of the last push
    int* holes;   // compaction scratch
    unsigned long long* acc;  // fixed-point number-density accumulators, one per node
    int capacity;
};

// ------------------------------------------------------------------------------------
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11)
// ------------------------------------------------------------------------------------
__host__ __device__ __forceinline__ unsigned mulhi32(unsigned a, unsigned b) {
#ifdef __CUDA_ARCH__
    return __umulhi(a, b);
#else
    return (unsigned)(((unsigned long long)a * b) >> 32);
#endif
}
__host__ __device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; r++) {
        unsigned hi0 = mulhi32(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        unsigned hi1 = mulhi32(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}
// uniform in (0,1): ((x >> 9) + 0.5) * 2^-23, 24 significant bits, exact in FP32
__host__ __device__ __forceinline__ float u01(unsigned x) { return ((float)(x >> 9) + 0.5f) * (1.0f / 8388608.0f); }

// splitmix64 finaliser (Steele, Lea, Flood 2014)
__device__ __forceinline__ unsigned long long mix64(unsigned long long x) {
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
// ids of collision products
__device__ __forceinline__ unsigned long long child_id(unsigned long long parent, unsigned step, unsigned kind) {
    return mix64(parent + 0x9E3779B97F4A7C15ull * ((((unsigned long long)step) << 2) | kind));
}
// 32-bit draw of the null-collision candidate test of particle id at a step: output step + 1 of
// a SplitMix64 stream whose seed is the scrambled (id xor key), so the decision is keyed by
// (seed, step, id) and independent of the particle order, for four 64-bit multiplies
__device__ __forceinline__ unsigned cand_draw(unsigned long long id, unsigned step, uint2 key) {
    const unsigned long long s = mix64(id ^ (((unsigned long long)key.y << 32) | key.x));
    return (unsigned)(mix64(s + 0x9E3779B97F4A7C15ull * ((unsigned long long)step + 1ull)) >> 32);
}

__device__ __forceinline__ void set_error(unsigned* err, unsigned bit) {
    if (err) atomicOr(err, bit);
}

// A particle's cell is stored packed, i | j << 9 | k << 18 (i, j < 512, k < 8192): decoding
// needs no division, and the packed value orders cells exactly like the linear index
// c = (k*(nj-1) + j)*(ni-1) + i of World::XtoC, which the sort and the cell lists use.
constexpr int kCellMaxIJ = 512, kCellMaxK = 8192;
__host__ __device__ __forceinline__ int pack_cell(int i, int j, int k) { return i | (j << 9) | (k << 18); }
// marks the packed cell of a particle that moved into an object during a push (the value is
// negative, so the particle is removed unless the object interaction re-creates it)
constexpr int kHitFlag = (int)0x80000000u;
__device__ __forceinline__ void cell_ijk(const GridDev&, int c, int& i, int& j, int& k) {
    i = c & 511;
    j = (c >> 9) & 511;
    k = c >> 18;
}
__device__ __forceinline__ int cell_linear(const GridDev& g, int c) {
    return ((c >> 18) * g.cj + ((c >> 9) & 511)) * g.ci + (c & 511);
}
// base node of the packed cell c
__device__ __forceinline__ int cell_base(const GridDev& g, int c) {
    return ((c >> 18) * g.nj + ((c >> 9) & 511)) * g.ni + (c & 511);
}
// linear cell index -> (i, j, k)
__device__ __forceinline__ void linear_ijk(const GridDev& g, int c, int& i, int& j, int& k) {
    int cij = g.ci * g.cj;
    k = c / cij;
    int r = c - k * cij;
    j = r / g.ci;
    i = r - j * g.ci;
}
// base node of cell (i,j,k)
__device__ __forceinline__ int cell_base_node(const GridDev& g, int i, int j, int k) {
    return (k * g.nj + j) * g.ni + i;
}

}  // namespace pic
