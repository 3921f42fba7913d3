// Host-side launch wrappers shared between the kernel translation units and the C ABI.
#pragma once
#include "pic_common.cuh"

namespace pic {

int set_last_error(int code, const char* msg);  // message for pic_last_error

// Electron-impact collisions against a uniform background gas (candidates, then collisions)
struct CollDev {
    int enabled;
    unsigned cand_max;       // candidate threshold 2^32 n_n (sigma v)_max dt on cand_draw (the largest
                             // of the slabs' when cand_slab is set)
    const unsigned* cand_slab;  // per instance slab (stacked instances with their own n_n), or nullptr
    float sigv_max;          // (sigma v)_max [m^3/s]
    float sig_n;             // sqrt(k T_n / m_n): neutral thermal speed per axis
    float m_n, m_e;
    float E_precalc_rel_eV;  // 0.5 m_red / q
    float half_mred;         // 0.5 m_red
    float E_precalc_ele_eV;  // m_e 0.5 / q
    float E_ion_eV, B_inc, two_q_over_me;
    int sig_kind;            // 0 reference fit, 1 Lotz
    float sig_a, sig_b, sig_c, sig_A;
    const float* tE;         // sigma_coll table energies [eV], ascending
    const float* tS;         // sigma_coll table values [m^2]
    int tn;
    uint2 key;
    unsigned step;
    SpeciesDev ion;          // ion products are appended here
    unsigned long long* stats;  // [0] candidates [1] collisions [2] ionisations [3] products lost
};

struct PushArgs {
    GridDev g;
    SpeciesDev sp;
    const float4* ef;
    float qm_dt;     // q/m dt
    float dtdx[3];   // dt/dx per axis
    int deposit;     // scatter the weight at the new position
    float dep_scale; // fixed-point scale (power of two)
    int staged;      // allow TMA-staged E tiles
    unsigned* err;
    CollDev coll;
    // mbarrier polls of a wait for a bulk copy before it gives up: 0 (the zero-initialised
    // value) kMbarWaitPolls, > 0 that many, < 0 none (a test makes the wait run out).  The drain
    // of the copies in flight after a timeout always allows kMbarWaitPolls.
    long long wait_polls;
};
__host__ __device__ inline long long wait_poll_limit(long long arg, long long dflt) {
    return arg == 0 ? dflt : (arg < 0 ? 0 : arg);
}
constexpr long long kMbarWaitPolls = 1ll << 24;

// particles
int push_blocks_per_sm();  // resident push CTAs per SM (the push grid is this times the SM count)
void launch_push(const PushArgs& a, cudaStream_t s, int grid);
// collisions of a.coll for the electrons a.sp as two passes (candidates, their collisions); the
// push that follows runs without collisions.  cand holds up to the species capacity.
void launch_mcc(const PushArgs& a, int* cand, int* ncand, cudaStream_t s, int sms);
void launch_commit_appends(SpeciesDev sp, unsigned* err, cudaStream_t s);
void launch_compact(SpeciesDev sp, cudaStream_t s, int grid);
void launch_sort(const GridDev& g, SpeciesDev sp, float4* pos_alt, float4* vel_alt, unsigned long long* id_alt,
                 int* cell_count, int* cell_start, int* scan_aux, cudaStream_t s, int grid);
void launch_from_abs(const GridDev& g, SpeciesDev sp, const double* pos, const double* vel, const double* w,
                     const unsigned long long* id, unsigned long long id0, int n, int rewind, float qm_half_dt,
                     const float4* ef, cudaStream_t s,
                     int max_grid = 4096);
// particles first + p * stride, p < n, to absolute FP64 positions (null outputs are skipped)
void launch_to_abs(const GridDev& g, SpeciesDev sp, double* pos, double* vel, double* w, unsigned long long* id,
                   int n, cudaStream_t s, long long first = 0, long long stride = 1);
struct LoadArgs {
    double lo[3], hi[3];   // absolute box
    float vth;             // sqrt(kT/m) per axis (Maxwellian) or sqrt(2kT/m) (reference sampleV3th)
    int ref_thermal;       // 1: Species::sampleV3th speeds and directions (Species.cpp:855-869)
    float w_mean, w_sigma; // lognormal weight (sigma 0: constant w_mean)
    unsigned long long id0;
    uint2 key;
    int n;
};
void launch_load_uniform(const GridDev& g, SpeciesDev sp, const LoadArgs& la, cudaStream_t s);
// one step of a beam source (ColdBeamSource / WarmBeamSource::sample, Source.cpp:35-192):
// n particles on the inlet face, FP64 positions and velocities into pos / vel / w (then added
// with Species::addParticle semantics)
struct SourceArgs {
    double x0[3], L[3];     // domain origin; extents of the sampled face (the + faces one cell in)
    int face;               // 0..5: x-, x+, y-, y+, z-, z+
    double v_drift;         // along the inward normal
    double vth;             // sqrt(2kT/m) of Species::sampleVth, 0 for a cold beam
    double mpw0;            // macroparticle weight
    uint2 key;              // Philox key (seed)
    unsigned step, src;     // counter words: the step and the source index
    int first, n;           // particles first .. first + n - 1 of the step
};
void launch_source(const SourceArgs& sa, double* pos, double* vel, double* w, cudaStream_t s);

// Object interaction of a non-electron species (Species::advanceNoSputteringSerial and
// advanceSputteringSerial, Species.cpp:79-256) for the particles the last push flagged with
// kHitFlag: neutrals bounce diffusely off the object, ions are removed and leave neutrals
// (and, with sputtering, sputtered particles) at the impact point.  FP64, one thread per hit.
struct ObjArgs {
    PushArgs a;                 // the pushed species, its deposit settings and the grid
    double dt;                  // time step of that push
    double mass;                // the pushed species' mass (Species::sampleVth)
    int charged;                // ions are neutralised, neutrals bounce
    SpeciesDev neu, spu;        // neutral and sputtered-material species (charged species only)
    double neu_mpw0, spu_mpw0;  // their macroparticle weights (Species::addParticle(pos, vel))
    double neu_qm, spu_qm;      // their charge / mass, for addParticle's half-step rewind
    double half_dt_global;      // 0.5 World::getDt()
    int sputtering;             // Config::SPUTTERING
    int n_boxes;
    double box_c[kMaxBoxes][3], box_half[kMaxBoxes][3];  // Rectangle pos and half_sides
    uint2 key;                  // Philox key (seed)
    unsigned step;              // counter word
    unsigned long long* stats;  // [0] hits, [1] bounces, [2] neutrals created, [3] sputtered created
};
void launch_object_hits(const ObjArgs& o, cudaStream_t s, int grid);

// DSMC_MEX on sorted species: cell c of species k owns particles [start_k[c], start_k[c+1])
// (the last cell ends at the species count *n_k); vel2 == vel1 and one = 1 for one species
struct DsmcArgs {
    float4* vel1;
    float4* vel2;
    const int* start1;
    const int* start2;
    const int* n1;
    const int* n2;
    int nc, one;
    float K, ex;                  // sigma v_rel = K (v_rel^2)^ex, ex = 1 - omega
    float f1, f2;                 // m1 / (m1 + m2), m2 / (m1 + m2)
    double half_coef;             // 0.5 mpw0 dt / dV
    float* svmax;                 // (sigma v)_max read by the kernel, updated by the finishing launch
    unsigned* svmax_step;         // largest candidate sigma v of the call (float bits, atomicMax)
    unsigned long long* stats;    // [0] collisions, [1] candidate pairs, [2] collisions of the call
    uint2 key;                    // Philox key (seed)
    unsigned call, tag;           // counter words: the call number and the interaction's tag
};
void launch_dsmc(const DsmcArgs& a, cudaStream_t s);
void launch_sums(SpeciesDev sp, double* out, cudaStream_t s, int grid);
void launch_sample_moments(const GridDev& g, SpeciesDev sp, float* mom, cudaStream_t s, int grid);
void launch_merge(const GridDev& g, SpeciesDev sp, const float4* ef, const int* cell_start, int* list, int* nlist,
                  int min_count, float qm_half_dt, uint2 key, unsigned step, unsigned* err,
                  unsigned long long* stats, cudaStream_t s, int grid);

// fields
struct FinalizeArgs {
    GridDev g;
    int ns;
    const unsigned long long* acc[kMaxSpecies];
    float inv_scale[kMaxSpecies];
    float charge[kMaxSpecies];
    float* den[kMaxSpecies];
    // integer path: every species shares one fixed-point scale and carries an integer number of
    // elementary charges, so rho = q_e * sum_s z_s acc_s is formed exactly in 64-bit integers
    int int_path;
    int z[kMaxSpecies];
    float rho_scale;  // q_e / scale
    float* rho;
};
void launch_finalize_rho(const FinalizeArgs& a, cudaStream_t s, int grid);
void launch_efield(const GridDev& g, const float2* phi, float4* ef, cudaStream_t s, int grid);
// per-block partials of sum |E|^2 f over the distinct nodes, f the node's volume in cells
void launch_field_energy(const GridDev& g, const float4* ef, double* part, cudaStream_t s, int grid);
void launch_kinds(const GridDev& g, uint8_t* kind, cudaStream_t s);

struct SolveWork {
    float2* phi;      // master potential, float-float (FIXED nodes hold their values)
    float2* phi_alt;  // ping-pong partner
    const float* rho;
    const uint8_t* kind;
    float* r;         // FP32 residual / right-hand side of the correction equation
    float* e;         // FP32 correction
    float* d;         // CG direction
    float* q;         // CG L d
    float* z;         // CG preconditioned residual
    double* part;     // per-block partial sums [kParts * nslots]
    double* scal;     // device scalars (slots below)
    int* flag;        // [0] inner converged, [1] iterations completed
    double* gpart;    // node-kernel block partials [8][gstride]
    int gstride;
    unsigned* ticket; // last-block counter of the node-kernel reductions
};
constexpr int kParts = 1024;
// Node kernels take a tile of kNodeTile consecutive nodes per block, kNodeTile / blockDim.x per
// thread, strided by blockDim.x so that every load is coalesced and a thread's loads are
// independent of each other.
constexpr int kNodeThreads = 256;
constexpr int kNodeTile = 4 * kNodeThreads;
inline int node_blocks(int nv) { return (nv + kNodeTile - 1) / kNodeTile; }
// streaming node kernels (four consecutive nodes per thread and 16-byte loads, grid-stride): a
// few CTAs per SM keep every SM busy, and the grid sum adds few partials
inline int stream_blocks(int nv, int cap = 1216) {
    const int want = (nv / 4 + 255) / 256;
    return want < 1 ? 1 : (want < cap ? want : cap);
}
inline int stream_blocks(const GridDev& g) { return stream_blocks(g.nv, g.node_grid > 0 ? g.node_grid : 1216); }
// the CG stencil kernels wait on five neighbour rows per group of four nodes: they want more warps
// in flight than the streaming kernels, so their CTA count is tuned on its own
inline int cg_blocks(const GridDev& g) { return g.cg_grid > 0 ? stream_blocks(g.nv, g.cg_grid) : stream_blocks(g); }
// device scalar slots of the solvers
enum : int {
    kS_RZ = 0,      // [0..1] r.z of iterations it (double-buffered by parity)
    kS_ALPHA = 2,   // [2..3] alpha (learned preconditioner CG)
    kS_DQ = 4,      // d.q
    kS_RZN = 5,     // new r.z (Jacobi) / z.r (learned)
    kS_RZO = 6,     // r_new.z_old (Jacobi) / z.q (learned)
    kS_RR = 7,      // r.r
    kS_R2 = 8,      // residual |r|^2, |b|^2 at 8, 9
    kS_T2 = 10,     // |(rho - rho_prev) / eps0|^2 of the last FP32 residual update
    kS_S2 = 11,     // |rho / eps0|^2 over the FREE nodes (the space-charge part of b)
    kS_VAL = 12,    // validation norm
};
// residual (optionally after phi += e); |r|^2, |b|^2 and |rho/eps0|^2 into scal[kS_R2], [kS_R2 + 1],
// [kS_S2] (scal[kS_T2] is set to 0)
void launch_residual(const GridDev& g, SolveWork& w, int apply_e, cudaStream_t s, float* rho_prev, float* bfix_out);
void launch_rhs_update(const GridDev& g, SolveWork& w, float* rho_prev, const float* bfix, cudaStream_t s);
void launch_reduce_partials(const double* part, int nslots, int nblocks, double* out, cudaStream_t s);
void launch_rbsor_sweeps(const GridDev& g, SolveWork& w, float omega, int sweeps, cudaStream_t s);
void launch_pcg_init(const GridDev& g, SolveWork& w, cudaStream_t s);
void launch_pcg_iter_impl(const GridDev& g, SolveWork& w, float* d_in, float* d_out, int it, double target_rr,
                          cudaStream_t s);
// phi[dst] = phi[src] for the MIRROR pairs (first n_mirror entries), then the ALIAS pairs
void launch_fill_aux(const int2* pairs, int n_mirror, int n_alias, float2* phi, cudaStream_t s);
void launch_den_avg(float* avg, const float* den, int nv, float a, float b, cudaStream_t s, int grid);
// dst += src (n floats; both 16-byte aligned)
void launch_add(float* dst, const float* src, int n, cudaStream_t s, int grid);

}  // namespace pic
