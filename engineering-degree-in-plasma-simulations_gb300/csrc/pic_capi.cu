// C ABI and host-side orchestration of the GB300 PIC + DSMC library.
//
// One pic_world = the reference World with its fields plus the species, solver and collision
// model that the reference keeps in main.cpp (ch4/v3/src/main.cpp:71-139).  All device work
// is issued on the world's own stream; only calls that hand data back to the host, and the
// solver's convergence checks, synchronise it.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>
#include "../../include/pic_gb300.h"
#include "pic_kernels.h"
#include "pic_learned.h"
#include "pic_ff.cuh"
#include "pic_stencil.cuh"

using namespace pic;

constexpr double kFp32Unit = 0x1p-24;  // unit roundoff of FP32 round-to-nearest
constexpr long kUploadChunk = 1l << 22;  // particles per upload staging round (256 MB)
constexpr long kSortMovedFraction = 50;   // re-sort a species when 2 % of it left cell order

namespace {

thread_local char g_err[512] = "";

int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

#define CU(call)                                                                                   \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess) return fail(PIC_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

constexpr double kQe = 1.602176565e-19;  // ch4/v3/src/all.h:17
constexpr double kMe = 9.10938215e-31;
constexpr double kKb = 1.380648e-23;
constexpr double kPiRef = 3.141592653;  // Const::pi, ch4/v3/src/all.h:20

struct SpeciesHost {
    std::string name;
    double mass = 0, charge = 0, mpw0 = 0;
    long capacity = 0;
    SpeciesDev dev{};
    float4* pos2 = nullptr;
    float4* vel2 = nullptr;
    unsigned long long* id2 = nullptr;
    float* den = nullptr;
    float* den_avg = nullptr;
    float* mom = nullptr;  // velocity moments, 7 node planes, allocated on first sampleMoments
    int avg_samples = 0;
    double scale = 1.0;  // fixed-point scale of the density accumulator
    unsigned long long next_id = 0;
    bool deposited = false;
    // object interaction of a push (0: absorbed, as Species::advanceElectrons; 1: the
    // reference's advanceNonElectron(neutrals, spherium): neutrals bounce, ions are neutralised)
    int obj_mode = 0;
    int obj_neu = -1, obj_spu = -1, obj_sputtering = 0;
    uint2 obj_key{0, 0};
    unsigned long long* obj_stats = nullptr;  // hits, bounces, neutrals created, sputtered created
};

struct TimerAcc {
    double ms = 0;
    long launches = 0;
};
struct PendingEvent {
    std::string name;
    cudaEvent_t a, b;
};

}  // namespace

struct pic_world {
    int device = 0;
    int sms = 152;
    cudaStream_t stream = nullptr;
    cudaStream_t upload_stream = nullptr;  // uploads of a batch (pic_species_add_particles_batch)
    GridDev g{};
    // node fields
    float4* ef = nullptr;
    float2* phi = nullptr;  // potential as float-float (hi, lo) pairs
    float2* phi_alt = nullptr;
    float* rho = nullptr;
    uint16_t* kind = nullptr;
    unsigned* free_bits = nullptr;  // FREE nodes, one bit each (GridDev::free_bits)
    float *r = nullptr, *e = nullptr, *d = nullptr, *d2 = nullptr, *q = nullptr, *z = nullptr;
    double* part = nullptr;
    double* gpart = nullptr;     // block partials of the node-kernel reductions [8][gstride]
    int gstride = 0;
    unsigned* ticket = nullptr;  // last-block counter of those reductions
    double* scal = nullptr;
    int* flag = nullptr;
    double* h_scal = nullptr;  // pinned
    int* h_flag = nullptr;     // pinned
    // cells
    int* cell_count = nullptr;
    int* cell_start = nullptr;
    int* scan_aux = nullptr;
    int* merge_list = nullptr;  // candidate cells of a merge (num_cells + 1 ints)
    unsigned long long* merge_stats = nullptr;
    unsigned* err = nullptr;
    std::vector<SpeciesHost> sp;
    // boundaries
    int periodic[3] = {0, 0, 0};
    int face_mode[6] = {0, 0, 0, 0, 0, 0};
    double face_phi[6] = {0, 0, 0, 0, 0, 0};
    struct Box {
        double c[3], s[3], phi;
    };
    std::vector<Box> boxes;
    // beam sources (ColdBeamSource / WarmBeamSource, Source.h:13-68)
    struct Source {
        int sp, face;
        double v_drift, den, T;
        uint2 key;
    };
    std::vector<Source> sources;
    // particle-particle collisions (DSMC_MEX, Interactions.h:42-66), applied in list order
    struct Dsmc {
        int sp1, sp2;                  // sp2 == sp1: one species
        DsmcArgs a;                    // constants, state pointers; species pointers set per call
        int* start1 = nullptr;         // cell starts of the first species (two species only)
        unsigned long long* state = nullptr;  // stats[3], then svmax and svmax_step (32 bytes)
        double mpw0 = 0, dv = 0;
        unsigned calls = 0;
    };
    std::vector<Dsmc> dsmc;
    // stacked independent instances along z (0: one instance): electrode potentials per slab,
    // neutral density per slab and the candidate probabilities derived from it
    int nslabs = 0;
    std::vector<double> slab_lo, slab_hi, slab_n;
    unsigned* cand_slab = nullptr;  // candidate thresholds per slab
    double cand_slab_dt = -1.0;
    int* mcc_cand = nullptr;   // collision candidates of a step (electron capacity)
    int* mcc_ncand = nullptr;
    // time
    double dt = 1e-4;
    int num_ts = 0;
    int ts = -1;
    double time = 0.0;
    double* upload_buf = nullptr;  // particle upload staging (upload_cap particles, at most kUploadChunk)
    long upload_cap = 0;
    // bound on the 2-norm of the rounding error of the FP32 residual r (valid with rhs_valid)
    double r_err = 0.0;
    // solver
    int method = PIC_SOLVER_PCG;
    double tol = 1e-6;
    int stop_rule = PIC_STOP_REL_RHS;
    int warm_mode = PIC_WARM_PREVIOUS;  // start of a warm solve (PIC_WARM_*)
    int warm_jacobi = 16;  // Jacobi-PCG iterations a warm solve of the learned method runs first
    int lp_hint = 0;       // iterations of the last warm solve's converged first learned inner solve (0: none)
    float* dphi = nullptr;  // the last solve's total change of phi (FP32), for PIC_WARM_EXTRAPOLATE
    bool dphi_valid = false;  // dphi holds the change of one warm solve
    double last_norms[3] = {0, 0, 0};  // |r|, |b|, |rho/eps0| of the last solve's final residual
    int max_it = 10000;
    double omega = 1.4;
    long n_solves = 0, n_refine = 0, n_inner = 0;
    LpState* lp = nullptr;  // learned preconditioner, created on first use
    // r (FP32) holds the FP64 residual of phi for rho_prev; the next solve updates it by
    // (rho - rho_prev) / eps0 instead of an FP64 pass.  Cleared when phi, the boundaries or r change.
    float* rho_prev = nullptr;
    float* bfix = nullptr;  // FP32 boundary part of b per node
    int2* aux_pairs = nullptr;  // (node, source node) of the MIRROR, then the ALIAS nodes
    int n_mirror = 0, n_alias = 0;
    bool rhs_valid = false;
    int lp_collect = 0;     // store (first residual, total correction) of each solve as a training pair
    long lp_fallbacks = 0;  // learned solves handed to Jacobi-PCG
    uint64_t lp_seed = 0x1ea2d5eedull;
    // collisions
    bool mcc_on = false;
    int mcc_e = -1, mcc_i = -1;
    CollDev coll{};
    float* tE = nullptr;
    float* tS = nullptr;
    unsigned long long* stats = nullptr;
    double mcc_n = 0, mcc_sigv = 0;
    uint64_t mcc_seed = 0;
    // loop
    int solve_each_step = 1, sort_every = 20, merge_every = 0, merge_after = 0, merge_min = 10;
    int subcycle[kMaxSpecies] = {1, 1, 1, 1};
    // timing
    bool timing = false;
    std::map<std::string, TimerAcc> timers;
    std::vector<PendingEvent> pending;
    std::vector<cudaEvent_t> event_pool;
    long launches = 0;
    int grid_nodes = 1024;
    int grid_push_mcc = 304, grid_push = 456, grid_parts = 1216;
    long long wait_polls_arg = 0;  // PushArgs::wait_polls of this world's pushes (0: the default)
};

namespace {

cudaEvent_t get_event(pic_world* w) {
    if (!w->event_pool.empty()) {
        cudaEvent_t e = w->event_pool.back();
        w->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
}

// brackets a group of launches with CUDA events on the world's stream
struct Scope {
    pic_world* w;
    const char* name;
    cudaEvent_t a = nullptr;
    int n;
    Scope(pic_world* w_, const char* name_, int nlaunch) : w(w_), name(name_), n(nlaunch) {
        w->launches += nlaunch;
        if (w->timing) {
            a = get_event(w);
            cudaEventRecord(a, w->stream);
        }
        w->timers[name].launches += nlaunch;
    }
    ~Scope() {
        if (w->timing) {
            cudaEvent_t b = get_event(w);
            cudaEventRecord(b, w->stream);
            w->pending.push_back({name, a, b});
        }
    }
};

void collect_timers(pic_world* w) {
    if (w->pending.empty()) return;
    cudaStreamSynchronize(w->stream);
    for (auto& p : w->pending) {
        float ms = 0;
        cudaEventElapsedTime(&ms, p.a, p.b);
        w->timers[p.name].ms += ms;
        w->event_pool.push_back(p.a);
        w->event_pool.push_back(p.b);
    }
    w->pending.clear();
}

int check_device_error(pic_world* w) {
    unsigned h = 0;
    CU(cudaMemcpyAsync(&h, w->err, sizeof(unsigned), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    if (h) {
        CU(cudaMemsetAsync(w->err, 0, sizeof(unsigned), w->stream));
        if (h & kErrCapacity) return fail(PIC_ERR_CAPACITY, "a species ran out of capacity (device flags 0x%x)", h);
        return fail(PIC_ERR_DEVICE, "device fault flags 0x%x (bounded wait expired or merge truncated)", h);
    }
    return PIC_OK;
}

bool valid_sp(pic_world* w, int s) { return w && s >= 0 && s < (int)w->sp.size(); }

}  // namespace

namespace pic {
// records the message returned by pic_last_error for entry points in other translation units
int set_last_error(int code, const char* msg) { return fail(code, "%s", msg); }
}  // namespace pic

namespace {

// node kinds and masks; Dirichlet values written into phi_host
bool node_in_box(const pic_world::Box& b, const double x[3]) {  // Rectangle::inObject, Object.cpp:231-238
    for (int d = 0; d < 3; d++)
        if (std::fabs(x[d] - b.c[d]) > b.s[d] / 2) return false;
    return true;
}

void build_kinds(pic_world* w, std::vector<uint16_t>& kind, std::vector<double>& phi_host) {
    const GridDev& g = w->g;
    int nn[3] = {g.ni, g.nj, g.nk};
    kind.assign(g.nv, kFree);
    phi_host.assign(g.nv, 0.0);
    for (int k = 0; k < g.nk; k++)
        for (int j = 0; j < g.nj; j++)
            for (int i = 0; i < g.ni; i++) {
                int n = (k * g.nj + j) * g.ni + i, ijk[3] = {i, j, k};
                bool alias = false;
                for (int d = 0; d < 3; d++)
                    if (w->periodic[d] && ijk[d] == nn[d] - 1) alias = true;
                if (alias) {
                    kind[n] = kAlias;
                    continue;
                }
                double x[3] = {g.x0[0] + i * g.dxd[0], g.x0[1] + j * g.dxd[1], g.x0[2] + k * g.dxd[2]};
                bool in_box = false;
                for (auto& b : w->boxes)  // a later box overrides an earlier one (World.cpp:277-293)
                    if (node_in_box(b, x)) {
                        in_box = true;
                        phi_host[n] = b.phi;
                    }
                if (in_box) {
                    kind[n] = kFixed;
                    continue;
                }
                if (w->nslabs > 0) {
                    // instance slabs: their first and last node planes are electrodes
                    const int P = g.nk / w->nslabs, sl = k / P, lz = k - sl * P;
                    if (lz == 0 || lz == P - 1) {
                        kind[n] = kFixed;
                        phi_host[n] = lz == 0 ? w->slab_lo[sl] : w->slab_hi[sl];
                        continue;
                    }
                }
                int fixed_face = -1, wall = 0;
                for (int d = 0; d < 3; d++) {
                    if (w->periodic[d] || (d == 2 && w->nslabs > 0)) continue;
                    for (int s = 0; s < 2; s++) {
                        int f = 2 * d + s;
                        if ((s == 0 && ijk[d] == 0) || (s == 1 && ijk[d] == nn[d] - 1)) {
                            wall = 1;
                            if (w->face_mode[f] == 1 && fixed_face < 0) fixed_face = f;
                        }
                    }
                }
                if (fixed_face >= 0) {
                    kind[n] = kFixed;
                    phi_host[n] = w->face_phi[fixed_face];
                } else if (wall) {
                    kind[n] = kMirror;
                }
            }
    // neighbour masks of FREE nodes
    for (int k = 0; k < g.nk; k++)
        for (int j = 0; j < g.nj; j++)
            for (int i = 0; i < g.ni; i++) {
                int n = (k * g.nj + j) * g.ni + i;
                if ((kind[n] & 3) != kFree) continue;
                int ijk[3] = {i, j, k};
                uint16_t mask = 0;
                for (int d = 0; d < 3; d++)
                    for (int s = 0; s < 2; s++) {
                        int c = ijk[d] + (s ? 1 : -1);
                        if (w->periodic[d]) {
                            if (c < 0) c = nn[d] - 2;
                            else if (c >= nn[d] - 1) c = 0;
                        }
                        int q3[3] = {ijk[0], ijk[1], ijk[2]};
                        q3[d] = c;
                        int qn = (q3[2] * g.nj + q3[1]) * g.ni + q3[0];
                        int bit = 2 * d + s;
                        if ((kind[qn] & 3) == kMirror) mask |= 1u << (2 + bit);
                        if ((kind[qn] & 3) == kFixed) mask |= 1u << (8 + bit);
                    }
                kind[n] = (uint16_t)(kFree | mask);
            }
}

int upload_kinds(pic_world* w, bool reset_phi) {
    w->rhs_valid = false;
    std::vector<uint16_t> kind;
    std::vector<double> ph;
    build_kinds(w, kind, ph);
    const GridDev& g = w->g;
    {
        // copy lists of the MIRROR nodes (clamped interior node) and the ALIAS nodes (periodic source)
        std::vector<int2> mir, ali;
        const int nn[3] = {g.ni, g.nj, g.nk};
        for (int k = 0; k < g.nk; k++)
            for (int j = 0; j < g.nj; j++)
                for (int i = 0; i < g.ni; i++) {
                    const int n = (k * g.nj + j) * g.ni + i, kd = kind[n] & 3;
                    if (kd != kMirror && kd != kAlias) continue;
                    int ijk[3] = {i, j, k};
                    for (int d = 0; d < 3; d++) {
                        if (kd == kMirror && !w->periodic[d])
                            ijk[d] = ijk[d] < 1 ? 1 : (ijk[d] > nn[d] - 2 ? nn[d] - 2 : ijk[d]);
                        if (kd == kAlias && w->periodic[d] && ijk[d] == nn[d] - 1) ijk[d] = 0;
                    }
                    (kd == kMirror ? mir : ali).push_back(make_int2(n, (ijk[2] * g.nj + ijk[1]) * g.ni + ijk[0]));
                }
        if (w->aux_pairs) cudaFree(w->aux_pairs);
        w->aux_pairs = nullptr;
        w->n_mirror = (int)mir.size();
        w->n_alias = (int)ali.size();
        mir.insert(mir.end(), ali.begin(), ali.end());
        if (!mir.empty()) {
            CU(cudaMalloc(&w->aux_pairs, sizeof(int2) * mir.size()));
            CU(cudaMemcpy(w->aux_pairs, mir.data(), sizeof(int2) * mir.size(), cudaMemcpyHostToDevice));
        }
    }
    CU(cudaMemcpyAsync(w->kind, kind.data(), sizeof(uint16_t) * g.nv, cudaMemcpyHostToDevice, w->stream));
    {
        // the FREE nodes as a bit mask, rows padded to whole 32-bit words
        const int wpr = (g.ni + 31) / 32;
        std::vector<unsigned> bits((size_t)wpr * g.nj * g.nk, 0u);
        for (int r = 0; r < g.nj * g.nk; r++)
            for (int i = 0; i < g.ni; i++)
                if ((kind[(size_t)r * g.ni + i] & 3) == kFree) bits[(size_t)r * wpr + (i >> 5)] |= 1u << (i & 31);
        if (!w->free_bits) CU(cudaMalloc((void**)&w->free_bits, sizeof(unsigned) * bits.size()));
        CU(cudaMemcpy(w->free_bits, bits.data(), sizeof(unsigned) * bits.size(), cudaMemcpyHostToDevice));
        w->g.free_bits = w->free_bits;
        w->g.free_wpr = wpr;
    }
    std::vector<float2> cur(g.nv);
    if (reset_phi) {
        for (int n = 0; n < g.nv; n++) cur[n] = ff_pack(ph[n]);
    } else {
        // keep the caller's phi but force Dirichlet values
        CU(cudaMemcpyAsync(cur.data(), w->phi, sizeof(float2) * g.nv, cudaMemcpyDeviceToHost, w->stream));
        CU(cudaStreamSynchronize(w->stream));
        for (int n = 0; n < g.nv; n++)
            if ((kind[n] & 3) == kFixed) cur[n] = ff_pack(ph[n]);
    }
    CU(cudaMemcpyAsync(w->phi, cur.data(), sizeof(float2) * g.nv, cudaMemcpyHostToDevice, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    return PIC_OK;
}

void fill_grid_boxes(pic_world* w) {
    GridDev& g = w->g;
    g.n_boxes = 0;
    for (auto& b : w->boxes) {
        if (g.n_boxes >= kMaxBoxes) break;
        for (int d = 0; d < 3; d++) {
            g.box_lo[g.n_boxes][d] = (float)(b.c[d] - b.s[d] / 2 - g.x0[d]);
            g.box_hi[g.n_boxes][d] = (float)(b.c[d] + b.s[d] / 2 - g.x0[d]);
        }
        g.n_boxes++;
    }
    for (int d = 0; d < 3; d++) g.periodic[d] = w->periodic[d];
}

// candidate threshold of probability p on the 32-bit candidate draw: candidate iff draw < T,
// probability T / 2^32 (within 2^-32 of p)
unsigned cand_threshold(double p) {
    if (!(p > 0.0)) return 0u;
    if (p >= 1.0) return 0xFFFFFFFFu;
    return (unsigned)(p * 4294967296.0);
}
// candidate thresholds of the collision model for a step of dt: the world's, or per instance slab
// from n_s (sigma v)_max dt (uploaded when dt changes) with the largest as the first-pass bound
int candidate_thresholds(pic_world* w, double dt, CollDev& c) {
    c.cand_slab = nullptr;
    c.cand_max = cand_threshold(w->mcc_n * w->mcc_sigv * dt);
    if (w->slab_n.empty()) return PIC_OK;
    std::vector<unsigned> th(w->slab_n.size());
    for (size_t q = 0; q < th.size(); q++) th[q] = cand_threshold(w->slab_n[q] * w->mcc_sigv * dt);
    if (w->cand_slab_dt != dt) {
        CU(cudaMemcpyAsync(w->cand_slab, th.data(), sizeof(unsigned) * th.size(), cudaMemcpyHostToDevice, w->stream));
        CU(cudaStreamSynchronize(w->stream));
        w->cand_slab_dt = dt;
    }
    c.cand_max = *std::max_element(th.begin(), th.end());
    c.cand_slab = w->cand_slab;
    return PIC_OK;
}

void free_lp(pic_world* w) {
    if (!w->lp) return;
    LpState* L = w->lp;
    for (int l = 1; l < kLpMaxLevels; l++) {
        if (L->z[l]) cudaFree(L->z[l]);
        if (L->e[l]) cudaFree(L->e[l]);
    }
    if (L->W) cudaFree(L->W);
    if (L->fold) cudaFree(L->fold);
    lp_free_train(*L);
    delete L;
    w->lp = nullptr;
}

// the learned preconditioner of the world's current grid and periodic axes (created on first use,
// weights at their multilevel-diagonal start)
int ensure_lp(pic_world* w) {
    const GridDev& g = w->g;
    if (w->lp && w->lp->per[0] == w->periodic[0] && w->lp->per[1] == w->periodic[1] &&
        w->lp->per[2] == w->periodic[2])
        return PIC_OK;
    free_lp(w);
    int n0[3] = {g.ni - w->periodic[0], g.nj - w->periodic[1], g.nk - w->periodic[2]};
    if (std::min(n0[0], std::min(n0[1], n0[2])) < 2)
        return fail(PIC_ERR_ARG, "the learned preconditioner needs at least 2 distinct nodes per axis");
    LpState* L = new LpState();
    w->lp = L;
    for (int d = 0; d < 3; d++) {
        L->per[d] = w->periodic[d];
        L->dims[0][d] = n0[d];
    }
    L->nlev = 1;
    while (L->nlev < kLpMaxLevels) {
        int nx[3];
        for (int d = 0; d < 3; d++) nx[d] = (L->dims[L->nlev - 1][d] + 1) / 2;
        if (std::min(nx[0], std::min(nx[1], nx[2])) < 2) break;
        if (nx[0] == L->dims[L->nlev - 1][0] && nx[1] == L->dims[L->nlev - 1][1] && nx[2] == L->dims[L->nlev - 1][2])
            break;
        for (int d = 0; d < 3; d++) L->dims[L->nlev][d] = nx[d];
        L->nlev++;
    }
    for (int l = 1; l < L->nlev; l++) {
        size_t nvox = (size_t)L->dims[l][0] * L->dims[l][1] * L->dims[l][2];
        CU(cudaMalloc(&L->z[l], sizeof(float) * nvox));
        CU(cudaMalloc(&L->e[l], sizeof(float) * nvox));
    }
    double c[3] = {1.0 / (g.dxd[0] * g.dxd[0]), 1.0 / (g.dxd[1] * g.dxd[1]), 1.0 / (g.dxd[2] * g.dxd[2])};
    lp_galerkin_diag(c, L->nlev, L->diag);
    lp_layout(L->lay);
    CU(cudaMalloc(&L->W, sizeof(float) * L->lay.total));
    CU(cudaMalloc(&L->fold, sizeof(float) * kLpFoldStride * kLpNetLevels));
    std::vector<float> hw(L->lay.total);
    lp_init_weights(L->lay, L->diag, L->nlev, hw.data());
    CU(cudaMemcpyAsync(L->W, hw.data(), sizeof(float) * hw.size(), cudaMemcpyHostToDevice, w->stream));
    launch_lp_fold(*L, w->stream);
    CU(cudaStreamSynchronize(w->stream));
    CU(cudaGetLastError());
    return PIC_OK;
}

int ensure_lp_train(pic_world* w) {
    int rc = ensure_lp(w);
    if (rc) return rc;
    if (w->lp->train) return PIC_OK;
    std::vector<float> hw(w->lp->lay.total);
    CU(cudaMemcpyAsync(hw.data(), w->lp->W, sizeof(float) * hw.size(), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    if (lp_alloc_train(w->g, *w->lp, hw.data())) {
        cudaGetLastError();
        free_lp(w);
        return fail(PIC_ERR_CUDA, "device allocation failed for the preconditioner training state");
    }
    launch_lp_prep(*w->lp, w->stream);
    CU(cudaStreamSynchronize(w->stream));
    return PIC_OK;
}

SolveWork solve_work(pic_world* w) {
    SolveWork s;
    s.phi = w->phi;
    s.phi_alt = w->phi_alt;
    s.rho = w->rho;
    s.kind = reinterpret_cast<const uint8_t*>(w->kind);
    s.r = w->r;
    s.e = w->e;
    s.d = w->d;
    s.q = w->q;
    s.z = w->z;
    s.part = w->part;
    s.scal = w->scal;
    s.flag = w->flag;
    s.gpart = w->gpart;
    s.gstride = w->gstride;
    s.ticket = w->ticket;
    return s;
}

}  // namespace


// =====================================================================================
// World
// =====================================================================================
extern "C" int pic_world_create(pic_world** out, int ni, int nj, int nk, const double* x0, const double* xm,
                                int device) {
    if (!out || !x0 || !xm) return fail(PIC_ERR_ARG, "null argument");
    *out = nullptr;
    if (ni < 2 || nj < 2 || nk < 2) return fail(PIC_ERR_ARG, "need at least 2 nodes per axis");
    // particles store their cell packed as i | j << 9 | k << 18
    if (ni - 1 > kCellMaxIJ || nj - 1 > kCellMaxIJ || nk - 1 > kCellMaxK)
        return fail(PIC_ERR_ARG, "at most %d x %d x %d cells", kCellMaxIJ, kCellMaxIJ, kCellMaxK);
    long long nv = (long long)ni * nj * nk;
    if (nv > (1ll << 30)) return fail(PIC_ERR_ARG, "grid too large (%lld nodes)", nv);
    for (int d = 0; d < 3; d++)
        if (!(xm[d] > x0[d])) return fail(PIC_ERR_ARG, "xm must exceed x0 on every axis");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= device || device < 0)
        return fail(PIC_ERR_CUDA, "no CUDA device %d available", device);
    CU(cudaSetDevice(device));
    pic_world* w = new pic_world();
    w->device = device;
    cudaDeviceGetAttribute(&w->sms, cudaDevAttrMultiProcessorCount, device);
    GridDev& g = w->g;
    g.ni = ni;
    g.nj = nj;
    g.nk = nk;
    g.ci = ni - 1;
    g.cj = nj - 1;
    g.ck = nk - 1;
    g.nv = (int)nv;
    g.nc = g.ci * g.cj * g.ck;
    g.fd_ni = make_fastdiv((unsigned)ni);
    g.fd_nj = make_fastdiv((unsigned)nj);
    int nn[3] = {ni, nj, nk};
    for (int d = 0; d < 3; d++) {
        g.x0[d] = x0[d];
        g.xm[d] = xm[d];
        g.dxd[d] = (xm[d] - x0[d]) / (nn[d] - 1);  // World::setExtents, World.cpp:72-76
        g.dx[d] = (float)g.dxd[d];
        g.inv_dx[d] = (float)(1.0 / g.dxd[d]);
        const double c = 1.0 / (g.dxd[d] * g.dxd[d]);
        g.c_hi[d] = (float)c;
        g.c_lo[d] = (float)(c - (double)g.c_hi[d]);
        g.inv2dx[d] = (float)(1.0 / (2.0 * g.dxd[d]));
    }
    g.inv_cell_vol = (float)(1.0 / (g.dxd[0] * g.dxd[1] * g.dxd[2]));
    auto alloc = [&](void** p, size_t bytes) -> bool { return cudaMalloc(p, bytes) == cudaSuccess; };
    bool ok = cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && alloc((void**)&w->ef, sizeof(float4) * nv) && alloc((void**)&w->phi, sizeof(float2) * nv) &&
         alloc((void**)&w->phi_alt, sizeof(float2) * nv) && alloc((void**)&w->rho, sizeof(float) * nv) &&
         alloc((void**)&w->kind, sizeof(uint16_t) * nv) && alloc((void**)&w->r, sizeof(float) * nv) &&
         alloc((void**)&w->e, sizeof(float) * nv) && alloc((void**)&w->d, sizeof(float) * nv) &&
         alloc((void**)&w->d2, sizeof(float) * nv) && alloc((void**)&w->q, sizeof(float) * nv) &&
         alloc((void**)&w->z, sizeof(float) * nv) && alloc((void**)&w->part, sizeof(double) * kParts * 8) &&
         alloc((void**)&w->scal, sizeof(double) * 16) && alloc((void**)&w->flag, sizeof(int) * 4) &&
         alloc((void**)&w->gpart, sizeof(double) * 8 * (size_t)std::max(kParts, 2 * node_blocks(nv))) &&
         alloc((void**)&w->ticket, sizeof(unsigned) * 4) &&
         alloc((void**)&w->cell_count, sizeof(int) * (g.nc + 1)) &&
         alloc((void**)&w->cell_start, sizeof(int) * (g.nc + 1)) &&
         alloc((void**)&w->scan_aux, sizeof(int) * (g.nc / 2048 + 2)) && alloc((void**)&w->err, sizeof(unsigned)) &&
         cudaMallocHost((void**)&w->h_scal, sizeof(double) * 16) == cudaSuccess &&
         cudaMallocHost((void**)&w->h_flag, sizeof(int) * 4) == cudaSuccess;
    if (!ok) {
        pic_world_destroy(w);
        return fail(PIC_ERR_CUDA, "device allocation failed for a %d x %d x %d grid", ni, nj, nk);
    }
    cudaMemsetAsync(w->ef, 0, sizeof(float4) * nv, w->stream);
    cudaMemsetAsync(w->rho, 0, sizeof(float) * nv, w->stream);
    for (float* p : {w->r, w->e, w->d, w->d2, w->q, w->z}) cudaMemsetAsync(p, 0, sizeof(float) * nv, w->stream);
    cudaMemsetAsync(w->err, 0, sizeof(unsigned), w->stream);
    cudaMemsetAsync(w->flag, 0, sizeof(int) * 4, w->stream);
    cudaMemsetAsync(w->ticket, 0, sizeof(unsigned) * 4, w->stream);
    w->gstride = std::max(kParts, 2 * node_blocks(nv));
    w->grid_nodes = (int)std::min<long long>(kParts, std::max<long long>(1, (nv + 255) / 256));
    w->grid_parts = w->sms * 8;
    w->grid_push = w->sms * push_blocks_per_sm();
    w->grid_push_mcc = w->sms * 2;
    fill_grid_boxes(w);
    int rc = upload_kinds(w, true);
    if (rc != PIC_OK) {
        pic_world_destroy(w);
        return rc;
    }
    *out = w;
    return PIC_OK;
}

extern "C" int pic_world_destroy(pic_world* w) {
    if (!w) return PIC_OK;
    cudaSetDevice(w->device);
    if (w->stream) cudaStreamSynchronize(w->stream);
    free_lp(w);
    if (w->rho_prev) cudaFree(w->rho_prev);
    if (w->dphi) cudaFree(w->dphi);
    if (w->free_bits) cudaFree(w->free_bits);
    if (w->aux_pairs) cudaFree(w->aux_pairs);
    if (w->cand_slab) cudaFree(w->cand_slab);
    if (w->mcc_cand) cudaFree(w->mcc_cand);
    if (w->mcc_ncand) cudaFree(w->mcc_ncand);
    if (w->bfix) cudaFree(w->bfix);
    for (auto& d : w->dsmc) {
        if (d.start1) cudaFree(d.start1);
        if (d.state) cudaFree(d.state);
    }
    for (auto& s : w->sp) {
        cudaFree(s.dev.pos);
        cudaFree(s.dev.vel);
        cudaFree(s.dev.id);
        cudaFree(s.dev.counts);
        cudaFree(s.dev.dead);
        cudaFree(s.dev.holes);
        cudaFree(s.dev.acc);
        cudaFree(s.pos2);
        cudaFree(s.vel2);
        cudaFree(s.id2);
        cudaFree(s.den);
        cudaFree(s.den_avg);
        if (s.mom) cudaFree(s.mom);
        if (s.obj_stats) cudaFree(s.obj_stats);
    }
    void* ptrs[] = {w->ef,   w->phi,  w->phi_alt, w->rho,        w->kind,       w->r,        w->e,
                    w->d,    w->d2,   w->q,       w->z,          w->part,       w->scal,     w->flag,
                    w->gpart, w->ticket,
                    w->cell_count,    w->cell_start,             w->scan_aux,   w->err,      w->tE,
                    w->tS,   w->stats,  w->merge_list, w->merge_stats};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (w->h_scal) cudaFreeHost(w->h_scal);
    if (w->upload_buf) cudaFree(w->upload_buf);
    if (w->h_flag) cudaFreeHost(w->h_flag);
    for (auto& p : w->pending) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    for (auto e : w->event_pool) cudaEventDestroy(e);
    if (w->stream) cudaStreamDestroy(w->stream);
    if (w->upload_stream) cudaStreamDestroy(w->upload_stream);
    delete w;
    return PIC_OK;
}

extern "C" int pic_world_set_time(pic_world* w, double dt, int num_ts) {
    if (!w || !(dt > 0)) return fail(PIC_ERR_ARG, "dt must be positive");
    w->dt = dt;
    w->num_ts = num_ts;
    return PIC_OK;
}
extern "C" int pic_world_advance_time(pic_world* w, int* running) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    w->time += w->dt;
    w->ts++;
    if (running) *running = w->ts <= w->num_ts;
    return PIC_OK;
}
extern "C" int pic_world_get_time(pic_world* w, double* time) {
    if (!w || !time) return fail(PIC_ERR_ARG, "null argument");
    *time = w->time;
    return PIC_OK;
}
extern "C" int pic_world_get_ts(pic_world* w, int* ts) {
    if (!w || !ts) return fail(PIC_ERR_ARG, "null argument");
    *ts = w->ts;
    return PIC_OK;
}
extern "C" int pic_world_set_boundaries(pic_world* w, const int* periodic, const int* face_mode,
                                        const double* face_phi) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    CU(cudaSetDevice(w->device));
    for (int d = 0; d < 3; d++) w->periodic[d] = periodic ? (periodic[d] != 0) : 0;
    for (int f = 0; f < 6; f++) {
        w->face_mode[f] = face_mode ? face_mode[f] : 0;
        w->face_phi[f] = face_phi ? face_phi[f] : 0.0;
    }
    int nn[3] = {w->g.ni, w->g.nj, w->g.nk};
    for (int d = 0; d < 3; d++)
        if (w->periodic[d] && nn[d] < 4) return fail(PIC_ERR_ARG, "periodic axis needs at least 4 nodes");
    fill_grid_boxes(w);
    return upload_kinds(w, false);
}
extern "C" int pic_world_add_box(pic_world* w, const double* center, const double* sides, double phi) {
    if (!w || !center || !sides) return fail(PIC_ERR_ARG, "null argument");
    if ((int)w->boxes.size() >= kMaxBoxes) return fail(PIC_ERR_ARG, "at most %d boxes", kMaxBoxes);
    CU(cudaSetDevice(w->device));
    pic_world::Box b;
    for (int d = 0; d < 3; d++) {
        b.c[d] = center[d];
        b.s[d] = sides[d];
    }
    b.phi = phi;
    w->boxes.push_back(b);
    fill_grid_boxes(w);
    return upload_kinds(w, false);
}

extern "C" int pic_world_set_slabs(pic_world* w, int nslabs, const double* phi_lo, const double* phi_hi) {
    if (!w || nslabs < 0 || (nslabs > 0 && (!phi_lo || !phi_hi))) return fail(PIC_ERR_ARG, "bad arguments");
    CU(cudaSetDevice(w->device));
    GridDev& g = w->g;
    if (nslabs > 0) {
        if (w->periodic[2]) return fail(PIC_ERR_ARG, "instance slabs need a non-periodic z axis");
        if (g.nk % nslabs || g.nk / nslabs < 3)
            return fail(PIC_ERR_ARG, "%d z nodes do not split into %d slabs of at least 3 nodes", g.nk, nslabs);
    }
    w->nslabs = nslabs;
    w->slab_lo.assign(phi_lo, phi_lo + nslabs);
    w->slab_hi.assign(phi_hi, phi_hi + nslabs);
    g.zslab = nslabs > 0 ? g.nk / nslabs : 0;
    g.fd_zslab = make_fastdiv((unsigned)(g.zslab > 1 ? g.zslab : 2));
    if (w->lp) free_lp(w);
    return upload_kinds(w, false);
}

extern "C" int pic_world_get_field(pic_world* w, int which, double* out) {
    if (!w || !out) return fail(PIC_ERR_ARG, "null argument");
    CU(cudaSetDevice(w->device));
    const GridDev& g = w->g;
    if (which == 0) {
        std::vector<float2> t(g.nv);
        CU(cudaMemcpyAsync(t.data(), w->phi, sizeof(float2) * g.nv, cudaMemcpyDeviceToHost, w->stream));
        CU(cudaStreamSynchronize(w->stream));
        for (int n = 0; n < g.nv; n++) out[n] = ff_to_double(t[n]);
    } else if (which == 1) {
        std::vector<float> t(g.nv);
        CU(cudaMemcpyAsync(t.data(), w->rho, sizeof(float) * g.nv, cudaMemcpyDeviceToHost, w->stream));
        CU(cudaStreamSynchronize(w->stream));
        for (int n = 0; n < g.nv; n++) out[n] = t[n];
    } else if (which == 2) {
        // World::computeNodeVolumes: half a cell per non-periodic face (of each stacked instance)
        const int nn[3] = {g.ni, g.nj, g.zslab ? g.zslab : g.nk};
        for (int k = 0; k < g.nk; k++)
            for (int j = 0; j < g.nj; j++)
                for (int i = 0; i < g.ni; i++) {
                    int ijk[3] = {i, j, g.zslab ? k % g.zslab : k};
                    double v = g.dxd[0] * g.dxd[1] * g.dxd[2];
                    for (int d = 0; d < 3; d++)
                        if (!w->periodic[d] && (ijk[d] == 0 || ijk[d] == nn[d] - 1)) v *= 0.5;
                    out[(k * g.nj + j) * g.ni + i] = v;
                }
    } else if (which == 4 || which == 5) {
        // node_type (World.h:17: REGULAR 0, NEUMANN 1, DIRICHLET 2) or object_id (1 inside an object)
        std::vector<uint16_t> kind;
        std::vector<double> ph;
        build_kinds(w, kind, ph);
        const int nn[3] = {g.ni, g.nj, g.nk};
        for (int k = 0; k < g.nk; k++)
            for (int j = 0; j < g.nj; j++)
                for (int i = 0; i < g.ni; i++) {
                    const int n = (k * g.nj + j) * g.ni + i;
                    if (which == 4) {
                        // the duplicate last plane of a periodic axis reports its source node
                        int ijk[3] = {i, j, k};
                        for (int d = 0; d < 3; d++)
                            if (w->periodic[d] && ijk[d] == nn[d] - 1) ijk[d] = 0;
                        const int kd = kind[(ijk[2] * g.nj + ijk[1]) * g.ni + ijk[0]] & 3;
                        out[n] = kd == kFixed ? 2.0 : kd == kMirror ? 1.0 : 0.0;
                        continue;
                    }
                    const double x[3] = {g.x0[0] + i * g.dxd[0], g.x0[1] + j * g.dxd[1], g.x0[2] + k * g.dxd[2]};
                    double id = 0.0;
                    for (auto& b : w->boxes)
                        if (node_in_box(b, x)) id = 1.0;
                    out[n] = id;
                }
    } else if (which == 3) {
        std::vector<float4> t(g.nv);
        CU(cudaMemcpyAsync(t.data(), w->ef, sizeof(float4) * g.nv, cudaMemcpyDeviceToHost, w->stream));
        CU(cudaStreamSynchronize(w->stream));
        for (int n = 0; n < g.nv; n++) {
            out[3 * n] = t[n].x;
            out[3 * n + 1] = t[n].y;
            out[3 * n + 2] = t[n].z;
        }
    } else {
        return fail(PIC_ERR_ARG, "unknown field %d", which);
    }
    return check_device_error(w);
}
extern "C" int pic_world_potential_energy(pic_world* w, double* pe) {
    if (!w || !pe) return fail(PIC_ERR_ARG, "null argument");
    CU(cudaSetDevice(w->device));
    const int grid = 512;
    {
        Scope sc(w, "diagnostics", 1);
        launch_field_energy(w->g, w->ef, w->part, w->stream, grid);
    }
    std::vector<double> h(grid);
    CU(cudaMemcpyAsync(h.data(), w->part, sizeof(double) * grid, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    double t = 0;
    for (int b = 0; b < grid; b++) t += h[b];
    const GridDev& g = w->g;
    *pe = 0.5 * kEps0 * g.dxd[0] * g.dxd[1] * g.dxd[2] * t;
    return check_device_error(w);
}
extern "C" int pic_world_set_field(pic_world* w, int which, const double* in) {
    if (!w || !in) return fail(PIC_ERR_ARG, "null argument");
    CU(cudaSetDevice(w->device));
    const GridDev& g = w->g;
    if (which == 0) {
        w->rhs_valid = false;
        std::vector<float2> t(g.nv);
        for (int n = 0; n < g.nv; n++) t[n] = ff_pack(in[n]);
        CU(cudaMemcpyAsync(w->phi, t.data(), sizeof(float2) * g.nv, cudaMemcpyHostToDevice, w->stream));
        CU(cudaStreamSynchronize(w->stream));
    } else if (which == 1) {
        std::vector<float> t(in, in + g.nv);
        CU(cudaMemcpyAsync(w->rho, t.data(), sizeof(float) * g.nv, cudaMemcpyHostToDevice, w->stream));
        CU(cudaStreamSynchronize(w->stream));
    } else if (which == 3) {
        std::vector<float4> t(g.nv);
        for (int n = 0; n < g.nv; n++) t[n] = make_float4((float)in[3 * n], (float)in[3 * n + 1], (float)in[3 * n + 2], 0.f);
        CU(cudaMemcpyAsync(w->ef, t.data(), sizeof(float4) * g.nv, cudaMemcpyHostToDevice, w->stream));
        CU(cudaStreamSynchronize(w->stream));
    } else {
        return fail(PIC_ERR_ARG, "field %d is not settable", which);
    }
    return PIC_OK;
}

// =====================================================================================
// Species
// =====================================================================================
extern "C" int pic_species_create(pic_world* w, const char* name, double mass, double charge, double mpw0,
                                  long capacity, double weight_bound, int* species_id) {
    if (!w || !species_id) return fail(PIC_ERR_ARG, "null argument");
    if ((int)w->sp.size() >= kMaxSpecies) return fail(PIC_ERR_ARG, "at most %d species", kMaxSpecies);
    if (!(mass > 0) || capacity <= 0 || capacity > (1l << 30)) return fail(PIC_ERR_ARG, "bad mass or capacity");
    CU(cudaSetDevice(w->device));
    SpeciesHost s;
    s.name = name ? name : "";
    s.mass = mass;
    s.charge = charge;
    s.mpw0 = mpw0;
    s.capacity = capacity;
    const GridDev& g = w->g;
    auto alloc = [&](void** p, size_t bytes) -> bool { return cudaMalloc(p, bytes) == cudaSuccess; };
    bool ok = alloc((void**)&s.dev.pos, sizeof(float4) * capacity) && alloc((void**)&s.dev.vel, sizeof(float4) * capacity) &&
              alloc((void**)&s.dev.id, sizeof(unsigned long long) * capacity) &&
              alloc((void**)&s.dev.counts, sizeof(int) * 8) && alloc((void**)&s.dev.dead, sizeof(int) * capacity) &&
              alloc((void**)&s.dev.holes, sizeof(int) * capacity) &&
              alloc((void**)&s.dev.acc, sizeof(unsigned long long) * g.nv) &&
              alloc((void**)&s.pos2, sizeof(float4) * capacity) && alloc((void**)&s.vel2, sizeof(float4) * capacity) &&
              alloc((void**)&s.id2, sizeof(unsigned long long) * capacity) && alloc((void**)&s.den, sizeof(float) * g.nv) &&
              alloc((void**)&s.den_avg, sizeof(float) * g.nv);
    if (!ok) {
        cudaFree(s.dev.pos); cudaFree(s.dev.vel); cudaFree(s.dev.id); cudaFree(s.dev.counts); cudaFree(s.dev.dead);
        cudaFree(s.dev.holes); cudaFree(s.dev.acc); cudaFree(s.pos2); cudaFree(s.vel2); cudaFree(s.id2);
        cudaFree(s.den); cudaFree(s.den_avg);
        return fail(PIC_ERR_CUDA, "device allocation failed for species %s (capacity %ld)", s.name.c_str(), capacity);
    }
    s.dev.capacity = (int)capacity;
    CU(cudaMemsetAsync(s.dev.counts, 0, sizeof(int) * 8, w->stream));
    CU(cudaMemsetAsync(s.dev.acc, 0, sizeof(unsigned long long) * g.nv, w->stream));
    CU(cudaMemsetAsync(s.den, 0, sizeof(float) * g.nv, w->stream));
    CU(cudaMemsetAsync(s.den_avg, 0, sizeof(float) * g.nv, w->stream));
    double bound = weight_bound > 0 ? weight_bound : (double)capacity * (mpw0 > 0 ? mpw0 : 1.0) * 64.0;
    // largest power of two keeping every node sum below 2^62
    int ex = (int)std::floor(std::log2(std::ldexp(1.0, 62) / bound));
    // a particle of the mean weight deposits at most 2^26 units (quantum 2^-26 of its weight), so
    // the push keeps typical particles on its 32-bit run-sum path and its tile rarely carries
    if (mpw0 > 0) ex = std::min(ex, (int)std::floor(std::log2(std::ldexp(1.0, 26) / mpw0)));
    if (ex > 60) ex = 60;
    if (ex < -60) ex = -60;
    s.scale = std::ldexp(1.0, ex);
    // one scale for all species (the smallest), so rho can be summed exactly in integers;
    // species are created before anything is deposited
    for (auto& o : w->sp) s.scale = std::min(s.scale, o.scale);
    for (auto& o : w->sp) o.scale = s.scale;
    w->sp.push_back(s);
    *species_id = (int)w->sp.size() - 1;
    return PIC_OK;
}

namespace {
// the particle upload staging buffer holds at least min(n, kUploadChunk) particles
int ensure_upload(pic_world* w, long n) {
    const long want = std::min<long>(kUploadChunk, n);
    if (w->upload_cap < want) {
        if (w->upload_buf) CU(cudaFree(w->upload_buf));
        w->upload_buf = nullptr;
        w->upload_cap = 0;
        CU(cudaMalloc(&w->upload_buf, (size_t)want * 8 * sizeof(double)));
        w->upload_cap = want;
    }
    return PIC_OK;
}
}  // namespace

// a pointer the world's device can dereference: its own device memory, or pinned host memory
// mapped into the unified address space (the kernel then reads it over the host link);
// nullptr for pageable memory
static const void* device_view(const pic_world* w, const void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type == cudaMemoryTypeHost) return at.devicePointer;
    if ((at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) && at.device == w->device)
        return at.devicePointer;
    return nullptr;
}

extern "C" int pic_species_add_particles(pic_world* w, int sp, const double* pos, const double* vel,
                                         const double* wgt, const uint64_t* ids, long n, int rewind) {
    if (!valid_sp(w, sp) || (n > 0 && (!pos || !vel || !wgt))) return fail(PIC_ERR_ARG, "bad species or arrays");
    if (n == 0) return PIC_OK;
    CU(cudaSetDevice(w->device));
    SpeciesHost& s = w->sp[sp];
    // arrays the device can read (pinned host or device memory): converted where they lie
    {
        const double* dp = static_cast<const double*>(device_view(w, pos));
        const double* dv = static_cast<const double*>(device_view(w, vel));
        const double* dw = static_cast<const double*>(device_view(w, wgt));
        const auto* di = static_cast<const unsigned long long*>(ids ? device_view(w, ids) : nullptr);
        if (dp && dv && dw && (!ids || di)) {
            const unsigned long long id0 = s.next_id;
            const long step = 1l << 30;
            for (long a = 0; a < n; a += step) {
                const long m = std::min<long>(step, n - a);
                Scope sc(w, "load", 5);
                launch_from_abs(w->g, s.dev, dp + 3 * a, dv + 3 * a, dw + a, di ? di + a : nullptr,
                                id0 + (unsigned long long)a, (int)m, rewind, (float)(s.charge / s.mass * 0.5 * w->dt),
                                w->ef, w->stream);
            }
            if (!ids) s.next_id += n;
            CU(cudaStreamSynchronize(w->stream));
            return check_device_error(w);
        }
    }
    // through a reusable device staging buffer, kUploadChunk particles at a time (pos, vel, w and
    // ids in FP64 / u64); without ids the device numbers the particles from next_id on
    int urc = ensure_upload(w, n);
    if (urc) return urc;
    const long cap = w->upload_cap;
    double* dp = w->upload_buf;
    double* dv = dp + 3 * (size_t)cap;
    double* dw = dv + 3 * (size_t)cap;
    unsigned long long* di = reinterpret_cast<unsigned long long*>(dw + cap);
    const unsigned long long id0 = s.next_id;
    for (long a = 0; a < n; a += cap) {
        const long m = std::min<long>(cap, n - a);
        CU(cudaMemcpyAsync(dp, pos + 3 * a, sizeof(double) * 3 * m, cudaMemcpyHostToDevice, w->stream));
        CU(cudaMemcpyAsync(dv, vel + 3 * a, sizeof(double) * 3 * m, cudaMemcpyHostToDevice, w->stream));
        CU(cudaMemcpyAsync(dw, wgt + a, sizeof(double) * m, cudaMemcpyHostToDevice, w->stream));
        if (ids) CU(cudaMemcpyAsync(di, ids + a, sizeof(unsigned long long) * m, cudaMemcpyHostToDevice, w->stream));
        Scope sc(w, "load", 5);
        launch_from_abs(w->g, s.dev, dp, dv, dw, ids ? di : nullptr, id0 + (unsigned long long)a, (int)m, rewind,
                        (float)(s.charge / s.mass * 0.5 * w->dt), w->ef, w->stream);
    }
    if (!ids) s.next_id += n;
    CU(cudaStreamSynchronize(w->stream));
    return check_device_error(w);
}

namespace {
int sort_species(pic_world* w, int sp);
}  // namespace

// Several species at once: every upload runs on a side stream, and a species is sorted on the
// world's stream as soon as its upload is done, so a species' sort (HBM) overlaps the next
// species' upload (host link).  Arrays that the device cannot read in place (pageable memory)
// take the one-species path in turn.
extern "C" int pic_species_add_particles_batch(pic_world* w, int count, const int* sps, const double* const* pos,
                                               const double* const* vel, const double* const* wgt,
                                               const uint64_t* const* ids, const long* n, int rewind, int sort) {
    if (!w || count < 0 || (count > 0 && (!sps || !pos || !vel || !wgt || !n)))
        return fail(PIC_ERR_ARG, "bad arguments");
    CU(cudaSetDevice(w->device));
    bool inplace = true;
    for (int k = 0; k < count; k++) {
        if (!valid_sp(w, sps[k]) || n[k] < 0 || (n[k] > 0 && (!pos[k] || !vel[k] || !wgt[k])))
            return fail(PIC_ERR_ARG, "bad species or arrays at batch entry %d", k);
        for (int j = 0; j < k; j++)
            if (sps[j] == sps[k]) return fail(PIC_ERR_ARG, "species %d appears twice in the batch", sps[k]);
        const uint64_t* idk = ids ? ids[k] : nullptr;
        if (n[k] > 0 && (!device_view(w, pos[k]) || !device_view(w, vel[k]) || !device_view(w, wgt[k]) ||
                         (idk && !device_view(w, idk))))
            inplace = false;
    }
    if (!inplace) {
        for (int k = 0; k < count; k++) {
            int rc = pic_species_add_particles(w, sps[k], pos[k], vel[k], wgt[k], ids ? ids[k] : nullptr, n[k], rewind);
            if (rc) return rc;
            if (sort) sort_species(w, sps[k]);
        }
        CU(cudaStreamSynchronize(w->stream));
        return check_device_error(w);
    }
    if (!w->upload_stream) CU(cudaStreamCreateWithFlags(&w->upload_stream, cudaStreamNonBlocking));
    std::vector<cudaEvent_t> ev(count + 1, nullptr);
    for (auto& e : ev) CU(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    // the uploads start after the world's pending work
    CU(cudaEventRecord(ev[count], w->stream));
    CU(cudaStreamWaitEvent(w->upload_stream, ev[count], 0));
    for (int k = 0; k < count; k++) {
        SpeciesHost& s = w->sp[sps[k]];
        const double* dp = static_cast<const double*>(device_view(w, pos[k]));
        const double* dv = static_cast<const double*>(device_view(w, vel[k]));
        const double* dw = static_cast<const double*>(device_view(w, wgt[k]));
        const uint64_t* idk = ids ? ids[k] : nullptr;
        const auto* di = static_cast<const unsigned long long*>(idk ? device_view(w, idk) : nullptr);
        const unsigned long long id0 = s.next_id;
        const long step = 1l << 30;
        for (long a = 0; a < n[k]; a += step) {
            const long m = std::min<long>(step, n[k] - a);
            // two CTAs per SM keep the host link busy and leave the SMs to the previous species' sort
            launch_from_abs(w->g, s.dev, dp + 3 * a, dv + 3 * a, dw + a, di ? di + a : nullptr,
                            id0 + (unsigned long long)a, (int)m, rewind, (float)(s.charge / s.mass * 0.5 * w->dt),
                            w->ef, w->upload_stream, 2 * w->sms);
        }
        if (!idk) s.next_id += n[k];
        CU(cudaEventRecord(ev[k], w->upload_stream));
        CU(cudaStreamWaitEvent(w->stream, ev[k], 0));
        if (sort) sort_species(w, sps[k]);  // on the world's stream, beside the next upload
    }
    CU(cudaStreamSynchronize(w->stream));  // it waited for every upload
    for (auto e : ev) cudaEventDestroy(e);
    CU(cudaGetLastError());
    return check_device_error(w);
}

extern "C" int pic_species_load_uniform(pic_world* w, int sp, const double* lo, const double* hi, long n, double T,
                                        double w_mean, double w_sigma, uint64_t seed) {
    if (!valid_sp(w, sp) || !lo || !hi || n < 0) return fail(PIC_ERR_ARG, "bad arguments");
    CU(cudaSetDevice(w->device));
    SpeciesHost& s = w->sp[sp];
    LoadArgs la;
    for (int d = 0; d < 3; d++) {
        la.lo[d] = std::max(lo[d], w->g.x0[d]);
        la.hi[d] = std::min(hi[d], w->g.xm[d]);
    }
    la.vth = (float)std::sqrt(kKb * T / s.mass);
    la.ref_thermal = 0;
    la.w_mean = (float)w_mean;
    la.w_sigma = (float)w_sigma;
    la.id0 = s.next_id;
    la.key = make_uint2((unsigned)seed, (unsigned)(seed >> 32) ^ (unsigned)(sp * 0x9E3779B9u));
    la.n = (int)n;
    s.next_id += n;
    {
        Scope sc(w, "load", 2);
        launch_load_uniform(w->g, s.dev, la, w->stream);
    }
    sort_species(w, sp);  // loaded particles leave in cell order, like after a sort step
    return check_device_error(w);
}

extern "C" int pic_species_load_box_thermal(pic_world* w, int sp, const double* center, const double* sides,
                                            double num_den, double T, uint64_t seed) {
    if (!valid_sp(w, sp) || !center || !sides) return fail(PIC_ERR_ARG, "bad arguments");
    CU(cudaSetDevice(w->device));
    SpeciesHost& s = w->sp[sp];
    double vol = sides[0] * sides[1] * sides[2];
    long n = (long)(num_den * vol / s.mpw0);  // Species.cpp:565-567
    if (n < 1) return fail(PIC_ERR_ARG, "number of macroparticles less than 1, change initial values");
    LoadArgs la;
    for (int d = 0; d < 3; d++) {
        la.lo[d] = std::max(center[d] - sides[d] / 2, w->g.x0[d]);
        la.hi[d] = std::min(center[d] + sides[d] / 2, w->g.xm[d]);
    }
    la.vth = (float)std::sqrt(2 * kKb * T / s.mass);
    la.ref_thermal = 1;
    la.w_mean = (float)s.mpw0;
    la.w_sigma = 0.f;
    la.id0 = s.next_id;
    la.key = make_uint2((unsigned)seed, (unsigned)(seed >> 32) ^ (unsigned)(sp * 0x9E3779B9u));
    la.n = (int)n;
    s.next_id += n;
    {
        Scope sc(w, "load", 2);
        launch_load_uniform(w->g, s.dev, la, w->stream);
    }
    sort_species(w, sp);  // loaded particles leave in cell order, like after a sort step
    return check_device_error(w);
}

extern "C" int pic_species_count(pic_world* w, int sp, long* n) {
    if (!valid_sp(w, sp) || !n) return fail(PIC_ERR_ARG, "bad arguments");
    CU(cudaSetDevice(w->device));
    int h = 0;
    CU(cudaMemcpyAsync(&h, w->sp[sp].dev.counts, sizeof(int), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    *n = h;
    return PIC_OK;
}

extern "C" int pic_species_get_particles(pic_world* w, int sp, double* pos, double* vel, double* wgt, uint64_t* ids,
                                         long cap, long* n_out) {
    if (!valid_sp(w, sp)) return fail(PIC_ERR_ARG, "bad species");
    long n = 0;
    int rc = pic_species_count(w, sp, &n);
    if (rc) return rc;
    if (n_out) *n_out = n;
    if (n > cap) return fail(PIC_ERR_ARG, "buffer holds %ld particles, species has %ld", cap, n);
    if (n == 0) return PIC_OK;
    SpeciesHost& s = w->sp[sp];
    double *dp, *dv, *dw;
    unsigned long long* di;
    CU(cudaMallocAsync((void**)&dp, sizeof(double) * 3 * n, w->stream));
    CU(cudaMallocAsync((void**)&dv, sizeof(double) * 3 * n, w->stream));
    CU(cudaMallocAsync((void**)&dw, sizeof(double) * n, w->stream));
    CU(cudaMallocAsync((void**)&di, sizeof(unsigned long long) * n, w->stream));
    {
        Scope sc(w, "export", 1);
        launch_to_abs(w->g, s.dev, dp, dv, dw, di, (int)n, w->stream);
    }
    if (pos) CU(cudaMemcpyAsync(pos, dp, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, w->stream));
    if (vel) CU(cudaMemcpyAsync(vel, dv, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, w->stream));
    if (wgt) CU(cudaMemcpyAsync(wgt, dw, sizeof(double) * n, cudaMemcpyDeviceToHost, w->stream));
    if (ids) CU(cudaMemcpyAsync(ids, di, sizeof(unsigned long long) * n, cudaMemcpyDeviceToHost, w->stream));
    cudaFreeAsync(dp, w->stream);
    cudaFreeAsync(dv, w->stream);
    cudaFreeAsync(dw, w->stream);
    cudaFreeAsync(di, w->stream);
    CU(cudaStreamSynchronize(w->stream));
    return check_device_error(w);
}

extern "C" int pic_species_sample_particles(pic_world* w, int sp, long num_out, double* pos, double* vel,
                                            long* n_out) {
    if (!valid_sp(w, sp) || num_out <= 0 || !n_out) return fail(PIC_ERR_ARG, "bad arguments");
    long n = 0;
    int rc = pic_species_count(w, sp, &n);
    if (rc) return rc;
    // Output::particlesOutput: every (n / num_out)-th particle, all of them when there are fewer
    long step = n / num_out, m = num_out;
    if (num_out > n) {
        m = n;
        step = 1;
    }
    *n_out = m;
    if (m == 0) return PIC_OK;
    double *dp, *dv;
    CU(cudaMallocAsync((void**)&dp, sizeof(double) * 3 * m, w->stream));
    CU(cudaMallocAsync((void**)&dv, sizeof(double) * 3 * m, w->stream));
    {
        Scope sc(w, "export", 1);
        launch_to_abs(w->g, w->sp[sp].dev, dp, dv, nullptr, nullptr, (int)m, w->stream, 0, step);
    }
    if (pos) CU(cudaMemcpyAsync(pos, dp, sizeof(double) * 3 * m, cudaMemcpyDeviceToHost, w->stream));
    if (vel) CU(cudaMemcpyAsync(vel, dv, sizeof(double) * 3 * m, cudaMemcpyDeviceToHost, w->stream));
    cudaFreeAsync(dp, w->stream);
    cudaFreeAsync(dv, w->stream);
    CU(cudaStreamSynchronize(w->stream));
    return check_device_error(w);
}

namespace {
// one push of species sp; collisions fused when sp is the collision model's electron species
int push_species(pic_world* w, int sp, double dt, int deposit, bool with_mcc, bool do_push) {
    SpeciesHost& s = w->sp[sp];
    PushArgs a{};
    a.g = w->g;
    a.sp = s.dev;
    a.ef = w->ef;
    a.qm_dt = do_push ? (float)(s.charge / s.mass * dt) : 0.f;
    for (int d = 0; d < 3; d++) a.dtdx[d] = do_push ? (float)(dt / w->g.dxd[d]) : 0.f;
    a.deposit = deposit;
    a.dep_scale = (float)s.scale;
    a.staged = 1;
    a.err = w->err;
    a.wait_polls = w->wait_polls_arg;
    a.coll.enabled = 0;
    if (with_mcc && w->mcc_on && sp == w->mcc_e) {
        a.coll = w->coll;
        a.coll.enabled = 1;
        int prc = candidate_thresholds(w, dt, a.coll);
        if (prc) return prc;
        a.coll.step = (unsigned)w->ts;
        a.coll.ion = w->sp[w->mcc_i].dev;
    }
    if (deposit) {
        s.deposited = true;
        CU(cudaMemsetAsync(s.dev.acc, 0, sizeof(unsigned long long) * w->g.nv, w->stream));
    }
    if (a.coll.enabled) {
        // collisions first (they may deposit ejected electrons), then a collision-free push
        Scope sc(w, "mcc", 3);
        launch_mcc(a, w->mcc_cand, w->mcc_ncand, w->stream, w->sms);
    }
    {
        Scope sc(w, deposit ? "push_deposit" : "push", 1);
        PushArgs ap = a;
        ap.coll.enabled = 0;
        launch_push(ap, w->stream, w->grid_push);
    }
    const bool objects = do_push && s.obj_mode == 1 && !w->boxes.empty();
    if (objects) {
        // the particles the push moved into an object (Species.cpp:211-235)
        ObjArgs o{};
        o.a = a;
        o.a.coll.enabled = 0;
        o.dt = dt;
        o.mass = s.mass;
        o.charged = s.charge != 0;
        if (o.charged) {
            const SpeciesHost& sn = w->sp[s.obj_neu];
            o.neu = sn.dev;
            o.neu_mpw0 = sn.mpw0;
            o.neu_qm = sn.charge / sn.mass;
            o.sputtering = s.obj_sputtering;
            if (o.sputtering) {
                const SpeciesHost& ss = w->sp[s.obj_spu];
                o.spu = ss.dev;
                o.spu_mpw0 = ss.mpw0;
                o.spu_qm = ss.charge / ss.mass;
            }
            o.half_dt_global = 0.5 * w->dt;
        }
        o.n_boxes = (int)w->boxes.size();
        for (int b = 0; b < o.n_boxes; b++)
            for (int d = 0; d < 3; d++) {
                o.box_c[b][d] = w->boxes[b].c[d];
                o.box_half[b][d] = w->boxes[b].s[d] * 0.5;  // Rectangle::half_sides (Object.cpp:166-171)
            }
        o.key = s.obj_key;
        o.step = (unsigned)w->ts;
        o.stats = s.obj_stats;
        Scope sc(w, "objects", 1);
        launch_object_hits(o, w->stream, w->sms);
    }
    {
        const bool neu = objects && s.charge != 0 && s.obj_neu != sp;
        const bool spu = objects && s.charge != 0 && s.obj_sputtering && s.obj_spu != s.obj_neu && s.obj_spu != sp;
        Scope sc(w, "compact", (a.coll.enabled ? 5 : 4) + neu + spu);
        launch_commit_appends(s.dev, w->err, w->stream);
        if (a.coll.enabled) launch_commit_appends(w->sp[w->mcc_i].dev, w->err, w->stream);
        if (neu) launch_commit_appends(w->sp[s.obj_neu].dev, w->err, w->stream);
        if (spu) launch_commit_appends(w->sp[s.obj_spu].dev, w->err, w->stream);
        launch_compact(s.dev, w->stream, w->sms * 4);
    }
    return PIC_OK;
}
}  // namespace

extern "C" int pic_species_push(pic_world* w, int sp, double dt, int deposit) {
    if (!valid_sp(w, sp)) return fail(PIC_ERR_ARG, "bad species");
    CU(cudaSetDevice(w->device));
    int rc = push_species(w, sp, dt, deposit, false, true);
    if (rc) return rc;
    CU(cudaGetLastError());
    return PIC_OK;
}

extern "C" int pic_species_object_interaction(pic_world* w, int sp, int mode, int neutral_sp, int spherium_sp,
                                              int sputtering, uint64_t seed) {
    if (!valid_sp(w, sp) || (mode != 0 && mode != 1)) return fail(PIC_ERR_ARG, "bad species or mode");
    SpeciesHost& s = w->sp[sp];
    if (mode == 1 && s.charge != 0) {
        if (!valid_sp(w, neutral_sp) || !(w->sp[neutral_sp].mpw0 > 0))
            return fail(PIC_ERR_ARG, "an ion species needs a species with mpw0 > 0 to neutralise into");
        if (sputtering && (!valid_sp(w, spherium_sp) || !(w->sp[spherium_sp].mpw0 > 0)))
            return fail(PIC_ERR_ARG, "sputtering needs a species with mpw0 > 0 for the sputtered material");
    }
    CU(cudaSetDevice(w->device));
    if (!s.obj_stats) {
        CU(cudaMalloc((void**)&s.obj_stats, sizeof(unsigned long long) * 4));
        CU(cudaMemsetAsync(s.obj_stats, 0, sizeof(unsigned long long) * 4, w->stream));
    }
    s.obj_mode = mode;
    s.obj_neu = neutral_sp;
    s.obj_spu = sputtering ? spherium_sp : -1;
    s.obj_sputtering = sputtering ? 1 : 0;
    s.obj_key = make_uint2((unsigned)seed, (unsigned)(seed >> 32));
    return PIC_OK;
}

extern "C" int pic_species_object_stats(pic_world* w, int sp, uint64_t* out) {
    if (!valid_sp(w, sp) || !out) return fail(PIC_ERR_ARG, "bad arguments");
    CU(cudaSetDevice(w->device));
    const SpeciesHost& s = w->sp[sp];
    if (!s.obj_stats) {
        for (int k = 0; k < 4; k++) out[k] = 0;
        return PIC_OK;
    }
    CU(cudaMemcpyAsync(out, s.obj_stats, sizeof(unsigned long long) * 4, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    return PIC_OK;
}

extern "C" int pic_species_number_density(pic_world* w, int sp) {
    if (!valid_sp(w, sp)) return fail(PIC_ERR_ARG, "bad species");
    CU(cudaSetDevice(w->device));
    int rc = push_species(w, sp, 0.0, 1, false, false);
    if (rc) return rc;
    CU(cudaGetLastError());
    return PIC_OK;
}

extern "C" int pic_species_sample_moments(pic_world* w, int sp) {
    if (!valid_sp(w, sp)) return fail(PIC_ERR_ARG, "bad species");
    CU(cudaSetDevice(w->device));
    SpeciesHost& s = w->sp[sp];
    if (!s.mom) {
        CU(cudaMalloc((void**)&s.mom, sizeof(float) * 7 * (size_t)w->g.nv));
        CU(cudaMemsetAsync(s.mom, 0, sizeof(float) * 7 * (size_t)w->g.nv, w->stream));
    }
    {
        Scope sc(w, "moments", 1);
        launch_sample_moments(w->g, s.dev, s.mom, w->stream, w->grid_parts);
    }
    CU(cudaGetLastError());
    return PIC_OK;
}

extern "C" int pic_species_clear_samples(pic_world* w, int sp) {
    if (!valid_sp(w, sp)) return fail(PIC_ERR_ARG, "bad species");
    CU(cudaSetDevice(w->device));
    SpeciesHost& s = w->sp[sp];
    if (s.mom) CU(cudaMemsetAsync(s.mom, 0, sizeof(float) * 7 * (size_t)w->g.nv, w->stream));
    return PIC_OK;
}

// Species::computeGasProperties (Species.cpp:777-804): vel = nv/n, T = m/(2k) (var_u + var_v + var_w)
extern "C" int pic_species_gas_properties(pic_world* w, int sp, double* vel, double* T) {
    if (!valid_sp(w, sp)) return fail(PIC_ERR_ARG, "bad species");
    CU(cudaSetDevice(w->device));
    SpeciesHost& s = w->sp[sp];
    const int nv = w->g.nv;
    std::vector<float> m((size_t)7 * nv, 0.f);
    if (s.mom) {
        CU(cudaMemcpyAsync(m.data(), s.mom, sizeof(float) * 7 * (size_t)nv, cudaMemcpyDeviceToHost, w->stream));
        CU(cudaStreamSynchronize(w->stream));
    }
    for (int n = 0; n < nv; n++) {
        double cnt = m[n];
        double u = cnt > 0 ? m[(size_t)nv + n] / cnt : 0, v = cnt > 0 ? m[(size_t)2 * nv + n] / cnt : 0,
               ww = cnt > 0 ? m[(size_t)3 * nv + n] / cnt : 0;
        if (vel) {
            vel[3 * n] = u;
            vel[3 * n + 1] = v;
            vel[3 * n + 2] = ww;
        }
        if (T) {
            if (cnt <= 0) {
                T[n] = 0;
                continue;
            }
            double uu = m[(size_t)4 * nv + n] / cnt - u * u, vv = m[(size_t)5 * nv + n] / cnt - v * v,
                   wq = m[(size_t)6 * nv + n] / cnt - ww * ww;
            T[n] = s.mass / (2 * kKb) * (uu + vv + wq);
        }
    }
    return PIC_OK;
}

extern "C" int pic_charge_density(pic_world* w) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    CU(cudaSetDevice(w->device));
    FinalizeArgs a{};
    a.g = w->g;
    a.ns = (int)w->sp.size();
    a.int_path = a.ns > 0;
    for (int s = 0; s < a.ns; s++) {
        SpeciesHost& sh = w->sp[s];
        a.acc[s] = sh.dev.acc;
        a.inv_scale[s] = (float)(1.0 / sh.scale);
        a.charge[s] = (float)sh.charge;
        a.den[s] = sh.den;
        double zf = sh.charge / kQe;
        a.z[s] = (int)std::lround(zf);
        if (std::fabs(zf - a.z[s]) > 1e-9 || std::abs(a.z[s]) > 8 || sh.scale != w->sp[0].scale) a.int_path = 0;
    }
    a.rho_scale = a.ns ? (float)(kQe / w->sp[0].scale) : 0.f;
    a.rho = w->rho;
    {
        Scope sc(w, "rho", 1);
        launch_finalize_rho(a, w->stream, w->grid_nodes);
    }
    // the accumulators are cleared when a species deposits again, so a species that was not
    // pushed this step keeps the density of its last push (main.cpp:222-234 subcycling)
    for (auto& s : w->sp) s.deposited = false;
    CU(cudaGetLastError());
    return PIC_OK;
}

extern "C" int pic_species_get_den(pic_world* w, int sp, double* out) {
    if (!valid_sp(w, sp) || !out) return fail(PIC_ERR_ARG, "bad arguments");
    CU(cudaSetDevice(w->device));
    std::vector<float> t(w->g.nv);
    CU(cudaMemcpyAsync(t.data(), w->sp[sp].den, sizeof(float) * w->g.nv, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    for (int n = 0; n < w->g.nv; n++) out[n] = t[n];
    return check_device_error(w);
}

extern "C" int pic_species_update_averages(pic_world* w, int sp) {
    if (!valid_sp(w, sp)) return fail(PIC_ERR_ARG, "bad species");
    CU(cudaSetDevice(w->device));
    SpeciesHost& s = w->sp[sp];
    // Field::updateMovingAverage (Field.h:245-261): restart after 20 samples
    s.avg_samples++;
    if (s.avg_samples > 20) s.avg_samples = 1;
    float b = 1.f / s.avg_samples, a = (float)(s.avg_samples - 1) / s.avg_samples;
    {
        Scope sc(w, "averages", 1);
        launch_den_avg(s.den_avg, s.den, w->g.nv, a, b, w->stream, w->grid_nodes);
    }
    CU(cudaGetLastError());
    return PIC_OK;
}
extern "C" int pic_species_get_den_avg(pic_world* w, int sp, double* out) {
    if (!valid_sp(w, sp) || !out) return fail(PIC_ERR_ARG, "bad arguments");
    CU(cudaSetDevice(w->device));
    std::vector<float> t(w->g.nv);
    CU(cudaMemcpyAsync(t.data(), w->sp[sp].den_avg, sizeof(float) * w->g.nv, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    for (int n = 0; n < w->g.nv; n++) out[n] = t[n];
    return PIC_OK;
}

namespace {
int sort_species(pic_world* w, int sp) {
    SpeciesHost& s = w->sp[sp];
    {
        Scope sc(w, "sort", 5);
        launch_sort(w->g, s.dev, s.pos2, s.vel2, s.id2, w->cell_count, w->cell_start, w->scan_aux, w->stream,
                    w->grid_parts);
    }
    std::swap(s.dev.pos, s.pos2);
    std::swap(s.dev.vel, s.vel2);
    std::swap(s.dev.id, s.id2);
    CU(cudaMemsetAsync(s.dev.counts + 5, 0, sizeof(int), w->stream));  // in cell order again
    return PIC_OK;
}
}  // namespace

extern "C" int pic_species_sort(pic_world* w, int sp, int32_t* cell_counts) {
    if (!valid_sp(w, sp)) return fail(PIC_ERR_ARG, "bad species");
    CU(cudaSetDevice(w->device));
    sort_species(w, sp);
    CU(cudaGetLastError());
    if (cell_counts) {
        // counts per cell = start[c+1] - start[c]; start has nc entries, the total is the count
        std::vector<int> st(w->g.nc);
        CU(cudaMemcpyAsync(st.data(), w->cell_start, sizeof(int) * w->g.nc, cudaMemcpyDeviceToHost, w->stream));
        int n = 0;
        CU(cudaMemcpyAsync(&n, w->sp[sp].dev.counts, sizeof(int), cudaMemcpyDeviceToHost, w->stream));
        CU(cudaStreamSynchronize(w->stream));
        for (int c = 0; c < w->g.nc; c++) cell_counts[c] = (c + 1 < w->g.nc ? st[c + 1] : n) - st[c];
    }
    return PIC_OK;
}

extern "C" int pic_species_sums(pic_world* w, int sp, double* out) {
    if (!valid_sp(w, sp) || !out) return fail(PIC_ERR_ARG, "bad arguments");
    CU(cudaSetDevice(w->device));
    // enough CTAs to keep the particle stream in flight (5 partials per CTA fit the partial buffer)
    const int grid = std::min(8 * w->sms, kParts * 8 / 5);
    {
        Scope sc(w, "sums", 1);
        launch_sums(w->sp[sp].dev, w->part, w->stream, grid);
    }
    std::vector<double> h(grid * 5);
    CU(cudaMemcpyAsync(h.data(), w->part, sizeof(double) * grid * 5, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    double t[5] = {0, 0, 0, 0, 0};
    for (int b = 0; b < grid; b++)
        for (int c = 0; c < 5; c++) t[c] += h[b * 5 + c];
    double m = w->sp[sp].mass;
    out[0] = t[0];
    out[1] = t[1] * m;
    out[2] = t[2] * m;
    out[3] = t[3] * m;
    out[4] = t[4] * m * 0.5;
    return check_device_error(w);
}

// =====================================================================================
// Poisson
// =====================================================================================
extern "C" int pic_solver_configure(pic_world* w, int method, double tol_rel, int max_it, double omega) {
    if (!w || (method != PIC_SOLVER_RBSOR && method != PIC_SOLVER_PCG && method != PIC_SOLVER_LEARNED) ||
        !(tol_rel > 0) || max_it <= 0)
        return fail(PIC_ERR_ARG, "bad solver configuration");
    if (method == PIC_SOLVER_LEARNED) {
        CU(cudaSetDevice(w->device));
        int rc = ensure_lp(w);
        if (rc) return rc;
    }
    w->method = method;
    w->tol = tol_rel;
    w->max_it = max_it;
    w->omega = omega > 0 && omega < 2 ? omega : 1.4;
    return PIC_OK;
}

extern "C" int pic_solver_set_stop(pic_world* w, int rule, double tol) {
    if (!w || (rule != PIC_STOP_REL_RHS && rule != PIC_STOP_ABS_RMS && rule != PIC_STOP_REL_CHARGE) || !(tol > 0))
        return fail(PIC_ERR_ARG, "bad stopping rule");
    w->stop_rule = rule;
    w->tol = tol;
    return PIC_OK;
}

extern "C" int pic_solver_set_warm_start(pic_world* w, int mode) {
    if (!w || (mode != PIC_WARM_PREVIOUS && mode != PIC_WARM_EXTRAPOLATE)) return fail(PIC_ERR_ARG, "bad warm-start mode");
    w->warm_mode = mode;
    w->dphi_valid = false;
    return PIC_OK;
}

extern "C" int pic_solver_set_warm_jacobi(pic_world* w, int iterations) {
    if (!w || iterations < 0 || iterations > 1000) return fail(PIC_ERR_ARG, "bad Jacobi iteration count");
    w->warm_jacobi = iterations;
    return PIC_OK;
}

extern "C" int pic_solver_last_norms(pic_world* w, double* out) {
    if (!w || !out) return fail(PIC_ERR_ARG, "null argument");
    for (int c = 0; c < 3; c++) out[c] = w->last_norms[c];
    return PIC_OK;
}

namespace {
// the quantity the residual norm is compared with: tol * stop_scale(...) (PIC_STOP_* rules)
double stop_scale(const pic_world* w, double b2, double s2) {
    const double bn = b2 > 0 ? std::sqrt(b2) : 1.0;
    switch (w->stop_rule) {
        case PIC_STOP_ABS_RMS:  // sqrt(|r|^2 / nv) <= tol (PotentialSolver.cpp:150-158)
            return std::sqrt((double)w->g.nv);
        case PIC_STOP_REL_CHARGE:  // relative to the smaller of |b| and its space-charge part
            return s2 > 0 ? std::min(bn, std::sqrt(s2)) : bn;
        default:
            return bn;
    }
}
// FP64 residual (optionally after phi += e), returns |r|^2, |b|^2 and |rho/eps0|^2 on the host
int residual_norms(pic_world* w, SolveWork& sw, int apply_e, double& r2, double& b2, double& s2) {
    if (!w->rho_prev) {
        CU(cudaMalloc(&w->rho_prev, sizeof(float) * w->g.nv));
        CU(cudaMalloc(&w->bfix, sizeof(float) * w->g.nv));
    }
    w->rhs_valid = false;
    {
        Scope sc(w, "poisson", 1);
        launch_residual(w->g, sw, apply_e, w->stream, w->rho_prev, w->bfix);
    }
    w->phi = sw.phi;
    w->phi_alt = sw.phi_alt;
    w->n_refine++;
    CU(cudaMemcpyAsync(w->h_scal, w->scal + kS_R2, sizeof(double) * 4, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    r2 = w->h_scal[0];
    b2 = w->h_scal[1];
    s2 = w->h_scal[3];
    w->rhs_valid = true;
    // r holds the float-float residual rounded to FP32: at most half an ulp per node, plus the
    // float-float evaluation error (about 2^-44 of the terms, bounded generously)
    w->r_err = kFp32Unit * std::sqrt(r2) + 1e-10 * std::sqrt(b2);
    return PIC_OK;
}
// the residual of the current phi for the new rho from the last FP64 residual (FP32 update)
int residual_update(pic_world* w, SolveWork& sw, double& r2, double& b2, double& s2) {
    {
        Scope sc(w, "poisson", 1);
        launch_rhs_update(w->g, sw, w->rho_prev, w->bfix, w->stream);
    }
    CU(cudaMemcpyAsync(w->h_scal, w->scal + kS_R2, sizeof(double) * 4, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    r2 = w->h_scal[0];
    b2 = w->h_scal[1];
    s2 = w->h_scal[3];
    // per FREE node the update t = fl(fl(rho - rho_prev) * fl(1/eps0)) is within 3.01 u |t| of
    // (rho - rho_prev) / eps0 and the sum r + t rounds by at most u |r_new|; by the triangle
    // inequality the 2-norm of the error of r grows by at most 3.01 u |t| + u |r_new|
    w->r_err += kFp32Unit * (3.01 * std::sqrt(w->h_scal[2]) + std::sqrt(r2));
    return PIC_OK;
}
// the FP32-updated residual is certified without a full pass when its norm plus the bound on its
// error stays below the tolerance (the FP32-summed norms carry a relative error below 1e-5)
bool estimate_certified(const pic_world* w, double r2, double scale) {
    return std::sqrt(r2) * (1.0 + 1e-5) + w->r_err <= w->tol * scale * (1.0 - 1e-5);
}

int ensure_lp_train(pic_world* w);

constexpr int kLearnedInnerCap = 400;  // iterations of one learned inner solve before falling back
// the last inner solve stops at sqrt(kInnerTarget) of the tolerance: below it with a margin for the
// FP32 recurrence of the inner residual, which the following float-float residual then certifies
constexpr double kInnerTarget = 0.64;

// FP32 flexible CG with the learned preconditioner on L e = r (w->r), e from zero, until
// r.r <= target or cap iterations; *done = iterations, *conv = reached the target.  Iterations go
// out in batches between which the host reads the stop flag (the iterations of a batch after the
// stop return at once, about 30 us each at 256^3): first_batch, then 2, 4, 4, ...
int learned_inner(pic_world* w, SolveWork& sw, double target, int cap, int first_batch, int* done, bool* conv) {
    {
        Scope sc(w, "poisson", 4 + 2 * w->lp->nlev);
        launch_lpcg_init(w->g, sw, *w->lp, w->stream, w->sms);
    }
    float* din = w->d;
    float* dout = w->d2;
    int it = 0;
    *done = 0;
    *conv = false;
    for (int nb = 0; it < cap; nb++) {
        int batch = std::min(nb == 0 ? std::max(1, first_batch) : std::min(4, 1 << nb), cap - it);
        {
            Scope sc(w, "poisson", (1 + 2 * w->lp->nlev) * batch);
            for (int b = 0; b < batch; b++) {
                launch_lpcg_iter(w->g, sw, *w->lp, din, dout, it, target, w->stream, w->sms);
                std::swap(din, dout);
                it++;
            }
        }
        CU(cudaMemcpyAsync(w->h_flag, w->flag, 2 * sizeof(int), cudaMemcpyDeviceToHost, w->stream));
        CU(cudaStreamSynchronize(w->stream));
        if (w->h_flag[0]) {
            *done = w->h_flag[1];  // the batch stopped at iteration flag[1]
            *conv = true;
            return PIC_OK;
        }
    }
    *done = it;
    return PIC_OK;
}

// iterations the learned preconditioner needs to reduce the residual r (FP32, node array) by
// 1e-6 from a zero start (at most cap); the validation of a training round
int learned_validation_iters(pic_world* w, const float* r, int cap, int* iters) {
    w->rhs_valid = false;
    CU(cudaMemcpyAsync(w->r, r, sizeof(float) * w->g.nv, cudaMemcpyDeviceToDevice, w->stream));
    launch_lp_norm2(w->r, w->g.nv, w->part, w->scal + 12, w->stream, w->grid_nodes);
    CU(cudaMemcpyAsync(w->h_scal, w->scal + 12, sizeof(double), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    SolveWork sw = solve_work(w);
    bool conv = false;
    int rc = learned_inner(w, sw, 1e-12 * w->h_scal[0], cap, 4, iters, &conv);
    if (!conv) *iters = cap;
    return rc;
}

int solve_impl(pic_world* w, int* iters_out, double* rel_out) {
    SolveWork sw = solve_work(w);
    double r2, b2, s2 = 0;
    // an FP32 update of the last full residual when phi is unchanged since; the answer is always
    // certified, by a full float-float residual pass or, without one, when the FP32 estimate plus
    // the bound on its accumulated rounding error is below the tolerance
    bool estimated = w->rhs_valid;
    const bool warm = estimated;  // phi unchanged since the last solve: a warm start
    bool use_pcg = false;  // set when the learned preconditioner stalls in this solve
    bool first_learned = true;  // no learned inner solve in this solve yet
    // extrapolated warm start: phi += (phi_n-1 - phi_n-2), the last warm solve's whole change,
    // then a full float-float residual of the extrapolated potential
    const bool extrapolate = warm && w->warm_mode == PIC_WARM_EXTRAPOLATE && w->dphi_valid;
    const bool track = w->warm_mode == PIC_WARM_EXTRAPOLATE;
    if (track && !w->dphi) CU(cudaMalloc((void**)&w->dphi, sizeof(float) * w->g.nv));
    int rc;
    if (extrapolate) {
        SolveWork sx = sw;
        sx.e = w->dphi;  // dphi stays as the first part of this solve's change
        rc = residual_norms(w, sx, 1, r2, b2, s2);
        sw = solve_work(w);  // phi and phi_alt were swapped
        estimated = false;
    } else {
        if (track) CU(cudaMemsetAsync(w->dphi, 0, sizeof(float) * w->g.nv, w->stream));
        rc = estimated ? residual_update(w, sw, r2, b2, s2) : residual_norms(w, sw, 0, r2, b2, s2);
    }
    if (rc) return rc;
    // a warm solve of the learned method first runs a few Jacobi iterations: even when they do
    // not reach the target they remove the high-frequency part of a warm residual (the particle
    // noise of the step's charge change) at a quarter of the cost of a learned iteration
    const bool jacobi_first = warm && w->method == PIC_SOLVER_LEARNED && w->warm_jacobi > 0;
    const bool collect = w->lp_collect && w->method != PIC_SOLVER_RBSOR;
    if (collect) {
        rc = ensure_lp_train(w);
        if (rc) return rc;
        if (lp_pair_begin(*w->lp, w->r, w->g.nv, w->stream)) return fail(PIC_ERR_CUDA, "training pair allocation");
    }
    // rel: the residual norm over the stopping rule's scale (PIC_STOP_*); converged when <= tol
    double bn = stop_scale(w, b2, s2);
    double rel = std::sqrt(r2) / bn;
    int iters = 0, outer = 0;
    const int grid = w->grid_nodes;
    for (;;) {
        if (rel <= w->tol) {
            if (!estimated || estimate_certified(w, r2, bn)) break;
            estimated = false;  // certify the FP32 estimate by a full residual pass
            rc = residual_norms(w, sw, 0, r2, b2, s2);
            if (rc) return rc;
            bn = stop_scale(w, b2, s2);
            rel = std::sqrt(r2) / bn;
            continue;
        }
        if (!(iters < w->max_it && outer < 1000)) break;
        outer++;
        estimated = false;
        if (w->method == PIC_SOLVER_LEARNED && !use_pcg) {
            int lrc = ensure_lp(w);
            if (lrc) return lrc;
        }
        if (w->method == PIC_SOLVER_RBSOR) {
            int sweeps = std::min(25, w->max_it - iters);
            {
                Scope sc(w, "poisson", 3 * sweeps);
                CU(cudaMemsetAsync(w->e, 0, sizeof(float) * w->g.nv, w->stream));
                launch_rbsor_sweeps(w->g, sw, (float)w->omega, sweeps, w->stream);
            }
            iters += sweeps;
        } else if (w->method == PIC_SOLVER_LEARNED && !use_pcg && !(jacobi_first && outer == 1)) {
            // inner FP32 flexible CG with the learned multilevel preconditioner, to eta = 1e-3 of
            // the current residual (or the final target); a preconditioner that stalls hands the
            // rest of this solve to Jacobi-PCG
            double target = std::max(1e-6 * r2, kInnerTarget * w->tol * w->tol * bn * bn);
            int done = 0;
            bool conv = false;
            // the first inner solve of a warm solve sized from the last warm one: consecutive warm
            // solves of a run need about the same count N, and iteration N is the one that finds the
            // first N converged, so the first batch runs N + 1 iterations (a cold solve, which needs
            // several times more, neither uses nor sets the count)
            const int first_batch = warm && first_learned && w->lp_hint > 0 ? w->lp_hint + 1 : 4;
            rc = learned_inner(w, sw, target, std::min(kLearnedInnerCap, w->max_it - iters), first_batch, &done, &conv);
            if (rc) return rc;
            if (warm && first_learned && conv) w->lp_hint = done;
            first_learned = false;
            iters += done;
            if (!conv) {
                use_pcg = true;
                w->lp_fallbacks++;
            }
        } else {
            // inner FP32 flexible PCG to eta = 1e-3 of the current residual (or the final target)
            double target = std::max(1e-6 * r2, kInnerTarget * w->tol * w->tol * bn * bn);
            {
                Scope sc(w, "poisson", 1);
                launch_pcg_init(w->g, sw, w->stream);
            }
            float* din = w->d;
            float* dout = w->d2;
            int it = 0;
            // a warm-started refinement of the learned method tries a few Jacobi iterations first
            const int cap = (w->method == PIC_SOLVER_LEARNED && !use_pcg) ? w->warm_jacobi : w->max_it;
            for (int nb = 2;; nb = std::min(16, 2 * nb)) {  // growing batches: early exits cost little
                int batch = std::min(std::min(nb, w->max_it - iters), cap - it);
                if (batch <= 0) break;
                {
                    Scope sc(w, "poisson", 2 * batch);
                    for (int b = 0; b < batch; b++) {
                        launch_pcg_iter_impl(w->g, sw, din, dout, it, target, w->stream);
                        std::swap(din, dout);
                        it++;
                    }
                }
                CU(cudaMemcpyAsync(w->h_flag, w->flag, 2 * sizeof(int), cudaMemcpyDeviceToHost, w->stream));
                CU(cudaStreamSynchronize(w->stream));
                if (w->h_flag[0]) {
                    iters += w->h_flag[1] - (it - batch);  // the batch stopped at iteration flag[1]
                    break;
                }
                iters += batch;
            }
        }
        if (collect) lp_pair_add(*w->lp, w->e, w->g.nv, w->stream, grid);
        if (track) {
            Scope sc(w, "poisson", 1);
            launch_add(w->dphi, w->e, w->g.nv, w->stream, grid);  // dphi += e
        }
        rc = residual_norms(w, sw, 1, r2, b2, s2);
        if (rc) return rc;
        bn = stop_scale(w, b2, s2);
        rel = std::sqrt(r2) / bn;
        if (!(rel == rel)) break;  // NaN: diverged
    }
    {
        Scope sc(w, "poisson", 2);
        launch_fill_aux(w->aux_pairs, w->n_mirror, w->n_alias, w->phi, w->stream);
    }
    if (collect) lp_pair_end(*w->lp);
    w->dphi_valid = track && warm;  // the change of a warm solve: one step's change
    w->last_norms[0] = std::sqrt(r2);
    w->last_norms[1] = std::sqrt(b2);
    w->last_norms[2] = std::sqrt(s2);
    if (iters_out) *iters_out = iters;
    if (rel_out) *rel_out = rel;
    w->n_solves++;
    w->n_inner += iters;
    CU(cudaGetLastError());
    if (!(rel <= w->tol))
        return fail(PIC_ERR_NOT_CONVERGED, "Poisson solve stopped at %d iterations, rel %.3e", iters, rel);
    return PIC_OK;
}
}  // namespace

extern "C" int pic_solver_solve(pic_world* w, int* iters, double* rel) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    CU(cudaSetDevice(w->device));
    return solve_impl(w, iters, rel);
}

extern "C" int pic_solver_stats(pic_world* w, long* solves, long* refinements, long* inner) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    if (solves) *solves = w->n_solves;
    if (refinements) *refinements = w->n_refine;
    if (inner) *inner = w->n_inner;
    return PIC_OK;
}

// ---- learned preconditioner -------------------------------------------------------------
extern "C" int pic_learned_levels(pic_world* w, int* nlev, int* dims, double* diag) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    CU(cudaSetDevice(w->device));
    int rc = ensure_lp(w);
    if (rc) return rc;
    const LpState& L = *w->lp;
    if (nlev) *nlev = L.nlev;
    for (int l = 0; l < L.nlev; l++) {
        if (dims)
            for (int d = 0; d < 3; d++) dims[3 * l + d] = L.dims[l][d];
        if (diag) diag[l] = L.diag[l];
    }
    return PIC_OK;
}
extern "C" int pic_learned_reset(pic_world* w) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    CU(cudaSetDevice(w->device));
    free_lp(w);
    return ensure_lp(w);
}
extern "C" int pic_learned_weights(pic_world* w, float* out, long capacity, long* count) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    CU(cudaSetDevice(w->device));
    int rc = ensure_lp(w);
    if (rc) return rc;
    const LpState& L = *w->lp;
    if (count) *count = L.lay.total;
    if (!out) return PIC_OK;
    if (capacity < L.lay.total) return fail(PIC_ERR_ARG, "capacity %ld < %d parameters", capacity, L.lay.total);
    CU(cudaMemcpyAsync(out, L.W, sizeof(float) * L.lay.total, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    return PIC_OK;
}
extern "C" int pic_learned_set_weights(pic_world* w, const float* in, long count) {
    if (!w || !in) return fail(PIC_ERR_ARG, "null argument");
    CU(cudaSetDevice(w->device));
    int rc = ensure_lp(w);
    if (rc) return rc;
    LpState& L = *w->lp;
    if (count != L.lay.total) return fail(PIC_ERR_ARG, "expected %d parameters, got %ld", L.lay.total, count);
    CU(cudaMemcpyAsync(L.W, in, sizeof(float) * count, cudaMemcpyHostToDevice, w->stream));
    if (L.train) launch_lp_prep(L, w->stream);  // the BF16 copies of the training GEMMs
    launch_lp_fold(L, w->stream);
    CU(cudaStreamSynchronize(w->stream));
    CU(cudaGetLastError());
    return PIC_OK;
}
extern "C" int pic_learned_apply(pic_world* w, const double* r, double* z) {
    if (!w || !r || !z) return fail(PIC_ERR_ARG, "null argument");
    CU(cudaSetDevice(w->device));
    int rc = ensure_lp(w);
    if (rc) return rc;
    const GridDev& g = w->g;
    std::vector<uint16_t> kind(g.nv);
    CU(cudaMemcpyAsync(kind.data(), w->kind, sizeof(uint16_t) * g.nv, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    std::vector<float> rf(g.nv);
    for (int n = 0; n < g.nv; n++) rf[n] = (kind[n] & 3) == kFree ? (float)r[n] : 0.f;
    w->rhs_valid = false;
    CU(cudaMemcpyAsync(w->r, rf.data(), sizeof(float) * g.nv, cudaMemcpyHostToDevice, w->stream));
    launch_lp_apply(g, *w->lp, w->r, w->z, w->kind, nullptr, nullptr, nullptr, w->stream, w->sms);
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(rf.data(), w->z, sizeof(float) * g.nv, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    for (int n = 0; n < g.nv; n++) z[n] = rf[n];
    return PIC_OK;
}

extern "C" int pic_learned_collect(pic_world* w, int on) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    CU(cudaSetDevice(w->device));
    if (on) {
        int rc = ensure_lp_train(w);
        if (rc) return rc;
    }
    w->lp_collect = on != 0;
    return PIC_OK;
}
namespace {
int lp_check_err(pic_world* w) {
    unsigned h = 0;
    CU(cudaMemcpyAsync(&h, lp_train_err(*w->lp), sizeof(unsigned), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    if (h) {
        CU(cudaMemsetAsync(lp_train_err(*w->lp), 0, sizeof(unsigned), w->stream));
        return fail(PIC_ERR_DEVICE, "a tensor-core wait of the preconditioner training ran out (flags 0x%x)", h);
    }
    return PIC_OK;
}
}  // namespace
extern "C" int pic_learned_loss_grad(pic_world* w, const double* r, const double* x, double* loss, float* grad) {
    if (!w || !r || !x) return fail(PIC_ERR_ARG, "null argument");
    CU(cudaSetDevice(w->device));
    int rc = ensure_lp_train(w);
    if (rc) return rc;
    const GridDev& g = w->g;
    std::vector<uint16_t> kind(g.nv);
    CU(cudaMemcpyAsync(kind.data(), w->kind, sizeof(uint16_t) * g.nv, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    std::vector<float> rf(g.nv), xf(g.nv);
    for (int n = 0; n < g.nv; n++) {
        bool f = (kind[n] & 3) == kFree;
        rf[n] = f ? (float)r[n] : 0.f;
        xf[n] = f ? (float)x[n] : 0.f;
    }
    LpState& L = *w->lp;
    CU(cudaMemcpyAsync(lp_train_r(L), rf.data(), sizeof(float) * g.nv, cudaMemcpyHostToDevice, w->stream));
    CU(cudaMemcpyAsync(lp_train_x(L), xf.data(), sizeof(float) * g.nv, cudaMemcpyHostToDevice, w->stream));
    {
        Scope sc(w, "learned_train", 1);
        launch_lp_loss_grad(g, L, w->kind, lp_train_r(L), lp_train_x(L), w->stream, w->grid_nodes, w->sms);
    }
    CU(cudaGetLastError());
    double h = 0;
    CU(cudaMemcpyAsync(&h, lp_train_red(L), sizeof(double), cudaMemcpyDeviceToHost, w->stream));
    if (grad) CU(cudaMemcpyAsync(grad, lp_train_grad(L), sizeof(float) * L.lay.total, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    if (loss) *loss = h;
    return lp_check_err(w);
}
// steps of Adam on the energy-norm loss; each step uses a stored solve pair when one exists and
// (step % pair_every == 0), else a white-noise pair x ~ N(0, 1) on FREE nodes with r = L x.
// The round is judged by the solver: the iterations of a validation solve (the latest pair's
// residual, or a white-noise residual) before and after; a round that needs more is rolled back.
extern "C" int pic_learned_train(pic_world* w, int steps, double lr, int pair_every, double* mean_loss,
                                 int* val_iters, int* accepted) {
    if (!w || steps < 0 || !(lr > 0)) return fail(PIC_ERR_ARG, "bad training arguments");
    CU(cudaSetDevice(w->device));
    int rc = ensure_lp_train(w);
    if (rc) return rc;
    LpState& L = *w->lp;
    const GridDev& g = w->g;
    const int np = lp_npairs(L);
    // validation right-hand side
    if (np > 0) {
        CU(cudaMemcpyAsync(lp_train_val(L), lp_pair_r(L, np - 1), sizeof(float) * g.nv, cudaMemcpyDeviceToDevice,
                           w->stream));
    } else {
        launch_lp_noise_pair(g, L, w->kind, w->lp_seed ^ 0x9e3779b97f4a7c15ull, w->stream, w->grid_nodes);
        CU(cudaMemcpyAsync(lp_train_val(L), lp_train_r(L), sizeof(float) * g.nv, cudaMemcpyDeviceToDevice, w->stream));
    }
    int before = 0, after = 0;
    rc = learned_validation_iters(w, lp_train_val(L), kLearnedInnerCap, &before);
    if (rc) return rc;
    CU(cudaMemcpyAsync(lp_train_wprev(L), L.W, sizeof(float) * L.lay.total, cudaMemcpyDeviceToDevice, w->stream));
    double sum = 0;
    int used_pairs = 0;
    for (int st = 0; st < steps; st++) {
        const float *r, *x;
        if (np > 0 && pair_every > 0 && st % pair_every == 0) {
            int k = used_pairs++ % np;
            r = lp_pair_r(L, k);
            x = lp_pair_x(L, k);
        } else {
            launch_lp_noise_pair(g, L, w->kind, w->lp_seed, w->stream, w->grid_nodes);
            r = lp_train_r(L);
            x = lp_train_x(L);
        }
        {
            Scope sc(w, "learned_train", 1);
            launch_lp_loss_grad(g, L, w->kind, r, x, w->stream, w->grid_nodes, w->sms);
            launch_lp_adam(L, (float)lr, w->stream);
        }
        double h = 0;
        CU(cudaMemcpyAsync(&h, lp_train_red(L), sizeof(double), cudaMemcpyDeviceToHost, w->stream));
        CU(cudaStreamSynchronize(w->stream));
        sum += h;
    }
    CU(cudaGetLastError());
    rc = lp_check_err(w);
    if (rc) return rc;
    rc = learned_validation_iters(w, lp_train_val(L), kLearnedInnerCap, &after);
    if (rc) return rc;
    const bool keep = after <= before;
    if (!keep) {
        CU(cudaMemcpyAsync(L.W, lp_train_wprev(L), sizeof(float) * L.lay.total, cudaMemcpyDeviceToDevice, w->stream));
        launch_lp_prep(L, w->stream);
        launch_lp_fold(L, w->stream);
        CU(cudaStreamSynchronize(w->stream));
    }
    if (mean_loss) *mean_loss = steps ? sum / steps : 0.0;
    if (val_iters) {
        val_iters[0] = before;
        val_iters[1] = after;
    }
    if (accepted) *accepted = keep ? 1 : 0;
    return PIC_OK;
}

// Level gains of the learned preconditioner, learned by the solver itself: each gain is kept only
// if a validation solve (the right-hand side of the last collected solve, else a white-noise one)
// needs fewer iterations.  The level-0 stencil is scaled first (doubling, then a half-octave
// refinement), then each network level's lift and projection together by sqrt(g), which keeps the
// projection the scaled adjoint of the lift (B stays symmetric).
extern "C" int pic_learned_calibrate(pic_world* w, int* val_iters) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    CU(cudaSetDevice(w->device));
    int rc = ensure_lp_train(w);
    if (rc) return rc;
    LpState& L = *w->lp;
    const GridDev& g = w->g;
    const int np = lp_npairs(L);
    if (np > 0) {
        CU(cudaMemcpyAsync(lp_train_val(L), lp_pair_r(L, np - 1), sizeof(float) * g.nv, cudaMemcpyDeviceToDevice,
                           w->stream));
    } else {
        launch_lp_noise_pair(g, L, w->kind, w->lp_seed ^ 0x9e3779b97f4a7c15ull, w->stream, w->grid_nodes);
        CU(cudaMemcpyAsync(lp_train_val(L), lp_train_r(L), sizeof(float) * g.nv, cudaMemcpyDeviceToDevice, w->stream));
    }
    std::vector<float> best(L.lay.total);
    CU(cudaMemcpyAsync(best.data(), L.W, sizeof(float) * best.size(), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    auto trial = [&](const std::vector<float>& wt, int* it) -> int {
        CU(cudaMemcpyAsync(L.W, wt.data(), sizeof(float) * wt.size(), cudaMemcpyHostToDevice, w->stream));
        launch_lp_prep(L, w->stream);
        launch_lp_fold(L, w->stream);
        return learned_validation_iters(w, lp_train_val(L), kLearnedInnerCap, it);
    };
    int before = 0;
    rc = trial(best, &before);
    if (rc) return rc;
    int cur = before;
    auto scaled = [&](const std::vector<float>& base, int off, int cnt, float f) {
        std::vector<float> t = base;
        for (int k = 0; k < cnt; k++) t[off + k] *= f;
        return t;
    };
    // level 0: doubling while it helps, then a half octave either side of the best
    {
        float gbest = 1.f;
        for (float gk = 2.f; gk <= 64.f; gk *= 2.f) {
            int it = 0;
            rc = trial(scaled(best, L.lay.s0, 27, gk / gbest), &it);
            if (rc) return rc;
            if (it < cur) {
                best = scaled(best, L.lay.s0, 27, gk / gbest);
                cur = it;
                gbest = gk;
            } else {
                break;
            }
        }
        for (float f : {1.41421356f, 0.70710678f}) {
            int it = 0;
            rc = trial(scaled(best, L.lay.s0, 27, f), &it);
            if (rc) return rc;
            if (it < cur) {
                best = scaled(best, L.lay.s0, 27, f);
                cur = it;
            }
        }
    }
    // network levels: gains 0.5, 0.7, 1.4, 2 on lift and projection (sqrt on each)
    for (int l = 1; l <= kLpNetLevels && l < L.nlev; l++) {
        const int C = lp_channels(l);
        for (float gl : {0.5f, 0.7f, 1.4f, 2.f}) {
            std::vector<float> t = scaled(best, L.lay.wl[l], 27 * C, std::sqrt(gl));
            t = scaled(t, L.lay.wp[l], 27 * C, std::sqrt(gl));
            int it = 0;
            rc = trial(t, &it);
            if (rc) return rc;
            if (it < cur) {
                best = t;
                cur = it;
            }
        }
    }
    int after = 0;
    rc = trial(best, &after);
    if (rc) return rc;
    if (val_iters) {
        val_iters[0] = before;
        val_iters[1] = after;
    }
    return check_device_error(w);
}

extern "C" int pic_solver_compute_ef(pic_world* w) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    CU(cudaSetDevice(w->device));
    {
        Scope sc(w, "efield", 1);
        launch_efield(w->g, w->phi, w->ef, w->stream, w->grid_nodes);
    }
    CU(cudaGetLastError());
    return PIC_OK;
}

// =====================================================================================
// collisions
// =====================================================================================
namespace {
double sigv_majorant(const std::vector<double>& E, const std::vector<double>& S, double m_red) {
    double best = 0;
    for (size_t s = 0; s < E.size(); s++) {
        double v = std::sqrt(2 * E[s] * kQe / m_red) * S[s];
        best = std::max(best, v);
        if (s + 1 < E.size()) {
            double b = (S[s + 1] - S[s]) / (E[s + 1] - E[s]), a = S[s] - b * E[s];
            if (b < 0) {
                double Es = -a / (3 * b);
                if (Es > E[s] && Es < E[s + 1]) best = std::max(best, std::sqrt(2 * Es * kQe / m_red) * (a + b * Es));
            }
        }
    }
    return best * 1.0001;
}
}  // namespace

// =====================================================================================
// Sources (Source.cpp)
// =====================================================================================
extern "C" int pic_source_create(pic_world* w, int sp, double v_drift, double den, double T, int face,
                                 uint64_t seed, int* source_id) {
    if (!valid_sp(w, sp) || !source_id || face < 0 || face > 5 || !(v_drift >= 0) || !(den >= 0) || !(T >= 0))
        return fail(PIC_ERR_ARG, "bad source arguments");
    if (w->periodic[face >> 1]) return fail(PIC_ERR_ARG, "an inlet face cannot lie on a periodic axis");
    if (!(w->sp[sp].mpw0 > 0)) return fail(PIC_ERR_ARG, "a source needs a species with a positive mpw0");
    CU(cudaSetDevice(w->device));
    pic_world::Source src;
    src.sp = sp;
    src.face = face;
    src.v_drift = v_drift;
    src.den = den;
    src.T = T;
    src.key = make_uint2((unsigned)seed, (unsigned)(seed >> 32));
    w->sources.push_back(src);
    *source_id = (int)w->sources.size() - 1;
    // World::addInlet(face) (World.cpp:206-260): the inlet face becomes Dirichlet at 0 V
    w->face_mode[face] = 1;
    w->face_phi[face] = 0.0;
    fill_grid_boxes(w);
    return upload_kinds(w, false);
}

extern "C" int pic_source_sample(pic_world* w, int source_id) {
    if (!w || source_id < 0 || source_id >= (int)w->sources.size()) return fail(PIC_ERR_ARG, "bad source");
    CU(cudaSetDevice(w->device));
    const pic_world::Source& src = w->sources[source_id];
    SpeciesHost& s = w->sp[src.sp];
    const GridDev& g = w->g;
    SourceArgs sa{};
    const int nn[3] = {g.ni, g.nj, g.nk};
    for (int d = 0; d < 3; d++) {
        sa.x0[d] = g.x0[d];
        sa.L[d] = g.dxd[d] * (nn[d] - 1);
    }
    const int ax = src.face >> 1;
    const double A = sa.L[0] * sa.L[1] * sa.L[2] / sa.L[ax];
    if (src.face & 1) sa.L[ax] -= g.dxd[ax];  // the + faces inject one cell in (Source.cpp:55, 74, 93)
    sa.face = src.face;
    sa.v_drift = src.v_drift;
    sa.vth = src.T > 0 ? std::sqrt(2 * kKb * src.T / s.mass) : 0.0;
    sa.mpw0 = s.mpw0;
    sa.key = src.key;
    sa.step = (unsigned)w->ts;
    sa.src = (unsigned)source_id;
    // num_macro = (int)(n v A dt / mpw0 + u) (Source.cpp:27, 41)
    const double num_micro = src.den * src.v_drift * A * w->dt;
    const uint4 ru = philox4x32_10(make_uint4(0xFFFFFFFFu, sa.step, 0x5C000000u + sa.src, 7u), sa.key);
    const long n = (long)(num_micro / s.mpw0 + (double)u01(ru.x));
    if (n <= 0) return PIC_OK;
    int rc = ensure_upload(w, n);
    if (rc) return rc;
    const long cap = w->upload_cap;
    double* dp = w->upload_buf;
    double* dv = dp + 3 * (size_t)cap;
    double* dw = dv + 3 * (size_t)cap;
    for (long a = 0; a < n; a += cap) {
        const long m = std::min<long>(cap, n - a);
        sa.first = (int)a;
        sa.n = (int)m;
        Scope sc(w, "source", 6);
        launch_source(sa, dp, dv, dw, w->stream);
        launch_from_abs(w->g, s.dev, dp, dv, dw, nullptr, s.next_id + (unsigned long long)a, (int)m, 1,
                        (float)(s.charge / s.mass * 0.5 * w->dt), w->ef, w->stream);
    }
    s.next_id += n;
    CU(cudaGetLastError());
    return PIC_OK;
}

extern "C" int pic_mcc_create(pic_world* w, int electrons, int ions, double n_neutral, double T_neutral,
                              double m_neutral, double E_ion_eV, double B_inc, int sigma_ion_kind,
                              const double* sigma_ion_params, const double* table_E, const double* table_s,
                              int table_n, uint64_t seed) {
    if (!valid_sp(w, electrons) || !valid_sp(w, ions) || electrons == ions)
        return fail(PIC_ERR_ARG, "electrons and ions must be two distinct species");
    if (!(E_ion_eV > 0)) return fail(PIC_ERR_ARG, "neutral species must have a positive ionisation energy");
    if (!table_E || !table_s || table_n < 1 || !sigma_ion_params) return fail(PIC_ERR_ARG, "missing cross sections");
    for (int i = 1; i < table_n; i++)
        if (!(table_E[i] > table_E[i - 1])) return fail(PIC_ERR_ARG, "sigma table energies must increase");
    CU(cudaSetDevice(w->device));
    std::vector<double> E(table_E, table_E + table_n), S(table_s, table_s + table_n);
    std::vector<float> Ef(E.begin(), E.end()), Sf(S.begin(), S.end());
    if (w->tE) cudaFree(w->tE);
    if (w->tS) cudaFree(w->tS);
    if (!w->stats) CU(cudaMalloc((void**)&w->stats, sizeof(unsigned long long) * 4));
    if (w->mcc_cand) cudaFree(w->mcc_cand);
    CU(cudaMalloc((void**)&w->mcc_cand, sizeof(int) * (size_t)w->sp[electrons].capacity));
    if (!w->mcc_ncand) CU(cudaMalloc((void**)&w->mcc_ncand, sizeof(int)));
    CU(cudaMalloc((void**)&w->tE, sizeof(float) * table_n));
    CU(cudaMalloc((void**)&w->tS, sizeof(float) * table_n));
    CU(cudaMemcpy(w->tE, Ef.data(), sizeof(float) * table_n, cudaMemcpyHostToDevice));
    CU(cudaMemcpy(w->tS, Sf.data(), sizeof(float) * table_n, cudaMemcpyHostToDevice));
    CU(cudaMemset(w->stats, 0, sizeof(unsigned long long) * 4));
    double m_e = w->sp[electrons].mass, m_n = m_neutral;
    double m_red = m_n * m_e / (m_n + m_e);
    CollDev& c = w->coll;
    c = CollDev{};
    c.sigv_max = (float)(w->mcc_sigv = sigv_majorant(E, S, m_red));
    c.sig_n = (float)std::sqrt(kKb * T_neutral / m_n);
    c.m_n = (float)m_n;
    c.m_e = (float)m_e;
    c.E_precalc_rel_eV = (float)(0.5 * m_red / kQe);
    c.half_mred = (float)(0.5 * m_red);
    c.E_precalc_ele_eV = (float)(kMe * 0.5 / kQe);
    c.E_ion_eV = (float)E_ion_eV;
    c.B_inc = (float)B_inc;
    c.two_q_over_me = (float)(2 * kQe / kMe);
    c.sig_kind = sigma_ion_kind;
    if (sigma_ion_kind == 0) {
        c.sig_a = (float)sigma_ion_params[0];
        c.sig_b = (float)sigma_ion_params[1];
        c.sig_c = (float)sigma_ion_params[2];
    } else {
        c.sig_A = (float)sigma_ion_params[0];
        c.sig_b = (float)sigma_ion_params[1];
        c.sig_c = (float)sigma_ion_params[2];
    }
    c.tE = w->tE;
    c.tS = w->tS;
    c.tn = table_n;
    c.key = make_uint2((unsigned)seed, (unsigned)(seed >> 32));
    c.stats = w->stats;
    w->mcc_n = n_neutral;
    w->mcc_seed = seed;
    w->mcc_e = electrons;
    w->mcc_i = ions;
    w->mcc_on = true;
    return PIC_OK;
}

extern "C" int pic_mcc_set_slab_density(pic_world* w, int nslabs, const double* n_neutral) {
    if (!w || !w->mcc_on) return fail(PIC_ERR_ARG, "no collision model");
    if (nslabs != w->nslabs || nslabs <= 0 || !n_neutral)
        return fail(PIC_ERR_ARG, "one density per instance slab (%d slabs)", w->nslabs);
    CU(cudaSetDevice(w->device));
    if (!w->cand_slab) CU(cudaMalloc(&w->cand_slab, sizeof(unsigned) * nslabs));
    w->slab_n.assign(n_neutral, n_neutral + nslabs);
    w->cand_slab_dt = -1.0;
    return PIC_OK;
}

extern "C" int pic_mcc_apply(pic_world* w, double dt) {
    if (!w || !w->mcc_on) return fail(PIC_ERR_ARG, "no collision model");
    CU(cudaSetDevice(w->device));
    PushArgs a{};
    SpeciesHost& s = w->sp[w->mcc_e];
    a.g = w->g;
    a.sp = s.dev;
    a.ef = w->ef;
    a.qm_dt = 0.f;
    a.deposit = 0;
    a.dep_scale = (float)s.scale;
    a.staged = 0;
    a.err = w->err;
    a.coll = w->coll;
    a.coll.enabled = 1;
    int prc = candidate_thresholds(w, dt, a.coll);
    if (prc) return prc;
    a.coll.step = (unsigned)w->ts;
    a.coll.ion = w->sp[w->mcc_i].dev;
    // collisions only: dt/dx = 0 keeps every particle in place, the products are not pushed
    {
        Scope sc(w, "mcc", 5);
        launch_mcc(a, w->mcc_cand, w->mcc_ncand, w->stream, w->sms);
        launch_commit_appends(s.dev, w->err, w->stream);
        launch_commit_appends(w->sp[w->mcc_i].dev, w->err, w->stream);
    }
    CU(cudaGetLastError());
    return PIC_OK;
}

extern "C" int pic_mcc_stats(pic_world* w, uint64_t* out) {
    if (!w || !out || !w->stats) return fail(PIC_ERR_ARG, "no collision model");
    CU(cudaSetDevice(w->device));
    CU(cudaMemcpyAsync(out, w->stats, sizeof(unsigned long long) * 4, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    return PIC_OK;
}

// =====================================================================================
// DSMC_MEX: VHS particle-particle collisions (Interactions.cpp:143-284)
// =====================================================================================
namespace {
int dsmc_apply(pic_world* w, int id, double dt) {
    pic_world::Dsmc& d = w->dsmc[id];
    // Species::sortPointers per call (Interactions.cpp:191, 227-228): the species in cell order
    int rc = sort_species(w, d.sp1);
    if (rc) return rc;
    if (!d.a.one) {
        CU(cudaMemcpyAsync(d.start1, w->cell_start, sizeof(int) * w->g.nc, cudaMemcpyDeviceToDevice, w->stream));
        rc = sort_species(w, d.sp2);
        if (rc) return rc;
    }
    DsmcArgs a = d.a;
    a.vel1 = w->sp[d.sp1].dev.vel;
    a.vel2 = w->sp[d.sp2].dev.vel;
    a.start1 = d.a.one ? w->cell_start : d.start1;
    a.start2 = w->cell_start;
    a.n1 = w->sp[d.sp1].dev.counts;
    a.n2 = w->sp[d.sp2].dev.counts;
    a.nc = w->g.nc;
    a.half_coef = 0.5 * d.mpw0 * dt / d.dv;
    a.call = d.calls++;
    {
        Scope sc(w, "dsmc", 2);
        launch_dsmc(a, w->stream);
    }
    CU(cudaGetLastError());
    return PIC_OK;
}
}  // namespace

extern "C" int pic_dsmc_create(pic_world* w, int sp1, int sp2, uint64_t seed, int* dsmc_id) {
    if (!valid_sp(w, sp1) || !dsmc_id) return fail(PIC_ERR_ARG, "bad species");
    if (sp2 < 0) sp2 = sp1;
    if (!valid_sp(w, sp2)) return fail(PIC_ERR_ARG, "bad second species");
    if (w->dsmc.size() >= 256) return fail(PIC_ERR_ARG, "at most 256 DSMC interactions per world");
    const SpeciesHost& s1 = w->sp[sp1];
    const SpeciesHost& s2 = w->sp[sp2];
    if (!(s1.mpw0 > 0)) return fail(PIC_ERR_ARG, "DSMC needs a positive macroparticle weight");
    // the two-species constructor's check (Interactions.cpp:160-162)
    if (s1.mpw0 != s2.mpw0)
        return fail(PIC_ERR_ARG, "species must have the same macroparticle weight for this algorithm to work properly.");
    CU(cudaSetDevice(w->device));
    pic_world::Dsmc d;
    d.sp1 = sp1;
    d.sp2 = sp2;
    const double m1 = s1.mass, m2 = s2.mass, m_red = m1 * m2 / (m1 + m2);
    // Bird's VHS parameters at 273.15 K (Interactions.cpp:152-156, 173-176)
    const double d_ref = 4.07e-10, omega = 0.77, c2 = 2 * kKb * 273.15 / m_red;
    d.a = DsmcArgs{};
    d.a.K = (float)(kPiRef * d_ref * d_ref * std::pow(c2, omega - 0.5) / std::tgamma(2.5 - omega));
    d.a.ex = (float)(1.0 - omega);
    d.a.f1 = (float)(m1 / (m1 + m2));
    d.a.f2 = (float)(m2 / (m1 + m2));
    d.a.one = sp1 == sp2;
    d.a.key = make_uint2((unsigned)seed, (unsigned)(seed >> 32));
    d.a.tag = 0xD5000000u + (unsigned)w->dsmc.size();
    d.mpw0 = s1.mpw0;
    d.dv = w->g.dxd[0] * w->g.dxd[1] * w->g.dxd[2];  // World::getCellVolume (World.cpp:101-103)
    CU(cudaMalloc((void**)&d.state, 32));
    if (!d.a.one && cudaMalloc((void**)&d.start1, sizeof(int) * (size_t)w->g.nc) != cudaSuccess) {
        cudaFree(d.state);
        return fail(PIC_ERR_CUDA, "out of device memory for the DSMC cell lists");
    }
    unsigned long long init[4] = {0, 0, 0, 0};
    const float sv0 = 1e-14f;  // DSMC_MEX::sigma_v_rel_max initial value (Interactions.h:58)
    std::memcpy(&init[3], &sv0, sizeof(float));
    CU(cudaMemcpy(d.state, init, sizeof(init), cudaMemcpyHostToDevice));
    d.a.stats = d.state;
    d.a.svmax = reinterpret_cast<float*>(d.state + 3);
    d.a.svmax_step = reinterpret_cast<unsigned*>(d.state + 3) + 1;
    w->dsmc.push_back(d);
    *dsmc_id = (int)w->dsmc.size() - 1;
    return PIC_OK;
}

extern "C" int pic_dsmc_apply(pic_world* w, int dsmc_id, double dt) {
    if (!w || dsmc_id < 0 || dsmc_id >= (int)w->dsmc.size()) return fail(PIC_ERR_ARG, "bad DSMC interaction");
    if (!(dt >= 0)) return fail(PIC_ERR_ARG, "dt must be non-negative");
    CU(cudaSetDevice(w->device));
    return dsmc_apply(w, dsmc_id, dt);
}

extern "C" int pic_dsmc_stats(pic_world* w, int dsmc_id, uint64_t* counts, double* sigma_v_rel_max) {
    if (!w || dsmc_id < 0 || dsmc_id >= (int)w->dsmc.size()) return fail(PIC_ERR_ARG, "bad DSMC interaction");
    CU(cudaSetDevice(w->device));
    unsigned long long st[4];
    CU(cudaMemcpyAsync(st, w->dsmc[dsmc_id].state, sizeof(st), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    if (counts) {
        counts[0] = st[0];
        counts[1] = st[1];
    }
    if (sigma_v_rel_max) {
        float sv;
        std::memcpy(&sv, &st[3], sizeof(float));
        *sigma_v_rel_max = sv;
    }
    return PIC_OK;
}

// =====================================================================================
// step loop (ch4/v3/src/main.cpp:177-286)
// =====================================================================================
extern "C" int pic_loop_configure(pic_world* w, int solve_each_step, int sort_every, const int* subcycle,
                                  int merge_every, int merge_after, int merge_min) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    w->solve_each_step = solve_each_step;
    w->sort_every = sort_every;
    for (int s = 0; s < kMaxSpecies; s++) w->subcycle[s] = subcycle && subcycle[s] > 0 ? subcycle[s] : 1;
    w->merge_every = merge_every;
    w->merge_after = merge_after;
    w->merge_min = merge_min;
    return PIC_OK;
}

extern "C" int pic_species_merge(pic_world* w, int sp, int min_count) {
    if (!valid_sp(w, sp) || min_count < 3) return fail(PIC_ERR_ARG, "bad species or min_count < 3");
    CU(cudaSetDevice(w->device));
    if (!w->merge_list) {
        CU(cudaMalloc((void**)&w->merge_list, sizeof(int) * (w->g.nc + 1)));
        CU(cudaMalloc((void**)&w->merge_stats, sizeof(unsigned long long) * 4));
        CU(cudaMemsetAsync(w->merge_stats, 0, sizeof(unsigned long long) * 4, w->stream));
    }
    sort_species(w, sp);  // cells must be contiguous runs
    SpeciesHost& s = w->sp[sp];
    uint64_t seed = w->mcc_seed ^ 0x6D65726765ull;
    {
        Scope sc(w, "merge", 2);
        launch_merge(w->g, s.dev, w->ef, w->cell_start, w->merge_list + 1, w->merge_list, min_count,
                     (float)(s.charge / s.mass * 0.5 * w->dt), make_uint2((unsigned)seed, (unsigned)(seed >> 32)),
                     (unsigned)w->ts, w->err, w->merge_stats, w->stream, w->sms * 8);
    }
    {
        Scope sc(w, "compact", 4);
        launch_commit_appends(s.dev, w->err, w->stream);
        launch_compact(s.dev, w->stream, w->sms * 4);
    }
    CU(cudaGetLastError());
    return PIC_OK;
}

extern "C" int pic_merge_stats(pic_world* w, uint64_t* out) {
    if (!w || !out) return fail(PIC_ERR_ARG, "null argument");
    CU(cudaSetDevice(w->device));
    if (!w->merge_stats) {
        out[0] = out[1] = out[2] = 0;
        return PIC_OK;
    }
    CU(cudaMemcpyAsync(out, w->merge_stats, sizeof(unsigned long long) * 3, cudaMemcpyDeviceToHost, w->stream));
    CU(cudaStreamSynchronize(w->stream));
    return PIC_OK;
}

extern "C" int pic_step(pic_world* w) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    CU(cudaSetDevice(w->device));
    Scope whole(w, "step", 0);
    w->ts++;  // World::advanceTime
    const int ts = w->ts;
    if (w->merge_every > 0 && ts > w->merge_after && ts % w->merge_every == 0) {
        for (int s = 0; s < (int)w->sp.size(); s++) {
            int rc = pic_species_merge(w, s, w->merge_min);
            if (rc) return rc;
        }
    }
    for (int q = 0; q < (int)w->sources.size(); q++) {  // main.cpp:196-198
        int rc = pic_source_sample(w, q);
        if (rc) return rc;
    }
    for (int q = 0; q < (int)w->dsmc.size(); q++) {  // main.cpp:201-203 (MC_MEX collisions ride on the push)
        int rc = dsmc_apply(w, q, w->dt);
        if (rc) return rc;
    }
    // collisions are fused into the electron push, which runs first so that the ion products
    // are pushed in this step too (the reference applies interactions before the species loop)
    std::vector<int> order;
    if (w->mcc_on) order.push_back(w->mcc_e);
    for (int s = 0; s < (int)w->sp.size(); s++)
        if (!(w->mcc_on && s == w->mcc_e)) order.push_back(s);
    for (int s : order) {
        int k = w->subcycle[s];
        if (ts % k != 0) continue;
        int rc = push_species(w, s, w->dt * k, 1, true, true);
        if (rc) return rc;
    }
    int rc = pic_charge_density(w);
    if (rc) return rc;
    if (w->solve_each_step) {
        rc = solve_impl(w, nullptr, nullptr);
        if (rc) return rc;
        rc = pic_solver_compute_ef(w);
        if (rc) return rc;
    }
    if (w->sort_every > 0 && ts % w->sort_every == 0) {
        // a species is re-sorted when at least 1/kSortMovedFraction of its particles changed cell
        // or were appended since its last sort (slow ions stay in order for many periods)
        const int ns = (int)w->sp.size();
        std::vector<int> cnt(8 * ns);
        for (int s = 0; s < ns; s++)
            CU(cudaMemcpyAsync(&cnt[8 * s], w->sp[s].dev.counts, sizeof(int) * 8, cudaMemcpyDeviceToHost, w->stream));
        CU(cudaStreamSynchronize(w->stream));
        for (int s = 0; s < ns; s++)
            if ((long)cnt[8 * s + 5] * kSortMovedFraction >= (long)cnt[8 * s] && cnt[8 * s + 5] > 0) sort_species(w, s);
    }
    CU(cudaGetLastError());
    return PIC_OK;
}

// =====================================================================================
// Autotuner: launch shapes measured on the world's own data
// =====================================================================================
namespace {
// mean device time of f() over reps launches after one warm-up launch, in milliseconds
template <class F>
float time_launches(pic_world* w, int reps, F f) {
    f();
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, w->stream);
    for (int r = 0; r < reps; r++) f();
    cudaEventRecord(b, w->stream);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    return ms / reps;
}
}  // namespace

extern "C" int pic_autotune(pic_world* w, int* push_ctas_per_sm, int* node_grid) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    CU(cudaSetDevice(w->device));
    // streaming node kernels (residual, CG, learned CG): CTA count from 2 to 16 per SM, timed on
    // the float-float residual, which only recomputes r from phi and rho
    {
        SolveWork sw = solve_work(w);
        double r2, b2, s2;
        int rc = residual_norms(w, sw, 0, r2, b2, s2);  // allocates the residual's side arrays
        if (rc) return rc;
        const int most = std::min<long>((w->g.nv / 4 + 255) / 256, (long)w->gstride);
        int best = 0;
        float best_ms = 0.f;
        for (int m : {2, 4, 8, 16}) {
            const int cand = std::min(w->sms * m, most);
            if (cand < 1 || cand == best) continue;
            w->g.node_grid = cand;
            sw = solve_work(w);
            const float ms = time_launches(w, 5, [&] { launch_residual(w->g, sw, 0, w->stream, w->rho_prev, w->bfix); });
            if (!best || ms < best_ms) {
                best = cand;
                best_ms = ms;
            }
        }
        w->g.node_grid = best;
        w->rhs_valid = false;  // r was rewritten: the next solve starts from a full residual
    }
    // CG stencil kernels (d = z + beta d, q = L d): timed on the learned-CG one at iteration 0, which
    // writes only the solver's scratch arrays (d2, q and the dot-product slot; every solve starts
    // them afresh)
    {
        SolveWork sw = solve_work(w);
        const int most = std::min<long>((w->g.nv / 4 + 255) / 256, (long)w->gstride);
        int best = 0;
        float best_ms = 0.f;
        for (int m : {2, 4, 8, 16}) {
            const int cand = std::min(w->sms * m, most);
            if (cand < 1 || cand == best) continue;
            w->g.cg_grid = cand;
            const float ms = time_launches(w, 5, [&] { launch_lpcg_k1_probe(w->g, sw, w->d, w->d2, w->stream); });
            if (!best || ms < best_ms) {
                best = cand;
                best_ms = ms;
            }
        }
        w->g.cg_grid = best;
    }
    // push + deposit: CTAs per SM from 1 to the occupancy limit, timed on pushes with dt = 0
    // (positions and velocities stay, and the deposit reproduces the density of the particles
    // where they are, which the last step deposited)
    {
        long n_all = 0;
        for (auto& s : w->sp) {
            int n = 0;
            CU(cudaMemcpyAsync(&n, s.dev.counts, sizeof(int), cudaMemcpyDeviceToHost, w->stream));
            CU(cudaStreamSynchronize(w->stream));
            n_all += n;
        }
        const int most = push_blocks_per_sm();
        int best = most;
        if (n_all > 0) {
            float best_ms = 0.f;
            for (int c = 1; c <= most; c++) {
                w->grid_push = w->sms * c;
                const float ms = time_launches(w, 3, [&] {
                    for (int s = 0; s < (int)w->sp.size(); s++) push_species(w, s, 0.0, 1, false, true);
                });
                if (c == 1 || ms < best_ms) {
                    best = c;
                    best_ms = ms;
                }
            }
        }
        w->grid_push = w->sms * best;
        if (push_ctas_per_sm) *push_ctas_per_sm = best;
    }
    if (node_grid) *node_grid = w->g.node_grid;
    return check_device_error(w);
}

extern "C" int pic_launch_shapes(pic_world* w, int* push_ctas_per_sm, int* node_grid, int* cg_grid) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    if (push_ctas_per_sm) *push_ctas_per_sm = w->sms > 0 ? w->grid_push / w->sms : 0;
    if (node_grid) *node_grid = w->g.node_grid;
    if (cg_grid) *cg_grid = w->g.cg_grid;
    return PIC_OK;
}

extern "C" int pic_set_launch_shapes(pic_world* w, int push_ctas_per_sm, int node_grid, int cg_grid) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    CU(cudaSetDevice(w->device));
    const int push_most = push_blocks_per_sm();
    if (push_ctas_per_sm < 0 || push_ctas_per_sm > push_most)
        return fail(PIC_ERR_ARG, "push CTAs per SM %d outside 0..%d", push_ctas_per_sm, push_most);
    // any positive count is safe: a launch never takes more than one CTA per 1024 nodes, which the
    // block-partial buffer holds
    for (int v : {node_grid, cg_grid})
        if (v < 0) return fail(PIC_ERR_ARG, "negative node-kernel grid %d", v);
    w->grid_push = w->sms * (push_ctas_per_sm > 0 ? push_ctas_per_sm : push_most);
    w->g.node_grid = node_grid;
    w->g.cg_grid = cg_grid;
    return PIC_OK;
}

extern "C" int pic_debug_set_wait_polls(pic_world* w, long long polls) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    CU(cudaSetDevice(w->device));
    const long long arg = polls < 0 ? 0 : (polls == 0 ? -1 : polls);
    w->wait_polls_arg = arg;
    if (lp_set_tc_wait_polls(arg)) return fail(PIC_ERR_CUDA, "setting the tensor-core wait limit failed");
    return PIC_OK;
}

extern "C" int pic_synchronize(pic_world* w) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    CU(cudaSetDevice(w->device));
    CU(cudaStreamSynchronize(w->stream));
    return check_device_error(w);
}

extern "C" int pic_last_error(char* buf, int len) {
    if (buf && len > 0) {
        strncpy(buf, g_err, len - 1);
        buf[len - 1] = 0;
    }
    return PIC_OK;
}

extern "C" int pic_timing_enable(pic_world* w, int on) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    w->timing = on != 0;
    return PIC_OK;
}
extern "C" int pic_timing_read(pic_world* w, const char* name, double* ms, long* launches) {
    if (!w || !name) return fail(PIC_ERR_ARG, "null argument");
    collect_timers(w);
    auto it = w->timers.find(name);
    if (ms) *ms = it == w->timers.end() ? 0.0 : it->second.ms;
    if (launches) *launches = it == w->timers.end() ? 0 : it->second.launches;
    return PIC_OK;
}
extern "C" int pic_timing_reset(pic_world* w) {
    if (!w) return fail(PIC_ERR_ARG, "null world");
    collect_timers(w);
    w->timers.clear();
    return PIC_OK;
}
extern "C" int pic_launch_count(pic_world* w, long* n) {
    if (!w || !n) return fail(PIC_ERR_ARG, "null argument");
    *n = w->launches;
    return PIC_OK;
}
extern "C" int pic_world_stream(pic_world* w, void** stream) {
    if (!w || !stream) return fail(PIC_ERR_ARG, "null argument");
    *stream = (void*)w->stream;
    return PIC_OK;
}
