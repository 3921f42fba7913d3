/* pic_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * Plain-C FP64 restatement of the reference's ch4/v3 electrostatic PIC + DSMC step
 * (Misquic/Engineering-degree-in-Plasma-Simulations).  It is the checker for the CUDA
 * library and the timed CPU baseline; only tests/, __graft_entry__.smoke() and
 * bench.py (cpu_baseline leg and --impl reference) may load it.  The product path
 * never calls it and has no CPU fallback.
 *
 * Two families of functions:
 *   or_*_ref  : restate the reference's own algorithms step for step (same loop order,
 *               same FP64 operation order, same MT19937 draws).  These are pinned
 *               bit-for-bit against the reference compiled from its sources
 *               (oracle/_ref, tests/golden).
 *   or_*      : FP64 restatements of the GPU forms that the reference lacks (periodic
 *               x/y, background-neutral collisions with Philox streams, red-black SOR,
 *               flexible PCG with FP64 residual refinement, Lotz cross-section).
 *
 * Layout conventions shared with the CUDA library:
 *   node index  n = (k*nj + j)*ni + i          (reference Field::U, Field.h:262-265)
 *   cell index  c = (k*(nj-1) + j)*(ni-1) + i  (reference World::XtoC, World.cpp:134-137)
 */
#ifndef PIC_ORACLE_H
#define PIC_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* physical constants exactly as ch4/v3/src/all.h:16-25 */
#define OR_EPS0 8.85418782e-12
#define OR_QE 1.602176565e-19
#define OR_AMU 1.660538921e-27
#define OR_ME 9.10938215e-31
#define OR_KB 1.380648e-23
#define OR_PI 3.141592653

/* node kinds */
enum { OR_FREE = 0, OR_FIXED = 1, OR_MIRROR = 2, OR_ALIAS = 3 };

typedef struct {
    double pos[3];
    double vel[3];
    double w;
} or_particle; /* reference Particle, Species.h:12-29 */

typedef struct {
    int ni, nj, nk;
    double x0[3], xm[3], dx[3], inv_dx[3];
    int periodic[3];
    int n_boxes; /* axis-aligned Rectangle objects (Object.cpp:231-238): absorbing */
    double box_c[8][3], box_half[8][3];
} or_grid;

void or_grid_init(or_grid* g, int ni, int nj, int nk, const double* x0, const double* xm, const int* periodic);
int or_grid_add_box(or_grid* g, const double* center, const double* sides);
/* node kinds for the three boundary flavours used by the configs:
 *  wall_mode 0: reference v3 walls (MIRROR = Neumann copy of inner neighbour)
 *  wall_mode 1: all non-periodic walls FIXED (Dirichlet, ch2 semantics)
 *  periodic axes get ALIAS at index n-1; nodes inside boxes are FIXED. */
void or_node_kinds(const or_grid* g, int wall_mode, uint8_t* kind);

/* ---- random numbers ---- */
typedef struct {
    uint32_t mt[624];
    int idx;
} or_mt;
void or_mt_seed(or_mt* r, uint32_t seed);
uint32_t or_mt_next(or_mt* r);
double or_mt_u01(or_mt* r); /* std::uniform_real_distribution<double>(0,1) over mt19937 */
void or_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);
double or_u01_from_u32(uint32_t x); /* ((x>>9)+0.5)*2^-23: the GPU's draw, exact in FP32 and FP64 */

/* ---- fields ---- */
void or_node_volumes(const or_grid* g, double* vol);
void or_gather3_ref(const or_grid* g, const double* f3, const double lc[3], double out[3]);
void or_scatter_ref(const or_grid* g, double* f, const double lc[3], double val);
void or_number_density_ref(const or_grid* g, const or_particle* p, long n, double* den);
void or_compute_ef_ref(const or_grid* g, const double* phi, double* ef);

/* ---- push ---- */
long or_push_electrons_ref(const or_grid* g, or_particle* p, long n, uint64_t* ids, const double* ef, double dt,
                           double charge, double mass);
long or_push_electrons_mt(const or_grid* g, or_particle* p, long n, uint64_t* ids, const double* ef, double dt,
                          double charge, double mass, int nthreads);

/* ---- Poisson ---- */
int or_solve_gs_ref(const or_grid* g, const uint8_t* kind, double* phi, const double* rho, int max_it, double tol,
                    int* iters, double* l2);
int or_solve_pcg_ref(const or_grid* g, const uint8_t* kind, double* phi, const double* rho, int max_it, double tol,
                     int axis_swap, int* iters, double* l2);
void or_fill_aux(const or_grid* g, const uint8_t* kind, double* phi);
void or_residual(const or_grid* g, const uint8_t* kind, const double* phi, const double* rho, double* rnorm2,
                 double* bnorm2);
int or_solve_rbsor(const or_grid* g, const uint8_t* kind, double* phi, const double* rho, double omega, double tol_rel,
                   int max_sweeps, int* sweeps, double* rel);
int or_solve_fpcg(const or_grid* g, const uint8_t* kind, double* phi, const double* rho, double tol_rel, int max_it,
                  int* iters, double* rel);

/* ---- collisions ---- */
typedef struct {
    double mass_neutral, mass_electron, E_ion_eV, B_inc;
    int sigma_ion_kind; /* 0: reference fit a*ln(E/b)/E*exp(-c/E); 1: Lotz A*ln(E/I)/(E*I)*(1-b*exp(-c*(E/I-1))) */
    double sig_a, sig_b, sig_c, sig_A;
    const double* table_E; /* sigma_coll table (eV, m^2), ascending */
    const double* table_s;
    int table_n;
    double n_neutral, T_neutral, sigv_max; /* background gas */
} or_coll_params;
double or_sigma_coll(const or_coll_params* cp, double E_eV);
double or_sigma_ion(const or_coll_params* cp, double E_eV);
double or_sigv_majorant(const or_coll_params* cp);

/* Background-gas electron-impact collisions (GPU form, restated in FP64).
 * Draws come from Philox-4x32-10 keyed by (seed, step, particle id) in the same order as
 * the CUDA kernel.  Products (electron + ion, weight of the parent electron) are appended
 * at ele[*n_ele] and ion[*n_ion] with ids derived from the parent id.  Returns the number
 * of real collisions; *n_ionized receives the ionisations. */
long or_mcc_background(const or_grid* g, const or_coll_params* cp, or_particle* ele, uint64_t* ele_id, long* n_ele,
                       long cap_ele, or_particle* ion, uint64_t* ion_id, long* n_ion, long cap_ion, double dt,
                       uint32_t seed_lo, uint32_t seed_hi, uint32_t step, long* n_ionized);
uint64_t or_child_id(uint64_t parent, uint32_t step, uint32_t kind);
uint32_t or_cand_draw(uint64_t id, uint32_t step, uint32_t seed_lo, uint32_t seed_hi);
uint32_t or_cand_threshold(double p);

/* Reference NTC ionisation with neutral macroparticles (Interactions.cpp:600-762), MT19937 draws.
 * wsv_max is the persistent (W*sigma*v)_max, updated in place. Returns collisions. */
long or_ntc_ionize_ref(const or_grid* g, const or_coll_params* cp, or_mt* r, or_particle* neu, long* n_neu,
                       long cap_neu, or_particle* ion, long* n_ion, long cap_ion, or_particle* ele, long* n_ele,
                       long cap_ele, double dt, double* wsv_max);

/* Reference merge (Species.cpp:981-1145) including addParticle's rewind with the global dt.
 * min_count: cells with fewer particles are skipped (reference: 10). Returns new count. */
long or_merge_ref(const or_grid* g, or_mt* r, or_particle* p, long n, long cap, const double* ef, double charge,
                  double mass, double dt_global, int min_count);

/* GPU form of the merge (restated from the CUDA kernel): per cell with >= min_count particles
 * (cells[] given, or computed from positions when NULL), velocities binned on 15^3 in FP32
 * exactly as the device does, members ordered by (bin, Philox hash of id); bins with more than
 * two particles become two particles placed at the two smallest-hash members, ids from
 * or_child_id(member id, step, 3).  Merged members get w = 0 and are removed at the end.
 * Returns the new count. */
long or_merge_gpuform(const or_grid* g, or_particle* p, uint64_t* ids, const int32_t* cells, long n, long cap,
                      const double* ef, double charge, double mass, double dt_global, int min_count,
                      uint32_t seed_lo, uint32_t seed_hi, uint32_t step);

/* Reference loadParticleBoxThermal (Species.cpp:564-599, 855-869), with rejection and rewind (E given). */
long or_load_box_thermal_ref(const or_grid* g, or_mt* r, or_particle* p, long cap, const double* x0,
                             const double* sides, double num_den, double T, double mpw0, double mass, double charge,
                             const double* ef, double dt);

/* Species::sampleMoments (Species.cpp:767-776): accumulates into mom[7*nv] (planes n, nvx,
 * nvy, nvz, nuu, nvv, nww); Species::computeGasProperties (777-804) -> vel[3*nv], T[nv] */
void or_sample_moments_ref(const or_grid* g, const or_particle* p, long n, double* mom);
void or_gas_properties_ref(const or_grid* g, const double* mom, double mass, double* vel, double* T);

/* ---- DSMC_MEX: VHS particle-particle collisions (Interactions.cpp:143-284) ---- */
typedef struct {
    double mass1, mass2, mpw0, dv; /* dv: cell volume dx dy dz (World::getCellVolume, World.cpp:101) */
    double c[4];                   /* d_ref, omega, 2 k 273.15 / m_r, Gamma(2.5 - omega) (Interactions.cpp:152-156) */
} or_dsmc_params;
void or_dsmc_params_init(or_dsmc_params* q, const or_grid* g, double mass1, double mass2, double mpw0);
double or_dsmc_sigma(const or_dsmc_params* q, double v_rel); /* DSMC_MEX::evaluateSigma */

/* DSMC_MEX::applyOneSpecies / applyTwoSpecies (p2 == NULL: one species), MT19937 draws in the
 * reference's order; *svmax is the persistent (sigma v_rel)_max, updated in place.  Returns
 * the collisions; *pairs receives the candidate pairs drawn. */
long or_dsmc_ref(const or_grid* g, const or_dsmc_params* q, or_mt* r, or_particle* p1, long n1, or_particle* p2,
                 long n2, double dt, double* svmax, long* pairs);

/* GPU form (restated from the CUDA kernel, in FP64 on the same draws): particles of each
 * species contiguous in cell order, cnt1/cnt2[nc] per cell (vel2/cnt2 NULL: one species);
 * group gi of cell c draws Philox block (c, call, tag, gi): the high 23 bits of its words for
 * the pair, the acceptance and cos(chi), the low 9 bits of the first three words (27 bits) for
 * the azimuth of a collision;
 * sigma v_rel is evaluated as K (v_rel^2)^(1-omega), K = pi d^2 c2^(omega-1/2) / Gamma.
 * svmax is the FP32 majorant the kernel reads; *svmax_step receives the largest sigma v of
 * the candidates (the next majorant when any pair collided).  Returns the collisions. */
long or_dsmc_gpuform(const or_dsmc_params* q, double* vel1, const int32_t* cnt1, double* vel2, const int32_t* cnt2,
                     long nc, double dt, double svmax, uint32_t seed_lo, uint32_t seed_hi, uint32_t call,
                     uint32_t tag, long* pairs, double* svmax_step);

/* ---- object interaction of non-electron species (Species.cpp:45-256) ---- */
typedef struct {
    or_particle* neu; /* neutral species particles are appended here (Species::addParticle) */
    uint64_t* neu_ids; /* GPU form: ids of the created neutrals */
    long* n_neu;
    long cap_neu;
    double neu_mpw0;
    or_particle* spu; /* sputtered material (spherium) */
    uint64_t* spu_ids;
    long* n_spu;
    long cap_spu;
    double spu_mpw0;
    int sputtering;   /* Config::SPUTTERING */
    double neu_qm, spu_qm; /* charge / mass of the two species (addParticle's rewind) */
    const double* ef; /* E for addParticle's rewind (no effect on neutral species) */
    double dt_global;
} or_obj_species;
/* Species::advanceNoSputteringSerial / advanceSputteringSerial with Rectangle objects, MT19937
 * draws in the reference's order; swap-with-last deletion.  Returns the new count; created[0]
 * neutrals and created[1] sputtered particles appended. */
long or_push_nonelectron_ref(const or_grid* g, or_mt* r, or_particle* p, long n, const double* ef, double dt,
                             double charge, double mass, const or_obj_species* t, long created[2]);
/* GPU form (restated from k_push + k_object_hits, FP64): periodic axes wrap; a particle that
 * enters an object draws from Philox stream (id, step, 0x0B000000 + block) with key seed;
 * survivors keep their ids.  stats: impacts, bounces, neutrals created, sputtered created. */
long or_push_nonelectron_gpuform(const or_grid* g, or_particle* p, uint64_t* ids, long n, const double* ef, double dt,
                                 double charge, double mass, const or_obj_species* t, uint32_t seed_lo,
                                 uint32_t seed_hi, uint32_t step, long stats[4]);

/* conservation sums (Species.cpp:732-752) */
void or_sums(const or_particle* p, long n, double mass, double* count, double mom[3], double* ke);

#ifdef __cplusplus
}
#endif
#endif
