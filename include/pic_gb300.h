/* pic_gb300.h -- C ABI of the GB300 (sm_103a) electrostatic PIC + DSMC step library.
 *
 * Drop-in boundary for the ch4/v3 step loop of Misquic/Engineering-degree-in-Plasma-Simulations.
 * The reference exposes C++ classes only (World, Species, PotentialSolver, Interaction); each
 * entry point below names the reference member it replaces.  Plain pointers and sizes only:
 * host arrays are FP64, node arrays are flat with i fastest (n = (k*nj + j)*ni + i, the
 * reference Field::U, ch4/v3/src/Field.h:262-265), particle arrays are xyz-interleaved.
 *
 * Every function returns PIC_OK (0) or a PIC_ERR_* code; pic_last_error() gives the message.
 * Device state lives in an opaque pic_world owned by the caller (World owns its fields and,
 * here, also its species, solver and collision model).  Calls on one world are not
 * re-entrant; work is issued on the world's own CUDA stream and the functions that return
 * host data synchronise that stream.  There is no CPU fallback: without a usable CUDA device
 * pic_world_create fails with PIC_ERR_CUDA.
 */
#ifndef PIC_GB300_H
#define PIC_GB300_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define PIC_OK 0
#define PIC_ERR_ARG 1           /* bad argument (the reference throws std::invalid_argument) */
#define PIC_ERR_CUDA 2          /* CUDA runtime error */
#define PIC_ERR_NOT_CONVERGED 3 /* solver stopped at max_it (reference solve() returns false) */
#define PIC_ERR_CAPACITY 4      /* a species ran out of capacity; particles were dropped */
#define PIC_ERR_DEVICE 5        /* a kernel reported a fault flag (bounded wait expired) */

typedef struct pic_world pic_world;

/* ---- World (ch4/v3/src/World.h:15-116) ------------------------------------------------ */

/* World(int ni, int nj, int nk, type_calc3 x0, type_calc3 xm)        World.h:63, World.cpp:22-26 */
int pic_world_create(pic_world** out, int ni, int nj, int nk, const double* x0, const double* xm, int device);
int pic_world_destroy(pic_world* w);
/* World::setTime(dt, num_ts)                                          World.cpp:321-324 */
int pic_world_set_time(pic_world* w, double dt, int num_ts);
/* World::advanceTime() -> *running = ts <= num_ts                     World.cpp:337-341 */
int pic_world_advance_time(pic_world* w, int* running);
/* World::getTs()                                                      World.cpp:328-330 */
int pic_world_get_ts(pic_world* w, int* ts);
/* World::getTime(): the sum of dt over the advanceTime calls          World.cpp:331-333, 337-341 */
int pic_world_get_time(pic_world* w, double* time);
/* Boundary set-up, replacing World::dirichletBoundries / addInlet / computeObjectID for the
 * domain faces (World.cpp:206-292).  periodic[3]: 1 makes an axis periodic (absent in the
 * reference).  face_mode[6] for faces -x,+x,-y,+y,-z,+z: 0 Neumann wall (reference v3 GS:
 * wall nodes copy their inner neighbour), 1 Dirichlet at face_phi[f].  Particles are absorbed
 * on every non-periodic face (World::inBounds, World.cpp:201-205). */
int pic_world_set_boundaries(pic_world* w, const int* periodic, const int* face_mode, const double* face_phi);
/* World::addObject<Rectangle>(pos, phi, sides) + computeObjectID     World.h:118-130, Object.cpp:231-238:
 * nodes inside the box are Dirichlet at phi; particles entering it are absorbed, or bounce and
 * are neutralised as pic_species_object_interaction sets. */
/* Stacked independent instances (no reference counterpart): the z nodes split into nslabs equal
 * slabs; each slab is one instance whose first and last node planes are Dirichlet electrodes at
 * phi_lo[s] and phi_hi[s] (the reference's cathode/anode planes), and the cell between two slabs
 * belongs to no instance (particles entering it are absorbed).  Every kernel launch then advances
 * all instances at once.  nslabs = 0 returns to a single instance. */
int pic_world_set_slabs(pic_world* w, int nslabs, const double* phi_lo, const double* phi_hi);
int pic_world_add_box(pic_world* w, const double* center, const double* sides, double phi);
/* public fields World::phi, rho, node_vol, ef, node_type, object_id  World.h:51-57
 * which: 0 phi, 1 rho, 2 node_vol, 3 ef (3 values per node), 4 node_type (World.h:17:
 * 0 REGULAR, 1 NEUMANN, 2 DIRICHLET), 5 object_id (1 on nodes inside a box, World.cpp:277-293).
 * Node arrays are x fastest: n = (k * nj + j) * ni + i. */
int pic_world_get_field(pic_world* w, int which, double* out);
int pic_world_set_field(pic_world* w, int which, const double* in); /* 0 phi, 1 rho, 3 ef */
/* World::getPE(): 0.5 eps0 sum |E|^2 node_vol in FP64                 World.cpp:108-119
 * (the duplicate last node plane of a periodic axis is not counted) */
int pic_world_potential_energy(pic_world* w, double* pe);

/* ---- Species (ch4/v3/src/Species.h:31-133) -------------------------------------------- */

/* Species(name, mass, charge, world, mpw0)                            Species.h:56
 * capacity: maximum macroparticles held on the device.  weight_bound: an upper bound of the
 * species' total macroweight; it fixes the 64-bit fixed-point scale of the density
 * accumulators (<= 0 picks capacity * mpw0 * 64). */
int pic_species_create(pic_world* w, const char* name, double mass, double charge, double mpw0, long capacity,
                       double weight_bound, int* species_id);
/* Species::addParticle(pos, vel, w) for n particles                   Species.cpp:420-434
 * rewind = 1: drop NaN / out-of-bounds / in-object particles and rewind v by q/m E dt/2 (as
 * the reference); rewind = 0: place as given (as the interactions' emplace_back).
 * ids may be NULL (sequential ids are assigned).  Arrays in pinned host memory (or in the
 * device's own memory) are read in place by the conversion kernel; pageable arrays go through
 * a device staging buffer. */
int pic_species_add_particles(pic_world* w, int sp, const double* pos, const double* vel, const double* wgt,
                              const uint64_t* ids, long n, int rewind);
/* Several species at once (no reference counterpart; the reference adds particles species by
 * species): entry k adds n[k] particles to species sps[k] as pic_species_add_particles does
 * (ids may be NULL, or hold NULL entries), and with sort = 1 sorts each species into cell order
 * (pic_species_sort) as soon as its upload is done.  When every array is device-readable in place
 * (pinned host or device memory), the uploads run on a side stream, so one species' sort overlaps
 * the next species' upload.  A species may appear once. */
int pic_species_add_particles_batch(pic_world* w, int count, const int* sps, const double* const* pos,
                                    const double* const* vel, const double* const* wgt, const uint64_t* const* ids,
                                    const long* n, int rewind, int sort);
/* Synthetic loader (GPU form of Species::loadParticleBoxThermal, Species.cpp:564-599): n
 * particles uniform in [lo, hi), Maxwellian at T [K], lognormal weights of mean w_mean and
 * log-sigma w_sigma (0: all w_mean), Philox stream keyed by seed. */
int pic_species_load_uniform(pic_world* w, int sp, const double* lo, const double* hi, long n, double T,
                             double w_mean, double w_sigma, uint64_t seed);
/* Species::loadParticleBoxThermal(x0, sides, num_den, T)             Species.cpp:564-599
 * floor(num_den * volume / mpw0) particles of weight mpw0, uniform in the box, speeds and
 * directions as sampleVth / sampleV3th (Species.cpp:855-869) with Philox draws. */
int pic_species_load_box_thermal(pic_world* w, int sp, const double* center, const double* sides, double num_den,
                                 double T, uint64_t seed);
/* Species::getNumParticles()                                          Species.cpp:43-45 */
int pic_species_count(pic_world* w, int sp, long* n);
/* Species::getConstPartRef(): host copy of the particles              Species.cpp:820-822 */
int pic_species_get_particles(pic_world* w, int sp, double* pos, double* vel, double* wgt, uint64_t* ids, long cap,
                              long* n);
/* The particle sample of Output::particlesOutput                     Outputs.cpp:207-245
 * particles 0, s, 2s, ... with s = n / num_out (all n when num_out > n), *n_out of them; pos and
 * vel hold 3 * num_out values.  Particles are in device storage order (by cell after a sort). */
int pic_species_sample_particles(pic_world* w, int sp, long num_out, double* pos, double* vel, long* n_out);
/* Species::advanceElectrons / advanceNonElectron (dt)                 Species.cpp:258-399, 47-256
 * One leapfrog push; with deposit = 1 the weight is also scattered at the new position, which
 * is Species::computeNumberDensity (Species.cpp:401-416) fused into the push. */
int pic_species_push(pic_world* w, int sp, double dt, int deposit);
/* What a push does with particles that enter a box object (pic_world_add_box).
 * mode 0 (default): they are removed, as in Species::advanceElectrons (Species.cpp:369-388).
 * mode 1: Species::advanceNonElectron(neutrals, spherium, dt) (Species.cpp:45-256): a neutral
 * species (charge 0) bounces diffusely off the object (sampleReflectedVelocity, full
 * accommodation at 300 K, Species.cpp:835-861), up to 20 moves per push; an ion is removed and
 * leaves (int)(w / mpw0_n + u) particles of neutral_sp at the impact point, plus, with
 * sputtering (Config::SPUTTERING), (int)(0.1 w / mpw0_s + u) of spherium_sp when it hit faster
 * than 5 km/s; both are added with Species::addParticle semantics (bounds and objects checked,
 * the target species' half-step rewind).  Draws: Philox streams keyed by (seed, particle id, step). */
int pic_species_object_interaction(pic_world* w, int sp, int mode, int neutral_sp, int spherium_sp, int sputtering,
                                   uint64_t seed);
/* counters since mode 1 was set: impacts, bounces, neutrals created, sputtered particles created */
int pic_species_object_stats(pic_world* w, int sp, uint64_t* out);
/* Species::computeNumberDensity() alone (deposit without moving)      Species.cpp:401-416 */
int pic_species_number_density(pic_world* w, int sp);
/* Species::den (public field) after pic_charge_density                Species.h:49 */
int pic_species_get_den(pic_world* w, int sp, double* out);
/* Species::den_avg and Species::updateAverages()                      Species.cpp:764-766 */
int pic_species_update_averages(pic_world* w, int sp);
int pic_species_get_den_avg(pic_world* w, int sp, double* out);
/* Species::sortIndexes(): reorder particles by cell; counts per cell  Species.cpp:905-915, 813-819
 * (macro_part_count) are written to cell_counts when it is not NULL (length num_cells). */
int pic_species_sort(pic_world* w, int sp, int32_t* cell_counts);
/* Species::getMicroCount / getMomentum / getKE in FP64                Species.cpp:732-752
 * out[0] sum w, out[1..3] mass * sum w v, out[4] 0.5 mass sum w v.v */
int pic_species_sums(pic_world* w, int sp, double* out);

/* Species::sampleMoments (Species.cpp:767-776): CIC scatter of n, n v, n u^2, n v^2, n w^2,
 * accumulated across calls (FP32 atomics, a diagnostic); Species::clearSamples (805-812);
 * Species::computeGasProperties (777-804): vel (3 per node) and T per node on the host. */
int pic_species_sample_moments(pic_world* w, int sp);
int pic_species_clear_samples(pic_world* w, int sp);
int pic_species_gas_properties(pic_world* w, int sp, double* vel, double* T);

/* World::computeChargeDensity(species): den_s and rho = sum q_s den_s  World.cpp:193-200 */
int pic_charge_density(pic_world* w);

/* ---- Sources (ch4/v3/src/Source.h:13-68, Source.cpp) ------------------------------------ */

/* ColdBeamSource(species, world, v_drift, den, face) (T = 0) and
 * WarmBeamSource(species, world, v_drift, den, T, face)               Source.cpp:3-30, 105-110
 * face: 0..5 for x-, x+, y-, y+, z-, z+ (inletName2Index, World.cpp:369-390); the face may not lie
 * on a periodic axis.  Like the reference constructor (World::addInlet, World.cpp:206-260) the
 * inlet face becomes Dirichlet at 0 V.  Draws are Philox streams keyed by seed. */
int pic_source_create(pic_world* w, int sp, double v_drift, double den, double T, int face, uint64_t seed,
                      int* source_id);
/* Source::sample() (Source.cpp:99-102, 186-190): (int)(den v_drift A dt / mpw0 + u) particles of
 * weight mpw0 on the inlet face (the + faces one cell in), the two other coordinates uniform,
 * velocity v_drift along the inward normal plus, for a warm beam, Species::sampleV3th(T); added
 * with Species::addParticle semantics (bounds and objects checked, velocity rewound by half a
 * step).  pic_step samples every source at the start of the step (main.cpp:196-198). */
int pic_source_sample(pic_world* w, int source_id);

/* ---- PotentialSolver (ch4/v3/src/PotentialSolver.h:26-88) ----------------------------- */

#define PIC_SOLVER_RBSOR 0 /* red-black SOR, FP32 sweeps in FP64 refinement (replaces GS) */
#define PIC_SOLVER_PCG 1   /* flexible Jacobi-PCG, FP32 iterations in FP64 refinement (replaces NR-PCG) */
#define PIC_SOLVER_LEARNED 2 /* flexible CG with the learned multilevel preconditioner, FP32 iterations in
                              * FP64 refinement (no reference counterpart) */
/* PotentialSolver(world, max_it, tolerance, SolverType)               PotentialSolver.cpp:44-52
 * Stopping rule: FP64 ||b - L phi||_2 / ||b||_2 <= tol_rel unless pic_solver_set_stop chose
 * another (the reference stops on an absolute RMS residual).  omega is the SOR weight
 * (reference 1.4). */
int pic_solver_configure(pic_world* w, int method, double tol_rel, int max_it, double omega);
/* PotentialSolver::solve()                                            PotentialSolver.cpp:55-67
 * iters: inner sweeps / iterations; rel: final FP64 relative residual.
 * Returns PIC_ERR_NOT_CONVERGED when max_it is reached (reference: solve() == false). */
int pic_solver_solve(pic_world* w, int* iters, double* rel);
/* PotentialSolver::computeEF()                                        PotentialSolver.cpp:354-408 */
int pic_solver_compute_ef(pic_world* w);
/* Stopping rule of pic_solver_solve (the tolerance set here replaces pic_solver_configure's):
 *   PIC_STOP_REL_RHS     ||b - L phi||_2 <= tol ||b||_2 (the default)
 *   PIC_STOP_ABS_RMS     sqrt(||b - L phi||_2^2 / nv) <= tol, the reference's own rule: the GS
 *                        check (PotentialSolver.cpp:150-158) and vec::norm of PCG
 *                        (PotentialSolver.cpp:36-38, 300) divide the squared residual by the
 *                        node count
 *   PIC_STOP_REL_CHARGE  ||b - L phi||_2 <= tol min(||b||_2, ||rho/eps0||_2): relative to the
 *                        space-charge part of b as well, so that a large Dirichlet (electrode)
 *                        term in b cannot hide an unresolved space-charge potential
 * (no reference counterpart for the relative rules).  rel of pic_solver_solve is the residual
 * norm over the rule's scale. */
#define PIC_STOP_REL_RHS 0
#define PIC_STOP_ABS_RMS 1
#define PIC_STOP_REL_CHARGE 2
int pic_solver_set_stop(pic_world* w, int rule, double tol);
/* Start of a warm solve (phi unchanged since the last solve), no reference counterpart:
 *   PIC_WARM_PREVIOUS     the last potential, as the reference's solvers continue from world.phi
 *   PIC_WARM_EXTRAPOLATE  the last potential plus the last warm solve's whole change (linear
 *                         extrapolation in time: ballistic particles change rho almost linearly
 *                         from step to step); one float-float residual pass evaluates it
 * Either way the solve ends at the same certified residual. */
#define PIC_WARM_PREVIOUS 0
#define PIC_WARM_EXTRAPOLATE 1
int pic_solver_set_warm_start(pic_world* w, int mode);
/* Jacobi-PCG iterations that a warm solve of PIC_SOLVER_LEARNED runs before the learned
 * preconditioner takes over (default 16; 0: none).  They remove the high-frequency part of a
 * warm residual at a quarter of the cost of a learned iteration.  No reference counterpart. */
int pic_solver_set_warm_jacobi(pic_world* w, int iterations);
/* ||b - L phi||_2, ||b||_2 and ||rho/eps0||_2 (FREE nodes) of the last solve's final residual
 * (no reference counterpart) */
int pic_solver_last_norms(pic_world* w, double* out3);
/* cumulative solver work since creation: solves, FP64 refinements (residual evaluations) and
 * inner FP32 sweeps / iterations (no reference counterpart; the reference prints progress) */
int pic_solver_stats(pic_world* w, long* solves, long* refinements, long* inner_iterations);

/* ---- learned multilevel preconditioner (no reference counterpart) ----------------------
 * B r = sum_l P^l o_l over a box hierarchy (level 0 = the distinct nodes; each level halves the
 * previous one, rounding up), cell-centred trilinear prolongation P, restriction P^T; level 0
 * applies a learned 3x3x3 stencil, levels 1-4 a linear 3-D convolutional network (lift 1->C,
 * mix CxC, projection C->1; C = 16, 32, 64, 64), deeper levels the inverse Galerkin diagonal.
 * The weights start as the BPX preconditioner.  Created on first use for the world's grid. */
/* number of levels, their extents (x, y, z per level, up to 12 levels) and Galerkin diagonals */
int pic_learned_levels(pic_world* w, int* nlev, int* dims, double* diag);
/* restores the starting (BPX) weights */
int pic_learned_reset(pic_world* w);
/* copies the FP32 parameters out (out may be NULL to query the count) or in: the level-0
 * stencil [27], then per network level lift [C][27], mix [C][C] (out, in), projection [27][C] */
int pic_learned_weights(pic_world* w, float* out, long capacity, long* count);
int pic_learned_set_weights(pic_world* w, const float* in, long count);
/* z = B r for host arrays of all nodes (r is read on FREE nodes; z is zero elsewhere) */
int pic_learned_apply(pic_world* w, const double* r, double* z);
/* Training.  Loss of a pair (r, x) with L x = r: (B r - x)^T L (B r - x) / x^T L x, its gradient
 * by the library's own forward and backward kernels (tensor-core GEMMs, BF16 operands, FP32
 * accumulation).  loss_grad evaluates one pair (host arrays of all nodes, read on FREE nodes)
 * and returns the loss and the gradient in the parameter layout, without updating. */
int pic_learned_loss_grad(pic_world* w, const double* r, const double* x, double* loss, float* grad);
/* collect (first residual, total correction) of every PCG / learned solve as a training pair
 * (the last four are kept) */
int pic_learned_collect(pic_world* w, int on);
/* steps of Adam (learning rate lr relative to each parameter group's size); a step uses a
 * collected pair when one exists and step % pair_every == 0, else a white-noise pair.  The round
 * is judged by the solver: val_iters[0..1] = iterations of a validation solve before and after;
 * a round that needs more iterations is rolled back (*accepted = 0). */
int pic_learned_train(pic_world* w, int steps, double lr, int pair_every, double* mean_loss, int* val_iters,
                      int* accepted);
/* Level-gain calibration, learned by the solver itself: the level-0 stencil gain (doubling, then a
 * half-octave refinement) and each network level's gain (0.5 .. 2, applied to lift and projection
 * alike so B stays symmetric) are kept only if a validation solve (the right-hand side of the last
 * collected solve, else white noise) needs fewer iterations.  val_iters[2]: before, after. */
int pic_learned_calibrate(pic_world* w, int* val_iters);

/* ---- Interaction: MC_MEX_Ionization (ch4/v3/src/Interactions.h:98-143) ------------------
 * Background-gas form: the neutral species is a uniform Maxwellian gas (density n_neutral,
 * temperature T_neutral, mass m_neutral) instead of macroparticles.  sigma_coll is a table
 * (E [eV], sigma [m^2]) interpolated as evaluateSigmaColl (Interactions.cpp:541-558).
 * sigma_ion_kind 0: the reference fit a*ln(E/b)/E*exp(-c/E) (Interactions.cpp:559-566) with
 * (p0,p1,p2) = (a,b,c); 1: Lotz form A*ln(E/I)/(E*I)*(1-b*exp(-c*(E/I-1))) with
 * (p0,p1,p2,p3) = (A,b,c,unused).  E_ion_eV is the threshold, B_inc the Opal energy-sharing
 * constant (Interactions.cpp:511).  Collisions use Philox streams keyed by (seed, step, id). */
int pic_mcc_create(pic_world* w, int electrons, int ions, double n_neutral, double T_neutral, double m_neutral,
                   double E_ion_eV, double B_inc, int sigma_ion_kind, const double* sigma_ion_params,
                   const double* table_E, const double* table_s, int table_n, uint64_t seed);
/* Interaction::apply(dt): collisions of every electron for the current step (no push). */
int pic_mcc_apply(pic_world* w, double dt);
/* background density per instance slab (one value per slab of pic_world_set_slabs) */
int pic_mcc_set_slab_density(pic_world* w, int nslabs, const double* n_neutral);
/* counters since creation: candidates, collisions, ionisations, products lost */
int pic_mcc_stats(pic_world* w, uint64_t* out);

/* ---- DSMC_MEX: VHS particle-particle collisions (ch4/v3/src/Interactions.h:42-66) ------ */
/* DSMC_MEX(species, world) when sp2 < 0 or sp2 == sp1 (Interactions.cpp:143-157), else
 * DSMC_MEX(species1, species2, world) (Interactions.cpp:158-177), which requires equal mpw0
 * (PIC_ERR_ARG otherwise, as the reference throws).  Bird's VHS cross-section with d = 4.07e-10
 * m, omega = 0.77 at 273.15 K; (sigma v)_max starts at 1e-14.  Pairs are drawn per cell from
 * Philox streams keyed by (seed, cell, call).  pic_step applies every interaction each step,
 * before the pushes, in creation order (main.cpp:201-203). */
int pic_dsmc_create(pic_world* w, int sp1, int sp2, uint64_t seed, int* dsmc_id);
/* DSMC_MEX::apply(dt) (Interactions.cpp:180-257): sorts the species into cell order, then
 * collides pairs in every cell; (sigma v)_max is updated on the device (no host round trip). */
int pic_dsmc_apply(pic_world* w, int dsmc_id, double dt);
/* counts[0] collisions, counts[1] candidate pairs since creation; the current (sigma v)_max */
int pic_dsmc_stats(pic_world* w, int dsmc_id, uint64_t* counts, double* sigma_v_rel_max);

/* ---- the step loop (ch4/v3/src/main.cpp:177-286) -------------------------------------- */

/* Loop options.  solve_each_step: Poisson + E every step (v3 comments it out, main.cpp:260-261;
 * ch2 solves every step).  sort_every: every k steps, a counting sort by cell of each species of
 * which at least 2 % of the particles changed cell or were appended since its last sort.  subcycle[sp]:
 * push species sp every k steps with k*dt (main.cpp:211-238); 1 = every step.
 * merge_every/merge_after/merge_min: merging (main.cpp:179: ts > 250 && ts % 50 == 0). */
int pic_loop_configure(pic_world* w, int solve_each_step, int sort_every, const int* subcycle, int merge_every,
                       int merge_after, int merge_min);
/* Autotuner (no reference counterpart): measures launch shapes on the world's own data and keeps
 * the fastest for the rest of the run: the CTA count of the streaming node kernels (2 to 16 per
 * SM, timed on the float-float residual), that of the CG stencil kernels (d = z + beta d, q = L d;
 * same range, timed on the learned-CG one) and the push's CTAs per SM (1 to the occupancy limit,
 * timed on pushes with dt = 0, which leave the particles and their deposit as they are).  Call it
 * once the world holds its particles and fields; the next solve starts from a full residual.
 * Outputs may be NULL. */
int pic_autotune(pic_world* w, int* push_ctas_per_sm, int* node_grid);
/* The launch shapes in use (no reference counterpart): push CTAs per SM, CTAs of the streaming
 * node kernels and of the CG stencil kernels (0: the built-in default).  Outputs may be NULL. */
int pic_launch_shapes(pic_world* w, int* push_ctas_per_sm, int* node_grid, int* cg_grid);
/* Sets the launch shapes, e.g. the ones pic_launch_shapes reported after pic_autotune on an earlier
 * world of the same size (no reference counterpart).  push_ctas_per_sm: 1 to the push's occupancy
 * limit; node_grid, cg_grid: CTA counts (a launch takes at most one CTA per 1024 nodes); 0 keeps
 * the built-in default for that shape.  PIC_ERR_ARG for a negative value or too many push CTAs. */
int pic_set_launch_shapes(pic_world* w, int push_ctas_per_sm, int node_grid, int cg_grid);
/* one iteration of the time loop: advanceTime, [merge], collisions + push + deposit,
 * compaction, [averages], charge density, [solve + E], [sort] */
int pic_step(pic_world* w);
/* velocity-binned merge (Species::merge, Species.cpp:981-1145) of cells holding at least
 * min_count particles; sorts the species first */
int pic_species_merge(pic_world* w, int sp, int min_count);
/* merge counters since creation: bins merged, particles removed, products dropped (NaN) */
int pic_merge_stats(pic_world* w, uint64_t* out);

/* ---- number density without device allocation -------------------------------------
 * No counterpart in the reference.  For callers that cannot allocate device memory: plugins
 * whose host application owns all device memory through its own allocator, and real-time loops
 * that forbid allocation after start-up.  It computes the number density of one species from
 * particle arrays the caller already holds on the current device, in the library's layout
 * (pos4: float4 {ox, oy, oz, packed cell i | j<<9 | k<<18}; vel4: float4 {vx, vy, vz, w}), and
 * writes it to den_out (FP32, one value per node, node order as above).  The deposit uses the
 * same CIC weights and 64-bit fixed-point rounding as this library's fused push deposit, with
 * fixed-point scale `scale` (rounded to FP32); scale times the weight summed at any one node
 * must stay below 2^63.  Grids are limited to 513 x 513 x 8193 nodes, as pic_world_create, and
 * a periodic axis needs at least 4 nodes.
 * The working accumulator is a library-owned device array of 2^20 nodes (8 MiB per GPU, held
 * until exit); larger grids are rejected with PIC_ERR_ARG.  No allocation is made.  The first
 * call on a device looks up that array's address and should come before any stream capture.
 * All calls share the array, which keeps the last call's contents (each call clears it first):
 * calls that overlap on the GPU race.  Work is queued on `stream` (a cudaStream_t, NULL for the
 * default stream) and not waited for; an error the caller left pending is not cleared. */
int pic_number_density_noalloc(int ni, int nj, int nk, const double* x0, const double* xm, const int* periodic,
                               const void* pos4, const void* vel4, long n, double scale, float* den_out,
                               void* stream);

/* ---- runtime ------------------------------------------------------------------------- */
int pic_synchronize(pic_world* w);
/* Test hook, no reference counterpart: how many times a kernel's first wait for a bulk copy
 * (the push) or for tensor-core MMAs (training) polls its mbarrier before it gives up, records
 * the fault and returns (pic_synchronize then returns PIC_ERR_DEVICE).  polls < 0 restores the
 * default 2^24; 0 makes every such wait give up at once.  The wait for the copies or MMAs still
 * in flight after a timeout always keeps the full limit, so no copy outlives its block.  The
 * tensor-core setting applies to the current device. */
int pic_debug_set_wait_polls(pic_world* w, long long polls);
/* message of the last failing call on this thread (empty if none) */
int pic_last_error(char* buf, int len);
/* per-kernel CUDA-event timing: enable, then read accumulated milliseconds and launch counts
 * of the named kernel groups ("push", "deposit", "rho", "poisson", "efield", "sort", ...). */
int pic_timing_enable(pic_world* w, int on);
int pic_timing_read(pic_world* w, const char* name, double* ms, long* launches);
int pic_timing_reset(pic_world* w);
/* kernels launched on this world since creation */
int pic_launch_count(pic_world* w, long* n);
/* the CUDA stream (cudaStream_t) the world issues its work on */
int pic_world_stream(pic_world* w, void** stream);

#ifdef __cplusplus
}
#endif
#endif
