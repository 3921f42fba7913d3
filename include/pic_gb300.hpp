// pic_gb300.hpp -- header-only C++ facade with the reference's class surface over the C ABI.
//
// A ch4/v3-style driver (ch4/v3/src/main.cpp) keeps its shape: World, Species,
// PotentialSolver and an Interaction with apply(dt), with the same member names.  The
// particles live on the GPU, so Species::getPartRef() returns a host copy instead of a
// mutable reference (Species.cpp:823-825), and the Poisson tolerance is the FP64 relative
// residual.  Errors throw like the reference: std::invalid_argument for bad arguments,
// std::runtime_error for device failures.
#ifndef PIC_GB300_HPP
#define PIC_GB300_HPP
#include <array>
#include <cctype>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <iostream>
#include <stdexcept>
#include <string>
#include <vector>
#include "pic_gb300.h"

namespace pic_gb300 {

using type_calc = double;
using type_calc3 = std::array<double, 3>;

inline void check(int rc) {
    if (rc == PIC_OK) return;
    char buf[512];
    pic_last_error(buf, sizeof(buf));
    if (rc == PIC_ERR_ARG) throw std::invalid_argument(buf);
    throw std::runtime_error(std::string("pic_gb300: ") + buf);
}

struct Particle {  // ch4/v3/src/Species.h:12-29 (host copy)
    type_calc3 pos, vel;
    type_calc macro_weight;
    uint64_t id;
};

enum SolverType { GS = PIC_SOLVER_RBSOR, PCG = PIC_SOLVER_PCG };  // PotentialSolver.h:24

class Species;

class World {  // ch4/v3/src/World.h:15-116
public:
    const int ni, nj, nk, nv, num_cells;
    World(int ni_, int nj_, int nk_, type_calc3 x0, type_calc3 xm, int device = 0)
        : ni(ni_), nj(nj_), nk(nk_), nv(ni_ * nj_ * nk_), num_cells((ni_ - 1) * (nj_ - 1) * (nk_ - 1)), x0_(x0),
          time_start_(std::chrono::high_resolution_clock::now()) {
        check(pic_world_create(&h_, ni, nj, nk, x0.data(), xm.data(), device));
        const int nn[3] = {ni, nj, nk};
        for (int d = 0; d < 3; d++) dx_[d] = (xm[d] - x0[d]) / (nn[d] - 1);  // World.cpp:58-66
    }
    World(const World&) = delete;
    World& operator=(const World&) = delete;
    ~World() { pic_world_destroy(h_); }
    pic_world* handle() const { return h_; }
    void setTime(type_calc dt, int num_ts) {
        dt_ = dt;
        num_ts_ = num_ts;
        check(pic_world_set_time(h_, dt, num_ts));
    }
    type_calc getDt() const { return dt_; }
    bool advanceTime() {
        int r = 0;
        check(pic_world_advance_time(h_, &r));
        return r != 0;
    }
    int getTs() const {
        int t = 0;
        check(pic_world_get_ts(h_, &t));
        return t;
    }
    type_calc getTime() const {  // World.cpp:331-333
        double t = 0;
        check(pic_world_get_time(h_, &t));
        return t;
    }
    bool isLastTimeStep() const { return getTs() == num_ts_ - 1; }
    type_calc getWallTime() const {  // seconds since construction or setTimeStart, World.cpp:342-346
        return std::chrono::duration<double>(std::chrono::high_resolution_clock::now() - time_start_).count();
    }
    void setTimeStart() { time_start_ = std::chrono::high_resolution_clock::now(); }
    type_calc3 getX0() const { return x0_; }
    type_calc3 getDx() const { return dx_; }
    type_calc getCellVolume() const { return dx_[0] * dx_[1] * dx_[2]; }
    int getNumCells() const { return num_cells; }
    type_calc getPE() const {  // World.cpp:108-119, summed on the device
        double pe = 0;
        check(pic_world_potential_energy(h_, &pe));
        return pe;
    }
    // World.cpp:167-191: steady once the total real count, |momentum| sum and energy all change
    // by less than 1e-3 (relative) between two calls
    template <class V>
    bool steadyState(V& species);
    bool steadyState() const { return steady_state_; }
    void dirichletBoundries(type_calc phi = 0) {  // World.cpp:263-274
        int per[3] = {0, 0, 0}, mode[6] = {1, 1, 1, 1, 1, 1};
        double val[6] = {phi, phi, phi, phi, phi, phi};
        check(pic_world_set_boundaries(h_, per, mode, val));
    }
    void setBoundaries(const int periodic[3], const int face_mode[6], const double face_phi[6]) {
        check(pic_world_set_boundaries(h_, periodic, face_mode, face_phi));
    }
    void addBox(type_calc3 pos, type_calc phi, type_calc3 sides) {  // addObject<Rectangle>(pos, phi, sides)
        check(pic_world_add_box(h_, pos.data(), sides.data(), phi));
    }
    std::vector<double> phi() const { return field(0, 1); }
    std::vector<double> rho() const { return field(1, 1); }
    std::vector<double> node_vol() const { return field(2, 1); }
    std::vector<double> ef() const { return field(3, 3); }
    std::vector<double> node_type() const { return field(4, 1); }  // World.h:17: REGULAR, NEUMANN, DIRICHLET
    std::vector<double> object_id() const { return field(5, 1); }
    void setPhi(const std::vector<double>& v) { check(pic_world_set_field(h_, 0, v.data())); }
    // launch shapes (no reference counterpart): measured on this world's data (pic_autotune), read,
    // or carried over from an earlier world of the same size; {push CTAs per SM, node-kernel CTAs,
    // CG-stencil CTAs}, 0 = built-in default
    void autotune() { check(pic_autotune(h_, nullptr, nullptr)); }
    std::array<int, 3> launchShapes() const {
        std::array<int, 3> s{};
        check(pic_launch_shapes(h_, &s[0], &s[1], &s[2]));
        return s;
    }
    void setLaunchShapes(const std::array<int, 3>& s) { check(pic_set_launch_shapes(h_, s[0], s[1], s[2])); }
    void computeChargeDensity() { check(pic_charge_density(h_)); }  // World.cpp:193-200
    template <class V>
    void computeChargeDensity(V&) {
        computeChargeDensity();
    }

private:
    std::vector<double> field(int which, int comps) const {
        std::vector<double> out((size_t)nv * comps);
        check(pic_world_get_field(h_, which, out.data()));
        return out;
    }
    pic_world* h_ = nullptr;
    type_calc dt_ = 1e-4;
    int num_ts_ = 0;
    type_calc3 x0_{}, dx_{};
    std::chrono::high_resolution_clock::time_point time_start_;
    bool steady_state_ = false;
    type_calc last_mass_ = 0, last_mom_ = 0, last_en_ = 0;
};

class Species {  // ch4/v3/src/Species.h:31-133
public:
    const std::string name;
    const type_calc mass, charge, mpw0;
    // host copies of the reference's public fields, filled by the calls that compute them
    std::vector<double> vel, T;                // computeGasProperties
    std::vector<int32_t> macro_part_count;     // computeMacroParticlesCount
    Species(std::string name_, type_calc mass_, type_calc charge_, World& world, type_calc mpw0_,
            long capacity = 1 << 20, double weight_bound = 0)
        : name(name_), mass(mass_), charge(charge_), mpw0(mpw0_), world_(&world) {
        check(pic_species_create(world.handle(), name.c_str(), mass, charge, mpw0, capacity, weight_bound, &id_));
    }
    int id() const { return id_; }
    size_t getNumParticles() const {
        long n = 0;
        check(pic_species_count(world_->handle(), id_, &n));
        return (size_t)n;
    }
    void addParticle(type_calc3 pos, type_calc3 vel, type_calc w) {  // Species.cpp:420-434
        check(pic_species_add_particles(world_->handle(), id_, pos.data(), vel.data(), &w, nullptr, 1, 1));
    }
    void addParticle(type_calc3 pos, type_calc3 vel) { addParticle(pos, vel, mpw0); }
    void addParticles(const std::vector<double>& pos, const std::vector<double>& vel, const std::vector<double>& w,
                      bool rewind = true) {
        check(pic_species_add_particles(world_->handle(), id_, pos.data(), vel.data(), w.data(), nullptr,
                                        (long)w.size(), rewind ? 1 : 0));
    }
    void loadUniform(type_calc3 lo, type_calc3 hi, long n, type_calc T, type_calc w_mean, type_calc w_sigma,
                     uint64_t seed) {
        check(pic_species_load_uniform(world_->handle(), id_, lo.data(), hi.data(), n, T, w_mean, w_sigma, seed));
    }
    // objects absorb electrons (Species.cpp:369-388)
    void advanceElectrons(type_calc dt) {
        setObjectInteraction(0, -1, -1, false);
        check(pic_species_push(world_->handle(), id_, dt, 1));
    }
    // neutrals bounce off objects, ions are neutralised into `neutrals` and, with
    // Config::SPUTTERING, sputter into `spherium` (Species.cpp:45-256)
    void advanceNonElectron(Species& neutrals, Species& spherium, type_calc dt);
    // counters of mode 1: impacts, bounces, neutrals created, sputtered particles created
    std::array<uint64_t, 4> objectStats() const {
        std::array<uint64_t, 4> s{};
        check(pic_species_object_stats(world_->handle(), id_, s.data()));
        return s;
    }
    void computeNumberDensity() { check(pic_species_number_density(world_->handle(), id_)); }
    void updateAverages() { check(pic_species_update_averages(world_->handle(), id_)); }
    void sortIndexes() { check(pic_species_sort(world_->handle(), id_, nullptr)); }
    // Species.cpp:813-819; the counts stay in macro_part_count (a cell field, x fastest)
    const std::vector<int32_t>& computeMacroParticlesCount() {
        macro_part_count.assign((size_t)world_->num_cells, 0);
        check(pic_species_sort(world_->handle(), id_, macro_part_count.data()));
        return macro_part_count;
    }
    void merge(int min_count = 10) { check(pic_species_merge(world_->handle(), id_, min_count)); }
    std::vector<double> den() const {
        std::vector<double> d((size_t)world_->nv);
        check(pic_species_get_den(world_->handle(), id_, d.data()));
        return d;
    }
    std::vector<double> den_avg() const {  // Species.h:50
        std::vector<double> d((size_t)world_->nv);
        check(pic_species_get_den_avg(world_->handle(), id_, d.data()));
        return d;
    }
    void sampleMoments() { check(pic_species_sample_moments(world_->handle(), id_)); }  // Species.cpp:767-776
    void clearSamples() { check(pic_species_clear_samples(world_->handle(), id_)); }    // Species.cpp:805-812
    // Species.cpp:777-804: stream velocity (3 per node) into vel and temperature into T
    void computeGasProperties() {
        vel.assign((size_t)world_->nv * 3, 0.0);
        T.assign((size_t)world_->nv, 0.0);
        check(pic_species_gas_properties(world_->handle(), id_, vel.data(), T.data()));
    }
    // every (n / num)-th particle, the sample Output::particlesOutput writes (Outputs.cpp:207-245)
    std::vector<Particle> sampleParticles(long num) const {
        std::vector<double> pos((size_t)num * 3), v((size_t)num * 3);
        long got = 0;
        check(pic_species_sample_particles(world_->handle(), id_, num, pos.data(), v.data(), &got));
        std::vector<Particle> out((size_t)got);
        for (long p = 0; p < got; p++)
            out[p] = {{pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]}, {v[3 * p], v[3 * p + 1], v[3 * p + 2]}, 0.0, 0};
        return out;
    }
    type_calc getMicroCount() const { return sums()[0]; }
    type_calc3 getMomentum() const {
        auto s = sums();
        return {s[1], s[2], s[3]};
    }
    type_calc getKE() const { return sums()[4]; }
    std::vector<Particle> getPartRef() const {
        size_t n = getNumParticles();
        std::vector<double> pos(3 * n + 3), vel(3 * n + 3), w(n + 1);
        std::vector<uint64_t> ids(n + 1);
        long got = 0;
        check(pic_species_get_particles(world_->handle(), id_, pos.data(), vel.data(), w.data(), ids.data(),
                                        (long)n + 1, &got));
        std::vector<Particle> out((size_t)got);
        for (long p = 0; p < got; p++)
            out[p] = {{pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]}, {vel[3 * p], vel[3 * p + 1], vel[3 * p + 2]}, w[p], ids[p]};
        return out;
    }

private:
    std::array<double, 5> sums() const {
        std::array<double, 5> s{};
        check(pic_species_sums(world_->handle(), id_, s.data()));
        return s;
    }
    void setObjectInteraction(int mode, int neu, int spu, bool sputtering) {
        const std::array<int, 4> key{mode, neu, spu, sputtering ? 1 : 0};
        if (key == obj_key_) return;
        check(pic_species_object_interaction(world_->handle(), id_, mode, neu, spu, sputtering ? 1 : 0,
                                             0x0B1EC7ull + 7919ull * (uint64_t)id_));
        obj_key_ = key;
    }
    World* world_;
    int id_ = -1;
    std::array<int, 4> obj_key_{0, -1, -1, 0};
};

// the reference's configuration singleton (ch4/v3/src/Config.h:6-45), for the switch the pushes read
class Config {
public:
    static Config& getInstance() {
        static Config c;
        return c;
    }
    bool setSPUTTERING(bool option) {
        sputtering_ = option;
        return sputtering_;
    }
    bool getSPUTTERING() const { return sputtering_; }

private:
    bool sputtering_ = false;
};

inline void Species::advanceNonElectron(Species& neutrals, Species& spherium, type_calc dt) {
    const bool sput = Config::getInstance().getSPUTTERING();
    setObjectInteraction(1, charge != 0 ? neutrals.id() : -1, charge != 0 && sput ? spherium.id() : -1,
                         charge != 0 && sput);
    check(pic_species_push(world_->handle(), id_, dt, 1));
}

namespace detail {
inline Species& sp_ref(Species& s) { return s; }
inline Species& sp_ref(Species* s) { return *s; }
}  // namespace detail

// One species' particles for addParticlesBatch: n positions and velocities (x, y, z each) and
// weights in FP64; pinned host or device memory is read in place.
struct ParticleArrays {
    const double* pos;
    const double* vel;
    const double* w;
    long n;
};
// Several species at once, each sorted into cell order as soon as its upload is done, its sort
// beside the next species' upload (no reference counterpart: pic_species_add_particles_batch)
inline void addParticlesBatch(World& world, const std::vector<Species*>& species,
                              const std::vector<ParticleArrays>& arrays, bool rewind = true, bool sort = true) {
    if (species.size() != arrays.size()) throw std::invalid_argument("addParticlesBatch: one array set per species");
    std::vector<int> ids;
    std::vector<const double*> pos, vel, w;
    std::vector<long> n;
    for (size_t k = 0; k < species.size(); k++) {
        ids.push_back(species[k]->id());
        pos.push_back(arrays[k].pos);
        vel.push_back(arrays[k].vel);
        w.push_back(arrays[k].w);
        n.push_back(arrays[k].n);
    }
    check(pic_species_add_particles_batch(world.handle(), (int)ids.size(), ids.data(), pos.data(), vel.data(),
                                          w.data(), nullptr, n.data(), rewind ? 1 : 0, sort ? 1 : 0));
}

template <class V>
bool World::steadyState(V& species) {
    if (steady_state_) return true;
    type_calc tot_mass = 0, tot_mom = 0, tot_en = getPE();
    for (auto& x : species) {
        Species& sp = detail::sp_ref(x);
        tot_mass += sp.getMicroCount();
        type_calc3 m = sp.getMomentum();
        tot_mom += std::sqrt(m[0] * m[0] + m[1] * m[1] + m[2] * m[2]);
        tot_en += sp.getKE();
    }
    const type_calc tol = 1e-3;
    if (std::fabs((tot_mass - last_mass_) / tot_mass) < tol && std::fabs(tot_mom - last_mom_) / tot_mom < tol &&
        std::fabs(tot_en - last_en_) / tot_en < tol) {
        steady_state_ = true;
        std::cout << "\nSteady state reached at time step " << getTs() << std::endl;
    }
    last_mass_ = tot_mass;
    last_mom_ = tot_mom;
    last_en_ = tot_en;
    return steady_state_;
}

class PotentialSolver {  // ch4/v3/src/PotentialSolver.h:26-88
public:
    PotentialSolver(World& world, unsigned max_solver_it, type_calc tolerance, SolverType type, double omega = 1.4)
        : world_(&world) {
        check(pic_solver_configure(world.handle(), (int)type, tolerance, (int)max_solver_it, omega));
    }
    bool solve() {  // PotentialSolver.cpp:55-67: false when not converged
        int rc = pic_solver_solve(world_->handle(), &iters_, &rel_);
        if (rc == PIC_ERR_NOT_CONVERGED) return false;
        check(rc);
        return true;
    }
    void computeEF() { check(pic_solver_compute_ef(world_->handle())); }
    // only the reference's n0 = 0 case (main.cpp:138) is supported: no Boltzmann electrons
    void setReferenceValues(type_calc, type_calc n0, type_calc) {
        if (n0 != 0) throw std::invalid_argument("Boltzmann-electron term is not supported (n0 must be 0)");
    }
    int iterations() const { return iters_; }
    double relativeResidual() const { return rel_; }
    // stopping rule PIC_STOP_*; PIC_STOP_ABS_RMS is the reference's own absolute RMS residual
    // (PotentialSolver.cpp:150-158), the relative rules have no reference counterpart
    void setStopRule(int rule, type_calc tolerance) { check(pic_solver_set_stop(world_->handle(), rule, tolerance)); }
    // start of warm solves: PIC_WARM_PREVIOUS (the reference's) or PIC_WARM_EXTRAPOLATE
    void setWarmStart(int mode) { check(pic_solver_set_warm_start(world_->handle(), mode)); }
    // ||b - L phi||_2, ||b||_2 and ||rho/eps0||_2 of the last solve's final residual
    void lastNorms(double out[3]) const { check(pic_solver_last_norms(world_->handle(), out)); }

private:
    World* world_;
    int iters_ = 0;
    double rel_ = 0;
};

// ch4/v3/src/Source.h:13-68: inlet_face "x-" .. "z+" (or "-x" .. "+z"); the face becomes
// Dirichlet at 0 V; sample() injects one step of particles (pic_step does it for every source)
class Source {
public:
    virtual ~Source() noexcept = default;
    virtual void sample() const noexcept { last_rc_ = pic_source_sample(world_->handle(), id_); }
    int lastStatus() const { return last_rc_; }

protected:
    Source(Species& sp, World& world, type_calc v_drift, type_calc den, type_calc T, std::string face,
           uint64_t seed)
        : world_(&world) {
        static const char* names[] = {"x-", "x+", "y-", "y+", "z-", "z+", "-x", "+x", "-y", "+y", "-z", "+z"};
        for (auto& ch : face) ch = (char)std::tolower((unsigned char)ch);
        int f = -1;
        for (int k = 0; k < 12; k++)
            if (face == names[k]) f = k % 6;
        if (f < 0) throw std::invalid_argument("Passed wrong face name.");
        check(pic_source_create(world.handle(), sp.id(), v_drift, den, T, f, seed, &id_));
    }
    World* world_;
    int id_ = -1;
    mutable int last_rc_ = PIC_OK;
};
class ColdBeamSource : public Source {
public:
    ColdBeamSource(Species& sp, World& world, type_calc v_drift, type_calc den, std::string inlet_face = "-z",
                   uint64_t seed = 1)
        : Source(sp, world, v_drift, den, 0.0, inlet_face, seed) {}
};
class WarmBeamSource : public Source {
public:
    WarmBeamSource(Species& sp, World& world, type_calc v_drift, type_calc den, type_calc T,
                   std::string inlet_face = "-z", uint64_t seed = 1)
        : Source(sp, world, v_drift, den, T, inlet_face, seed) {}
};

class Interaction {  // ch4/v3/src/Interactions.h:9-13
public:
    virtual void apply(type_calc dt) noexcept = 0;
    virtual ~Interaction() noexcept = default;
};

// background-gas form of MC_MEX_Ionization (Interactions.h:98-143)
class MC_MEX_Ionization : public Interaction {
public:
    MC_MEX_Ionization(Species& electrons, Species& ions, World& world, double n_neutral, double T_neutral,
                      double m_neutral, double E_ion_eV, const std::vector<double>& table_E,
                      const std::vector<double>& table_s, int sigma_ion_kind, std::array<double, 4> sigma_ion_params,
                      double B_inc = 10.0, uint64_t seed = 12345)
        : world_(&world) {
        if (table_E.size() != table_s.size()) throw std::invalid_argument("sigma table sizes differ");
        check(pic_mcc_create(world.handle(), electrons.id(), ions.id(), n_neutral, T_neutral, m_neutral, E_ion_eV,
                             B_inc, sigma_ion_kind, sigma_ion_params.data(), table_E.data(), table_s.data(),
                             (int)table_E.size(), seed));
    }
    void apply(type_calc dt) noexcept override { last_rc_ = pic_mcc_apply(world_->handle(), dt); }
    int lastStatus() const { return last_rc_; }
    std::array<uint64_t, 4> stats() const {
        std::array<uint64_t, 4> s{};
        check(pic_mcc_stats(world_->handle(), s.data()));
        return s;
    }

private:
    World* world_;
    int last_rc_ = PIC_OK;
};

// DSMC_MEX (Interactions.h:42-66): one species with itself, or two species of equal mpw0
// (std::invalid_argument otherwise, as the reference's constructor throws).  A driver loop
// calls apply(dt) with the other interactions (main.cpp:201-203); the one-call loop
// pic_step applies every created DSMC interaction by itself.
class DSMC_MEX : public Interaction {
public:
    DSMC_MEX(Species& species, World& world, uint64_t seed = 12345) : world_(&world) {
        check(pic_dsmc_create(world.handle(), species.id(), -1, seed, &id_));
    }
    DSMC_MEX(Species& species1, Species& species2, World& world, uint64_t seed = 12345) : world_(&world) {
        check(pic_dsmc_create(world.handle(), species1.id(), species2.id(), seed, &id_));
    }
    void apply(type_calc dt) noexcept override { last_rc_ = pic_dsmc_apply(world_->handle(), id_, dt); }
    int lastStatus() const { return last_rc_; }
    // collisions and candidate pairs since creation
    std::array<uint64_t, 2> stats() const {
        std::array<uint64_t, 2> s{};
        check(pic_dsmc_stats(world_->handle(), id_, s.data(), nullptr));
        return s;
    }
    double sigmaVRelMax() const {
        double sv = 0;
        check(pic_dsmc_stats(world_->handle(), id_, nullptr, &sv));
        return sv;
    }

private:
    World* world_;
    int id_ = -1;
    int last_rc_ = PIC_OK;
};

}  // namespace pic_gb300
#endif
