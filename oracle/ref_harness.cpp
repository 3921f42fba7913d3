// Test infrastructure only: a thin extern "C" shim over the reference's own,
// unmodified ch4/v3 classes (World, Species, PotentialSolver, MC_MEX_Ionization).
// oracle/Makefile compiles it together with the reference sources into
// oracle/_ref/libpicref.so.  Only tests/golden/make_golden.py and the CPU-side
// tests load it, to produce and check golden vectors.  Nothing in the product
// path links or calls this file.
//
// Every entry point drives the reference through its public API:
//   World(ni,nj,nk,x0,xm)                       ch4/v3/src/World.h:63
//   World::computeObjectID / object_id / phi     ch4/v3/src/World.cpp:276-292
//   Species(name,mass,charge,world,mpw0[,E_ion]) ch4/v3/src/Species.h:56-57
//   Species::advanceElectrons / advanceNonElectron ch4/v3/src/Species.cpp:258, 47
//   Species::computeNumberDensity                ch4/v3/src/Species.cpp:401
//   Species::updateAverages / den_avg            ch4/v3/src/Species.cpp:764
//   Species::computeMacroParticlesCount          ch4/v3/src/Species.cpp:813
//   World::computeChargeDensity                  ch4/v3/src/World.cpp:193
//   PotentialSolver::solve / computeEF           ch4/v3/src/PotentialSolver.cpp:55, 354
//   MC_MEX_Ionization::apply                     ch4/v3/src/Interactions.cpp:567
//   Species::merge                               ch4/v3/src/Species.cpp:1037
//   Species::loadParticleBoxThermal              ch4/v3/src/Species.cpp:564
//   DSMC_MEX(species[, species2], world) / apply   ch4/v3/src/Interactions.cpp:143-284
// The global RNG `rnd` (ch4/v3/src/Rnd.cpp:18) is reseeded by assignment so
// that runs are reproducible (the stock code seeds it from random_device).
#include <memory>
#include <sstream>
#include <vector>
#include <string>
#include <cstring>
#include <fstream>
#include "all.h"
#include "World.h"
#include "Species.h"
#include "PotentialSolver.h"
#include "Interactions.h"
#include "Config.h"
#include "Rnd.h"
#include "Object.h"

namespace {
struct RefSim {
    std::unique_ptr<World> world;
    std::vector<Species> species;
    std::unique_ptr<PotentialSolver> solver;
    std::unique_ptr<MC_MEX_Ionization> mcmex;
    std::unique_ptr<DSMC_MEX> dsmc;
};
// read access to the protected (sigma v_rel)_max, so that tests can follow its updates
struct DsmcProbe : DSMC_MEX {
    using DSMC_MEX::DSMC_MEX;
    double svmax() const { return sigma_v_rel_max; }
};
std::ofstream g_null_sink;
void quiet() {
    static bool done = false;
    if (done) return;
    done = true;
    // the reference writes progress to std::cerr/std::cout; drop it
    std::cerr.rdbuf(nullptr);
    std::cout.rdbuf(nullptr);
    Config::getInstance().setMULTITHREADING(false);  // serial push: the multithreaded one loses deletions
    Config::getInstance().setSPUTTERING(false);
}
}  // namespace

extern "C" {

void* ref_world_create(int ni, int nj, int nk, const double* x0, const double* xm) {
    quiet();
    RefSim* s = new RefSim();
    s->world = std::make_unique<World>(ni, nj, nk, type_calc3{x0[0], x0[1], x0[2]}, type_calc3{xm[0], xm[1], xm[2]});
    s->species.reserve(8);  // Species are referenced by the solver and interactions: no reallocation
    return s;
}
void ref_world_destroy(void* h) { delete static_cast<RefSim*>(h); }

void ref_seed(unsigned seed) { rnd = Rnd(seed); }
double ref_rnd() { return rnd(); }

void ref_set_time(void* h, double dt, int num_ts) { static_cast<RefSim*>(h)->world->setTime(dt, num_ts); }
int ref_advance_time(void* h) { return static_cast<RefSim*>(h)->world->advanceTime() ? 1 : 0; }
int ref_get_ts(void* h) { return static_cast<RefSim*>(h)->world->getTs(); }

// Marks every wall node as fixed (object_id = 1, node_type = DIRICHLET) at potential phi_wall:
// the ch2 "Dirichlet walls" semantics expressed through public World fields.
void ref_dirichlet_walls(void* h, double phi_wall) {
    World& w = *static_cast<RefSim*>(h)->world;
    for (int i = 0; i < w.ni; i++)
        for (int j = 0; j < w.nj; j++)
            for (int k = 0; k < w.nk; k++)
                if (i == 0 || i == w.ni - 1 || j == 0 || j == w.nj - 1 || k == 0 || k == w.nk - 1) {
                    w.object_id[i][j][k] = 1;
                    w.node_type[i][j][k] = 2;  // World::NodeType DIRICHLET
                    w.phi[i][j][k] = phi_wall;
                }
}
// Axis-aligned box electrode (ch4/v3/src/Object.cpp:231 Rectangle::inObject)
void ref_add_rectangle(void* h, const double* pos, double phi, const double* sides) {
    World& w = *static_cast<RefSim*>(h)->world;
    w.addObject<Rectangle>(type_calc3{pos[0], pos[1], pos[2]}, phi, type_calc3{sides[0], sides[1], sides[2]});
    w.computeObjectID();
}

int ref_species_create(void* h, const char* name, double mass, double charge, double mpw0, double E_ion) {
    RefSim* s = static_cast<RefSim*>(h);
    if (s->species.size() >= 8) return -1;
    if (E_ion > 0) s->species.emplace_back(std::string(name), mass, charge, *s->world, mpw0, E_ion);
    else s->species.emplace_back(std::string(name), mass, charge, *s->world, mpw0);
    return (int)s->species.size() - 1;
}
// Direct placement: no half-step rewind, no rejection (as the interactions do with emplace_back)
void ref_species_set(void* h, int sp, const double* pos, const double* vel, const double* w, long n) {
    std::vector<Particle>& parts = static_cast<RefSim*>(h)->species[sp].getPartRef();
    parts.clear();
    parts.reserve(4 * n + 4096);  // interactions emplace_back while holding element references
    for (long p = 0; p < n; p++)
        parts.emplace_back(type_calc3{pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]},
                           type_calc3{vel[3 * p], vel[3 * p + 1], vel[3 * p + 2]}, w[p]);
    static_cast<RefSim*>(h)->species[sp].setSorted(false);
}
// Species::addParticle (rejection + half-step rewind)
void ref_species_add(void* h, int sp, const double* pos, const double* vel, double w) {
    static_cast<RefSim*>(h)->species[sp].addParticle(type_calc3{pos[0], pos[1], pos[2]}, type_calc3{vel[0], vel[1], vel[2]}, w);
}
long ref_species_count(void* h, int sp) { return (long)static_cast<RefSim*>(h)->species[sp].getNumParticles(); }
void ref_species_get(void* h, int sp, double* pos, double* vel, double* w) {
    const std::vector<Particle>& parts = static_cast<RefSim*>(h)->species[sp].getConstPartRef();
    for (size_t p = 0; p < parts.size(); p++) {
        for (int d = 0; d < 3; d++) {
            pos[3 * p + d] = parts[p].pos[d];
            vel[3 * p + d] = parts[p].vel[d];
        }
        w[p] = parts[p].macro_weight;
    }
}
void ref_load_box_thermal(void* h, int sp, const double* x0, const double* sides, double num_den, double T) {
    static_cast<RefSim*>(h)->species[sp].loadParticleBoxThermal(type_calc3{x0[0], x0[1], x0[2]},
                                                                  type_calc3{sides[0], sides[1], sides[2]}, num_den, T);
}

void ref_push_electrons(void* h, int sp, double dt) { static_cast<RefSim*>(h)->species[sp].advanceElectrons(dt); }
void ref_push_nonelectron(void* h, int sp, int neutral_sp, double dt) {
    RefSim* s = static_cast<RefSim*>(h);
    s->species[sp].advanceNonElectron(s->species[neutral_sp], s->species[neutral_sp], dt);
}
// Species::advanceNonElectron(neutrals, spherium, dt) with Config::SPUTTERING set as given
void ref_push_nonelectron_sput(void* h, int sp, int neutral_sp, int spherium_sp, int sputtering, double dt) {
    RefSim* s = static_cast<RefSim*>(h);
    Config::getInstance().setSPUTTERING(sputtering != 0);
    s->species[sp].advanceNonElectron(s->species[neutral_sp], s->species[spherium_sp], dt);
    Config::getInstance().setSPUTTERING(false);
}
void ref_number_density(void* h, int sp) { static_cast<RefSim*>(h)->species[sp].computeNumberDensity(); }
void ref_charge_density(void* h) {
    RefSim* s = static_cast<RefSim*>(h);
    s->world->computeChargeDensity(s->species);
}
void ref_merge(void* h, int sp) { static_cast<RefSim*>(h)->species[sp].merge(); }
// Species::sampleMoments + computeGasProperties; the public vel and T fields come back
void ref_sample_moments(void* h, int sp) { static_cast<RefSim*>(h)->species[sp].sampleMoments(); }
void ref_gas_properties(void* h, int sp, double* vel, double* T) {
    Species& s = static_cast<RefSim*>(h)->species[sp];
    s.computeGasProperties();
    for (int k = 0; k < s.T.nk; k++)
        for (int j = 0; j < s.T.nj; j++)
            for (int i = 0; i < s.T.ni; i++) {
                int n = s.T.U(i, j, k);
                T[n] = s.T[i][j][k];
                for (int d = 0; d < 3; d++) vel[3 * n + d] = s.vel[i][j][k][d];
            }
}

static void get_scalar(const Field<type_calc>& f, double* out) {
    for (int k = 0; k < f.nk; k++)
        for (int j = 0; j < f.nj; j++)
            for (int i = 0; i < f.ni; i++) out[f.U(i, j, k)] = f[i][j][k];
}
static void set_scalar(Field<type_calc>& f, const double* in) {
    for (int k = 0; k < f.nk; k++)
        for (int j = 0; j < f.nj; j++)
            for (int i = 0; i < f.ni; i++) f[i][j][k] = in[f.U(i, j, k)];
}
// which: 0 phi, 1 rho, 2 node_vol, 3 object_id
void ref_get_field(void* h, int which, double* out) {
    World& w = *static_cast<RefSim*>(h)->world;
    if (which == 0) get_scalar(w.phi, out);
    else if (which == 1) get_scalar(w.rho, out);
    else if (which == 2) get_scalar(w.node_vol, out);
    else if (which == 3) {
        for (int k = 0; k < w.nk; k++)
            for (int j = 0; j < w.nj; j++)
                for (int i = 0; i < w.ni; i++) out[w.object_id.U(i, j, k)] = w.object_id[i][j][k];
    }
}
void ref_set_field(void* h, int which, const double* in) {
    World& w = *static_cast<RefSim*>(h)->world;
    if (which == 0) set_scalar(w.phi, in);
    else if (which == 1) set_scalar(w.rho, in);
}
void ref_get_den(void* h, int sp, double* out) { get_scalar(static_cast<RefSim*>(h)->species[sp].den, out); }
// Species::updateAverages (Species.cpp:764-766) and its public den_avg field
void ref_update_averages(void* h, int sp) { static_cast<RefSim*>(h)->species[sp].updateAverages(); }
void ref_get_den_avg(void* h, int sp, double* out) { get_scalar(static_cast<RefSim*>(h)->species[sp].den_avg, out); }
// Species::computeMacroParticlesCount (Species.cpp:813-819); the public macro_part_count field
// is cell-sized (Species.cpp:32), so out holds (ni-1)(nj-1)(nk-1) values in linear cell order
void ref_macro_count(void* h, int sp, double* out) {
    Species& s = static_cast<RefSim*>(h)->species[sp];
    s.computeMacroParticlesCount();
    get_scalar(s.macro_part_count, out);
}
void ref_get_ef(void* h, double* out) {
    World& w = *static_cast<RefSim*>(h)->world;
    for (int k = 0; k < w.nk; k++)
        for (int j = 0; j < w.nj; j++)
            for (int i = 0; i < w.ni; i++)
                for (int d = 0; d < 3; d++) out[3 * w.ef.U(i, j, k) + d] = w.ef[i][j][k][d];
}
void ref_set_ef(void* h, const double* in) {
    World& w = *static_cast<RefSim*>(h)->world;
    for (int k = 0; k < w.nk; k++)
        for (int j = 0; j < w.nj; j++)
            for (int i = 0; i < w.ni; i++)
                for (int d = 0; d < 3; d++) w.ef[i][j][k][d] = in[3 * w.ef.U(i, j, k) + d];
}

// solver_type: 0 GS, 1 PCG (ch4/v3/src/PotentialSolver.h:24)
void ref_solver_create(void* h, unsigned max_it, double tol, int solver_type) {
    RefSim* s = static_cast<RefSim*>(h);
    s->solver = std::make_unique<PotentialSolver>(*s->world, max_it, tol, static_cast<SolverType>(solver_type));
    s->solver->setReferenceValues(0, 0, 1e20);  // as main.cpp:138: no Boltzmann electrons
}
int ref_solve(void* h) { return static_cast<RefSim*>(h)->solver->solve() ? 1 : 0; }
void ref_compute_ef(void* h) { static_cast<RefSim*>(h)->solver->computeEF(); }

int ref_mcmex_create(void* h, int neu, int ion, int ele, const char* table_path) {
    RefSim* s = static_cast<RefSim*>(h);
    try {
        s->mcmex = std::make_unique<MC_MEX_Ionization>(s->species[neu], s->species[ion], s->species[ele], *s->world,
                                                       std::string(table_path), 10);
    } catch (const std::exception&) {
        return -1;
    }
    return 0;
}
void ref_mcmex_apply(void* h, double dt) { static_cast<RefSim*>(h)->mcmex->apply(dt); }

// sp2 < 0 or sp2 == sp1: the one-species constructor (Interactions.cpp:143), else the two-species one
int ref_dsmc_create(void* h, int sp1, int sp2) {
    RefSim* s = static_cast<RefSim*>(h);
    try {
        if (sp2 < 0 || sp2 == sp1)
            s->dsmc = std::make_unique<DsmcProbe>(s->species[sp1], *s->world);
        else
            s->dsmc = std::make_unique<DsmcProbe>(s->species[sp1], s->species[sp2], *s->world);
    } catch (const std::exception&) {
        return -1;
    }
    return 0;
}
void ref_dsmc_apply(void* h, double dt) { static_cast<RefSim*>(h)->dsmc->apply(dt); }
double ref_dsmc_svmax(void* h) { return static_cast<DsmcProbe*>(static_cast<RefSim*>(h)->dsmc.get())->svmax(); }

}  // extern "C"
