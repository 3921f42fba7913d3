// A ch4/v3-style driver (ch4/v3/src/main.cpp:20-295) written against the C++ facade: the same
// objects and calls, with the particles and fields on the GPU.
//   g++ -std=c++17 -O2 v3_loop.cpp -I<repo>/include -L<lib dir> -lpic_gb300 -o v3_loop
//   ./v3_loop [num_ts] [output mode: none|all|screen|fields|particles|diagnostics|convergence]
// With an output mode other than none the loop also keeps the per-step moments, cell counts and
// density averages and writes results/ (fields every 10 steps, runtime_diags.csv) as main.cpp does.
#include <cstdio>
#include <cmath>
#include <cstdlib>
#include <sstream>
#include <vector>
#include "pic_gb300.hpp"
#include "pic_gb300_outputs.hpp"

using namespace pic_gb300;

int main(int argc, char** argv) {
    int num_ts = argc > 1 ? std::atoi(argv[1]) : 20;
    Output::modes OUTPUT = Output::none;
    if (argc > 2) {
        std::stringstream a(argv[2]);
        a >> OUTPUT;
    }
    const double q_e = 1.602176565e-19, amu = 1.660538921e-27, m_e = 9.10938215e-31, k_B = 1.380648e-23;
    // World(ni, nj, nk, x0, xm) and the electrode planes (main.cpp:89-100)
    World world(33, 33, 65, {0.0, 0.0, 0.0}, {0.01, 0.01, 0.02});
    world.setTime(2e-12, num_ts);
    int periodic[3] = {1, 1, 0}, mode[6] = {1, 1, 1, 1, 1, 1};
    double phi[6] = {0, 0, 0, 0, 0.0, 500.0};
    world.setBoundaries(periodic, mode, phi);
    // species (main.cpp:105-108)
    Species ions("O2+", 32 * amu, q_e, world, 64.0, 400000);
    Species electrons("e-", m_e, -q_e, world, 64.0, 400000);
    electrons.loadUniform({0.0, 0.0, 0.006}, {0.01, 0.01, 0.014}, 200000, 2.0 * q_e / k_B, 64.0, 0.5, 1);
    ions.loadUniform({0.0, 0.0, 0.006}, {0.01, 0.01, 0.014}, 200000, 0.03 * q_e / k_B, 64.0, 0.5, 2);
    // interaction (main.cpp:122): background O2, Lotz ionisation, elastic table
    std::vector<double> E, S;
    for (int i = 0; i < 200; i++) {
        double e = 0.01 * std::pow(1e7, i / 199.0);
        E.push_back(e);
        S.push_back(6e-20 / std::sqrt(1 + e / 10.0));
    }
    MC_MEX_Ionization ionization(electrons, ions, world, 1e21, 300.0, 32 * amu, 12.06, E, S, 1,
                                 {2.107e-17, 1.0, 0.18, 0.0});
    // solver (main.cpp:136-138) and the initial field (main.cpp:172-173)
    PotentialSolver solver(world, 20000, 1e-6, PCG);
    solver.setReferenceValues(0, 0, 1e20);
    solver.solve();
    solver.computeEF();
    std::vector<Species*> species = {&ions, &electrons};
    const bool out_on = OUTPUT != Output::none;
    if (out_on) {
        for (Species* sp : species) sp->computeMacroParticlesCount();  // main.cpp:163-166
        Output::fieldsOutput(world, species);                          // main.cpp:172-174
    }
    while (world.advanceTime()) {  // main.cpp:177
        ionization.apply(world.getDt());
        electrons.advanceElectrons(world.getDt());
        ions.advanceNonElectron(ions, ions, world.getDt());
        if (out_on)  // main.cpp:228-239
            for (Species* sp : species) {
                sp->sampleMoments();
                sp->computeMacroParticlesCount();
            }
        world.computeChargeDensity(species);  // the densities of this step exist from here on
        if (out_on && world.getTs() > 5)      // main.cpp:242-246
            for (Species* sp : species) sp->updateAverages();
        if (!solver.solve()) std::fprintf(stderr, "solver did not converge at ts %d\n", world.getTs());
        solver.computeEF();
        // main.cpp:254-276
        if (OUTPUT == Output::all || OUTPUT >= Output::diagnostics) Output::diagOutput(world, species);
        if (OUTPUT == Output::all || OUTPUT >= Output::screen) Output::screenOutput(world, species);
        const int ts = world.getTs();
        if (ts % 10 == 0 || world.isLastTimeStep()) {
            if (OUTPUT == Output::all || OUTPUT >= Output::fields) Output::fieldsOutput(world, species);
            if (OUTPUT == Output::all || OUTPUT >= Output::particles) Output::particlesOutput(world, species, 1000);
        }
    }
    Output::closeDiagOutput();
    if (out_on) std::printf("\n");
    auto st = ionization.stats();
    std::printf("ts=%d electrons=%zu ions=%zu collisions=%llu ionizations=%llu KE_e=%.6e\n", world.getTs(),
                electrons.getNumParticles(), ions.getNumParticles(), (unsigned long long)st[1],
                (unsigned long long)st[2], electrons.getKE());
    return 0;
}
