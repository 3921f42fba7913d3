"""The C++ facade drives a ch4/v3-style loop (examples/v3_loop.cpp) through the C ABI."""
import os
import subprocess

import pytest

from conftest import ROOT, PKG_NAME

pytestmark = pytest.mark.gpu


def test_v3_style_cpp_driver(pic, tmp_path):
    pic.library()  # builds lib/libpic_gb300.so
    pkg = os.path.join(ROOT, PKG_NAME)
    exe = str(tmp_path / "v3_loop")
    r = subprocess.run(["g++", "-std=c++17", "-O2", os.path.join(pkg, "examples", "v3_loop.cpp"),
                        "-I", os.path.join(ROOT, "include"), "-L", os.path.join(pkg, "lib"), "-lpic_gb300",
                        "-Wl,-rpath," + os.path.join(pkg, "lib"), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "10"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    line = r.stdout.strip().splitlines()[-1]
    fields = dict(kv.split("=") for kv in line.split())
    assert int(fields["ts"]) == 11
    assert int(fields["electrons"]) >= 200000 and int(fields["ions"]) >= 200000
    assert int(fields["collisions"]) > 0


DRIVER = r"""
#include <cstdio>
#include <stdexcept>
#include "pic_gb300.hpp"
using namespace pic_gb300;
int main() {
    const double amu = 1.660538921e-27, q_e = 1.602176565e-19;
    World world(17, 17, 17, {0.0, 0.0, 0.0}, {0.016, 0.016, 0.016});
    world.setTime(1e-7, 100);
    world.addBox({0.008, 0.008, 0.008}, 0.0, {0.004, 0.004, 0.004});
    Species O("O", 16 * amu, 0, world, 2e10, 400000);
    Species O2("O2", 32 * amu, 0, world, 2e10, 400000);
    Species Op("O+", 16 * amu, q_e, world, 2e10, 100000);
    O.loadUniform({0, 0, 0}, {0.016, 0.0058, 0.016}, 100000, 600.0, 2e10, 0.0, 1);
    O2.loadUniform({0, 0, 0}, {0.016, 0.0058, 0.016}, 100000, 900.0, 2e10, 0.0, 2);
    Op.loadUniform({0, 0, 0}, {0.016, 0.0058, 0.016}, 50000, 30000.0, 2e10, 0.0, 3);
    DSMC_MEX self(O, world);          // DSMC_MEX(species, world)
    DSMC_MEX pair(O, O2, world, 7);   // DSMC_MEX(species1, species2, world)
    bool threw = false;
    try {
        Species heavy("X", 40 * amu, 0, world, 3e10, 10);
        DSMC_MEX bad(O, heavy, world);
    } catch (const std::invalid_argument&) {
        threw = true;
    }
    Config::getInstance().setSPUTTERING(true);
    for (int s = 0; s < 20; s++) {
        world.advanceTime();
        self.apply(world.getDt());
        pair.apply(world.getDt());
        O.advanceNonElectron(O, O, world.getDt() * 50);
        Op.advanceNonElectron(O, O, world.getDt() * 5);
    }
    auto so = O.objectStats(), si = Op.objectStats();
    auto c1 = self.stats(), c2 = pair.stats();
    std::printf("threw=%d self=%llu pair=%llu svmax=%g o_hits=%llu o_bounces=%llu i_hits=%llu last=%d\n", threw ? 1 : 0,
                (unsigned long long)c1[0], (unsigned long long)c2[0], self.sigmaVRelMax(), (unsigned long long)so[0],
                (unsigned long long)so[1], (unsigned long long)si[0], self.lastStatus() | pair.lastStatus());
    return 0;
}
"""


def test_cpp_facade_dsmc_and_objects(pic, tmp_path):
    pic.library()
    pkg = os.path.join(ROOT, PKG_NAME)
    src = tmp_path / "driver.cpp"
    src.write_text(DRIVER)
    exe = str(tmp_path / "driver")
    r = subprocess.run(["g++", "-std=c++17", "-O2", str(src), "-I", os.path.join(ROOT, "include"), "-L",
                        os.path.join(pkg, "lib"), "-lpic_gb300", "-Wl,-rpath," + os.path.join(pkg, "lib"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    f = dict(kv.split("=") for kv in r.stdout.strip().splitlines()[-1].split())
    assert f["threw"] == "1" and f["last"] == "0"
    assert int(f["self"]) > 1000 and int(f["pair"]) > 1000 and 1e-17 < float(f["svmax"]) < 1e-14
    assert int(f["o_hits"]) > 100 and int(f["o_bounces"]) >= int(f["o_hits"]) and int(f["i_hits"]) > 100


BATCH = r"""
#include <cstdio>
#include <vector>
#include "pic_gb300.hpp"
using namespace pic_gb300;
int main() {
    const double m_e = 9.10938215e-31, q_e = 1.602176565e-19;
    World world(17, 17, 17, {0.0, 0.0, 0.0}, {0.01, 0.01, 0.01});
    world.setTime(1e-11, 10);
    Species a("a", m_e, -q_e, world, 1.0, 20000), b("b", 40 * m_e, -q_e, world, 1.0, 20000);
    std::vector<double> pa, va, wa, pb, vb, wb;
    for (int k = 0; k < 9000; k++) {
        const double u = (k % 97) / 97.0, v = (k % 89) / 89.0, s = (k % 83) / 83.0;
        for (double x : {0.01 * u * 0.999, 0.01 * v * 0.999, 0.01 * s * 0.999}) pa.push_back(x);
        for (double x : {1e5 * (u - 0.5), 1e5 * (v - 0.5), 1e5 * (s - 0.5)}) va.push_back(x);
        wa.push_back(1.0 + u);
        if (k < 5000) {
            for (double x : {0.01 * s * 0.999, 0.01 * u * 0.999, 0.01 * v * 0.999}) pb.push_back(x);
            for (double x : {1e4 * (s - 0.5), 1e4 * (u - 0.5), 1e4 * (v - 0.5)}) vb.push_back(x);
            wb.push_back(2.0 - v);
        }
    }
    addParticlesBatch(world, {&a, &b}, {{pa.data(), va.data(), wa.data(), (long)wa.size()},
                                        {pb.data(), vb.data(), wb.data(), (long)wb.size()}});
    world.setLaunchShapes({2, 456, 608});
    const auto s = world.launchShapes();
    std::printf("a=%zu b=%zu shapes=%d,%d,%d\n", a.getNumParticles(), b.getNumParticles(), s[0], s[1], s[2]);
    return 0;
}
"""


def test_cpp_facade_batch_upload_and_launch_shapes(pic, tmp_path):
    pic.library()
    pkg = os.path.join(ROOT, PKG_NAME)
    src = tmp_path / "batch.cpp"
    src.write_text(BATCH)
    exe = str(tmp_path / "batch")
    r = subprocess.run(["g++", "-std=c++17", "-O2", str(src), "-I", os.path.join(ROOT, "include"), "-L",
                        os.path.join(pkg, "lib"), "-lpic_gb300", "-Wl,-rpath," + os.path.join(pkg, "lib"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == "a=9000 b=5000 shapes=2,456,608"
