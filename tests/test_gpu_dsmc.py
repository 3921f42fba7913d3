"""DSMC_MEX (ch4/v3/src/Interactions.cpp:143-284) on the GPU.

Three kinds of check:
  * particle by particle against the oracle's restatement of the GPU form (or_dsmc_gpuform, the
    same Philox draws, FP64 arithmetic) on the order the device sorted the particles into;
  * statistically against the reference's own algorithm (or_dsmc_ref, pinned bit-exactly by
    tests/golden/dsmc.npz): collision counts per call and the relaxation of a two-temperature
    mixture, from independent realisations;
  * conservation: every collision keeps the pair's momentum and energy."""
import numpy as np
import pytest

import oracle as O
from conftest import golden

pytestmark = pytest.mark.gpu

TAG = 0xD5000000


def world_from_golden(pic, d, species=("a",), capacity=20000):
    W = pic.World(*[int(v) for v in d["nn"]], tuple(d["x0"]), tuple(d["xm"]))
    W.setTime(float(d["dt"]), 100)
    out = []
    for k, (nm, m) in enumerate((("O", 16), ("O2", 32))):
        if nm == "O2" and "b" not in species:
            break
        s = pic.Species(nm, m * pic.AMU, 0.0, W, float(d["mpw0"]), capacity=capacity)
        pre = "ab"[k] + "0_"
        n = len(d[pre + "w"])
        s.addParticles(d[pre + "pos"], d[pre + "vel"], d[pre + "w"], ids=np.arange(n, dtype=np.uint64), rewind=False)
        out.append(s)
    return W, out


def cells_of(p, nn, x0, xm):
    ci = np.array(nn) - 1
    lc = ((p["pos"] - np.array(x0)) / (np.array(xm) - np.array(x0)) * ci).astype(int)
    lc = np.minimum(lc, ci - 1)
    return (lc[:, 2] * ci[1] + lc[:, 1]) * ci[0] + lc[:, 0]


def device_order(before, after, nn, x0, xm):
    """Velocities before the call in the order the call used, and the per-cell counts."""
    c = cells_of(after, nn, x0, xm)
    assert np.all(np.diff(c) >= 0)  # the call left the species in cell order
    pos = np.argsort(before["id"])
    idx = pos[np.searchsorted(before["id"][pos], after["id"])]
    vel = np.ascontiguousarray(before["vel"][idx], np.float64)
    return vel, np.bincount(c, minlength=int(np.prod(np.array(nn) - 1))).astype(np.int32)


def compare(v_gpu, v_ora, scale):
    """Particles whose velocity differs beyond FP32 rounding (an accept test that FP32 and FP64
    decide differently changes that pair and the later pairs of its cell)."""
    err = np.max(np.abs(v_gpu - v_ora), axis=1) / scale
    return int(np.sum(err > 2e-4))


@pytest.mark.parametrize("two", [False, True])
def test_dsmc_matches_gpu_form_oracle(pic, port, two):
    d = golden("dsmc")
    nn, x0, xm = [int(v) for v in d["nn"]], tuple(d["x0"]), tuple(d["xm"])
    dt, mpw0 = float(d["dt"]), float(d["mpw0"])
    W, sp = world_from_golden(pic, d, ("a", "b") if two else ("a",))
    seed = 0x0D5A_C0FFEE
    D = pic.DSMC_MEX(sp[0], sp[1], W, seed=seed) if two else pic.DSMC_MEX(sp[0], W, seed=seed)
    g = port.grid(nn, x0, xm)
    q = port.dsmc_params(g, sp[0].mass, sp[-1].mass, mpw0)
    svmax = float(np.float32(1e-14))
    tot_c = tot_p = 0
    for call in range(3):
        before = [s.getPartRef() for s in sp]
        D.apply(dt)
        after = [s.getPartRef() for s in sp]
        v1, c1 = device_order(before[0], after[0], nn, x0, xm)
        v2, c2 = device_order(before[1], after[1], nn, x0, xm) if two else (None, None)
        nc, pairs, mx = port.dsmc_gpuform(q, v1, c1, v2, c2, dt, svmax, seed, call, TAG)
        st = D.stats()
        assert st["pairs"] - tot_p == pairs  # same groups per cell
        assert abs(st["collisions"] - tot_c - nc) <= 3, (call, st, nc)
        assert nc > 100
        tot_c, tot_p = st["collisions"], st["pairs"]
        scale = np.sqrt(np.mean(v1 ** 2))
        bad = compare(after[0]["vel"], v1, scale) + (compare(after[1]["vel"], v2, scale) if two else 0)
        assert bad <= 0.01 * sum(len(a) for a in after), (call, bad)
        # the majorant follows the reference's rule: the largest candidate sigma v of a colliding call
        assert abs(st["sigma_v_rel_max"] / mx - 1) <= 1e-4
        svmax = float(np.float32(st["sigma_v_rel_max"]))


def test_dsmc_conserves_momentum_and_energy(pic):
    nn, x0, xm = (17, 17, 17), (0.0, 0.0, 0.0), (0.016, 0.016, 0.016)  # 4096 cells of 1 mm^3
    W = pic.World(*nn, x0, xm)
    W.setTime(1e-5, 100)
    mpw0 = 2e10
    a = pic.Species("O", 16 * pic.AMU, 0.0, W, mpw0, capacity=600_000)
    b = pic.Species("O2", 32 * pic.AMU, 0.0, W, mpw0, capacity=600_000)
    a.loadUniform(x0, xm, 400_000, 300.0, mpw0, 0.0, seed=1)
    b.loadUniform(x0, xm, 300_000, 1500.0, mpw0, 0.0, seed=2)
    D = pic.DSMC_MEX(a, b, W, seed=3)

    def sums():
        pa, pb = a.getPartRef(), b.getPartRef()
        ma, mb = 16 * pic.AMU, 32 * pic.AMU
        mom = ma * pa["vel"].sum(0) + mb * pb["vel"].sum(0)
        ke = 0.5 * (ma * np.sum(pa["vel"] ** 2) + mb * np.sum(pb["vel"] ** 2))
        p_scale = ma * np.sum(np.abs(pa["vel"])) + mb * np.sum(np.abs(pb["vel"]))
        return mom, ke, p_scale

    m0, k0, ps = sums()
    for _ in range(5):
        D.apply(1e-5)
    m1, k1, _ = sums()
    st = D.stats()
    assert st["collisions"] > 100_000
    # FP32 velocities: each collision conserves to rounding, errors add up as a random walk
    assert np.all(np.abs(m1 - m0) <= 1e-6 * ps)
    assert abs(k1 / k0 - 1) <= 1e-5


def test_dsmc_rates_and_relaxation_match_reference(pic, port):
    """A two-species mixture at 300 K / 1500 K: collisions per call and the temperature gap decay
    of the GPU form against independent realisations of the reference's algorithm."""
    nn, x0, xm = (9, 9, 9), (0.0, 0.0, 0.0), (0.008, 0.008, 0.008)  # 512 cells of 1 mm^3
    mpw0, dt, steps = 3.2e10, 1e-6, 8
    ma, mb = 16 * O.AMU, 32 * O.AMU
    per_cell = 30
    n = 512 * per_cell
    rng = np.random.default_rng(8)

    def load(T, m):
        pos = rng.uniform(x0, xm, (n, 3)) * 0.999999
        vel = rng.normal(size=(n, 3)) * np.sqrt(O.KB * T / m)
        return pos, vel

    pa, va = load(300.0, ma)
    pb, vb = load(1500.0, mb)

    def temps(vela, velb):
        return ma * np.mean(np.sum(vela ** 2, 1)) / (3 * O.KB), mb * np.mean(np.sum(velb ** 2, 1)) / (3 * O.KB)

    # reference algorithm, K independent realisations
    g = port.grid(nn, x0, xm)
    q = port.dsmc_params(g, ma, mb, mpw0)
    K = 6
    ref_c = np.zeros((K, steps))
    ref_T = np.zeros((K, steps, 2))
    for k in range(K):
        A = np.zeros(n, O.PARTICLE)
        B = np.zeros(n, O.PARTICLE)
        A["pos"], A["vel"], A["w"] = pa, va, mpw0
        B["pos"], B["vel"], B["w"] = pb, vb, mpw0
        mt = port.mt(1000 + k)
        sv = 1e-14
        for s in range(steps):
            ref_c[k, s], _, sv = port.dsmc_ref(g, q, mt, A, B, dt, sv)
            ref_T[k, s] = temps(A["vel"], B["vel"])

    # GPU form: K worlds' worth in K separate runs with different seeds
    gpu_c = np.zeros((K, steps))
    gpu_T = np.zeros((K, steps, 2))
    for k in range(K):
        W = pic.World(*nn, x0, xm)
        W.setTime(dt, 100)
        a = pic.Species("O", ma, 0.0, W, mpw0, capacity=2 * n)
        b = pic.Species("O2", mb, 0.0, W, mpw0, capacity=2 * n)
        a.addParticles(pa, va, np.full(n, mpw0), rewind=False)
        b.addParticles(pb, vb, np.full(n, mpw0), rewind=False)
        D = pic.DSMC_MEX(a, b, W, seed=500 + k)
        last = 0
        for s in range(steps):
            D.apply(dt)
            st = D.stats()
            gpu_c[k, s] = st["collisions"] - last
            last = st["collisions"]
            gpu_T[k, s] = temps(a.getPartRef()["vel"], b.getPartRef()["vel"])

    # collisions per call (the first call runs on the 1e-14 start majorant, the rest on the update)
    for s in range(steps):
        mr, mg = ref_c[:, s].mean(), gpu_c[:, s].mean()
        se = np.sqrt(ref_c[:, s].var(ddof=1) / K + gpu_c[:, s].var(ddof=1) / K + (mr + mg) / (2 * K))
        assert mr > 200 and abs(mg - mr) <= 4 * se + 0.01 * mr, (s, mr, mg, se)
    # temperatures: the gap between the species closes at the same rate
    gap_r = ref_T[:, :, 1] - ref_T[:, :, 0]
    gap_g = gpu_T[:, :, 1] - gpu_T[:, :, 0]
    assert gap_r[:, -1].mean() < 0.8 * 1200  # the mixture relaxes within the run
    se = np.sqrt(gap_r.var(0, ddof=1) / K + gap_g.var(0, ddof=1) / K)
    assert np.all(np.abs(gap_g.mean(0) - gap_r.mean(0)) <= 4 * se + 0.01 * 1200), (gap_g.mean(0), gap_r.mean(0))


def test_dsmc_rejects_unequal_weights(pic):
    W = pic.World(5, 5, 5, (0, 0, 0), (0.004, 0.004, 0.004))
    a = pic.Species("O", 16 * pic.AMU, 0.0, W, 1e10, capacity=100)
    b = pic.Species("O2", 32 * pic.AMU, 0.0, W, 2e10, capacity=100)
    with pytest.raises(Exception, match="same macroparticle weight"):
        pic.DSMC_MEX(a, b, W)


def test_dsmc_in_step_loop(pic):
    """World.step applies the interaction before the pushes (main.cpp:201-203)."""
    d = golden("dsmc")
    W, sp = world_from_golden(pic, d)
    W.set_boundaries((1, 1, 1), (1,) * 6, (0.0,) * 6)
    W.setTime(1e-7, 100)  # neutrals at ~500 m/s cross a twentieth of a cell per step
    W.configure_loop(solve_each_step=False, sort_every=0)
    D = pic.DSMC_MEX(sp[0], W, seed=9)
    for _ in range(5):
        W.step()
    st = D.stats()
    assert st["collisions"] > 50 and st["pairs"] >= st["collisions"]
    assert sp[0].getNumParticles() == 2000
