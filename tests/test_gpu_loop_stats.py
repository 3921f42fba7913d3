"""Time-averaged profiles of a small discharge with collisions, GPU loop against the FP64 oracle loop.

Both loops start from the same particles and draw collisions from the same Philox streams (the
oracle's or_mcc_background restates the GPU form, whose expectation matches the reference's NTC:
tests/test_gpu_stats.py).  FP32 against FP64 arithmetic makes single trajectories part after a
while, so the loops are compared the way the reference's results are read: profiles along the
electrode axis averaged over time, within their block-averaged standard errors."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

LOTZ = (2.107e-17, 1.0, 0.18, 0.0)


def test_time_averaged_profiles_match_oracle_loop(pic, port):
    nn, x0, xm = (9, 9, 33), (0.0, 0.0, 0.0), (0.004, 0.004, 0.016)
    V, n_gas, dt, seed = 100.0, 1e21, 2e-12, 0x51A7
    steps, skip, blocks = 160, 40, 12
    g = port.grid(nn, x0, xm, periodic=(1, 1, 0))
    kind = port.node_kinds(g, 1)
    nv = int(np.prod(nn))
    rng = np.random.default_rng(17)
    n0 = 30000
    band = (0.0, 0.0, 0.3 * xm[2]), (xm[0], xm[1], 0.7 * xm[2])
    w = 5e13 * xm[0] * xm[1] * 0.4 * xm[2] / n0

    def load(T, mass):
        pos = rng.uniform(band[0], band[1], (n0, 3)) * 0.999999
        vel = rng.normal(size=(n0, 3)) * np.sqrt(O.KB * T / mass)
        return pos, vel

    pe, ve = load(8 * 11604.5, O.ME)  # hot enough that the tail ionises within the run
    pi_, vi = load(0.03 * 11604.5, 32 * O.AMU)
    E_tab = np.geomspace(0.01, 1e5, 300)
    S_tab = 6e-20 / np.sqrt(1 + E_tab / 10.0)

    # ---- GPU loop
    W = pic.World(*nn, x0, xm)
    W.set_boundaries((1, 1, 0), (1,) * 6, (0, 0, 0, 0, 0.0, V))
    W.setTime(dt, 10 ** 6)
    e = pic.Species("e-", pic.ME, -pic.QE, W, w, capacity=4 * n0)
    i = pic.Species("O2+", 32 * pic.AMU, pic.QE, W, w, capacity=4 * n0)
    e.addParticles(pe, ve, np.full(n0, w), ids=np.arange(n0, dtype=np.uint64), rewind=False)
    i.addParticles(pi_, vi, np.full(n0, w), ids=np.arange(n0, dtype=np.uint64), rewind=False)
    M = pic.MC_MEX_Ionization(e, i, W, n_gas, 300.0, 32 * pic.AMU, 12.06, E_tab, S_tab, 1, LOTZ, seed=seed)
    S = pic.PotentialSolver(W, 20000, 1e-8, pic.SOLVER_PCG)
    assert S.solve(raise_on_fail=True)
    S.computeEF()
    W.configure_loop(solve_each_step=True, sort_every=20)

    # ---- oracle loop (same order as pic_step: collisions, electron push, ion push, density, solve, E)
    cp = port.coll_params(E_tab, S_tab, 32 * O.AMU, 12.06, 1, (0.0, 1.0, 0.18), sig_A=LOTZ[0])
    cp.n_neutral, cp.T_neutral = n_gas, 300.0
    cap = 4 * n0
    ele, ion = np.zeros(cap, O.PARTICLE), np.zeros(cap, O.PARTICLE)
    ele[:n0]["pos"], ele[:n0]["vel"], ele[:n0]["w"] = pe, ve, w
    ion[:n0]["pos"], ion[:n0]["vel"], ion[:n0]["w"] = pi_, vi, w
    eid, iid = np.zeros(cap, np.uint64), np.zeros(cap, np.uint64)
    eid[:n0] = np.arange(n0)
    iid[:n0] = np.arange(n0)
    ne_, ni_ = n0, n0
    phi = W.phi.copy()  # Dirichlet values on the electrode planes
    rho = -O.QE * port.number_density(g, ele[:ne_]) + O.QE * port.number_density(g, ion[:ni_])
    port.solve_fpcg(g, kind, phi, rho, 1e-10, 20000)
    ef = port.compute_ef(g, phi)

    prof = {k: [] for k in ("gpu_e", "gpu_phi", "ora_e", "ora_phi")}
    ions_made = [0, 0]
    for step in range(steps):
        W.step()
        ts = W.getTs()
        _, nion, ne_, ni_ = port.mcc_background(g, cp, ele, eid, ne_, ion, iid, ni_, dt, seed, ts)
        ions_made[1] += nion
        ne_ = port.push(g, ele[:ne_], ef, dt, -O.QE, O.ME, ids=eid[:ne_])
        ni_ = port.push(g, ion[:ni_], ef, dt, O.QE, 32 * O.AMU, ids=iid[:ni_])
        den_e = port.number_density(g, ele[:ne_])
        rho = -O.QE * den_e + O.QE * port.number_density(g, ion[:ni_])
        port.solve_fpcg(g, kind, phi, rho, 1e-10, 20000)
        ef = port.compute_ef(g, phi)
        if step >= skip:
            z = lambda a: a.reshape(nn[2], nn[1], nn[0])[:, :-1, :-1].mean(axis=(1, 2))
            prof["gpu_e"].append(z(e.den))
            prof["gpu_phi"].append(z(W.phi))
            prof["ora_e"].append(z(den_e))
            prof["ora_phi"].append(z(phi))
    ions_made[0] = M.stats()["ionizations"]
    assert ions_made[0] > 20 and ions_made[1] > 20  # the discharge ionises
    assert abs(ions_made[0] - ions_made[1]) <= 4 * np.sqrt(ions_made[0] + ions_made[1]) + 5

    def mean_se(a):
        a = np.array(a)
        b = a[: len(a) // blocks * blocks].reshape(blocks, -1, a.shape[1]).mean(axis=1)
        return a.mean(axis=0), b.std(axis=0, ddof=1) / np.sqrt(blocks)

    for key in ("e", "phi"):
        mg, sg = mean_se(prof["gpu_" + key])
        mo, so = mean_se(prof["ora_" + key])
        scale = np.max(np.abs(mo))
        tol = 4 * np.sqrt(sg ** 2 + so ** 2) + 0.02 * scale
        assert np.all(np.abs(mg - mo) <= tol), (key, np.max(np.abs(mg - mo) / scale))
