"""Statistical parity of the collision model with the reference's own algorithm.

The GPU form draws electron-impact collisions against a Maxwellian background gas (null-collision
candidates, Philox draws).  The reference pairs electrons with neutral macroparticles per cell
(variable-weight NTC, MC_MEX_Ionization::apply, Interactions.cpp:600-762), restated bit-exactly in
the oracle and pinned by tests/golden/ntc.npz.  For neutral weights far above the electron weight
both have the same expectation: n_n sigma(E_rel) v_rel dt per electron and step.  These tests draw
independent realisations of both and compare collision and ionisation counts, and the energy the
electrons keep, within four combined standard errors plus the reference's own rounding of the
number of candidate pairs per cell (below 0.2 % here)."""
import numpy as np
import pytest

import oracle as O
from conftest import PKG_NAME  # noqa: F401  (the package fixture imports it)

pytestmark = pytest.mark.gpu

E_ION, LOTZ, MASS_N = 12.06, (2.107e-17, 1.0, 0.18, 0.0), 32 * O.AMU
N_N, T_N = 1e21, 300.0


def sigma_table():
    E = np.geomspace(0.01, 1e5, 300)
    return E, 6e-20 / np.sqrt(1 + E / 10.0)


def electrons(rng, n, xm, energy_eV):
    pos = rng.uniform((0, 0, 0), xm, (n, 3)) * 0.999999
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    vel = d * np.sqrt(2 * energy_eV * O.QE / O.ME)
    return pos, vel


def test_collision_and_ionisation_rates_match_reference_ntc(pic, port):
    nn, xm = (5, 5, 5), (0.004, 0.004, 0.004)  # 64 cells of 1 mm^3
    ncell = 64
    per_cell = 2000
    dt = 2e-10
    energy = 60.0
    g = port.grid(nn, (0, 0, 0), xm)
    E, S = sigma_table()
    cp = port.coll_params(E, S, MASS_N, E_ION, 1, (0.0, 1.0, 0.18), sig_A=LOTZ[0])
    rng = np.random.default_rng(21)
    ne = ncell * per_cell
    pos, vel = electrons(rng, ne, xm, energy)
    w_e = 1.0
    w_n = N_N * np.prod(xm) / ne  # as many neutral macroparticles as electrons, weight >> electron weight
    npos = rng.uniform((0, 0, 0), xm, (ne, 3)) * 0.999999
    nvel = rng.normal(size=(ne, 3)) * np.sqrt(O.KB * T_N / MASS_N)

    # ---- reference NTC, independent realisations on fresh copies of the same particles
    cap = 3 * ne

    def fresh():
        ele = np.zeros(cap, O.PARTICLE)
        neu = np.zeros(cap, O.PARTICLE)
        ele[:ne]["pos"], ele[:ne]["vel"], ele[:ne]["w"] = pos, vel, w_e
        neu[:ne]["pos"], neu[:ne]["vel"], neu[:ne]["w"] = npos, nvel, w_n
        return ele, neu, np.zeros(cap, O.PARTICLE)

    # the majorant sigma v w from one call, as after the reference's first step
    ele, neu, ion = fresh()
    _, _, _, _, wsv = port.ntc_ionize_ref(g, cp, port.mt(1), neu, ne, ion, 0, ele, ne, dt, 1e-3)
    K = 16
    ref_coll = ref_ion = 0
    ref_energy = []
    for k in range(K):
        ele, neu, ion = fresh()
        nc, _, ni_, ne2, _ = port.ntc_ionize_ref(g, cp, port.mt(100 + k), neu, ne, ion, 0, ele, ne, dt, wsv)
        ref_coll += nc
        ref_ion += ni_
        ref_energy.append(np.sum(ele[:ne2]["vel"] ** 2))

    # ---- GPU form: K times as many electrons in one application
    W = pic.World(*nn, (0, 0, 0), xm)
    W.setTime(dt, 10)
    W.advanceTime()
    e = pic.Species("e-", pic.ME, -pic.QE, W, w_e, capacity=3 * K * ne)
    i = pic.Species("O2+", MASS_N, pic.QE, W, w_e, capacity=3 * K * ne)
    gpos = np.concatenate([pos] * K)
    gvel = np.concatenate([electrons(np.random.default_rng(100 + k), ne, xm, energy)[1] for k in range(K)])
    e.addParticles(gpos, gvel, np.full(K * ne, w_e), rewind=False)
    M = pic.MC_MEX_Ionization(e, i, W, N_N, T_N, MASS_N, E_ION, E, S, 1, LOTZ, seed=77)
    M.apply(dt)
    st = M.stats()
    gp = e.getPartRef()
    gpu_energy = np.sum(gp["vel"] ** 2)

    n_samples = K * ne
    # expected collision probability per electron (the sanity scale): n sigma v dt
    for name, a, b in (("collisions", st["collisions"], ref_coll), ("ionisations", st["ionizations"], ref_ion)):
        assert a > 1000 and b > 1000, (name, a, b)
        se = np.sqrt(1.0 / a + 1.0 / b)
        assert abs(a / b - 1.0) <= 4 * se + 0.005, (name, a, b, 4 * se)
        # both are per-electron probabilities of the same size
        assert abs(a / n_samples - b / n_samples) <= 0.01
    # energy bookkeeping: the energy the electrons lose (ionisation thresholds, recoil) per
    # ionisation agrees, so both share the ejected electron's energy the same way on average
    e0 = np.sum(vel ** 2)
    loss_ref = (e0 - np.mean(ref_energy)) / (ref_ion / K)
    loss_gpu = (e0 - gpu_energy / K) / (st["ionizations"] / K)
    assert loss_ref > 0 and loss_gpu > 0
    assert abs(loss_gpu / loss_ref - 1.0) <= 0.02, (loss_gpu, loss_ref)
