"""Stacked independent instances (one world, instance slabs along z) against the same instances
run as separate worlds: potential, E field, particles, densities and collision counts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NI, NJ, NKS = 17, 17, 20          # nodes per instance
DZ = 0.0005
LX = LY = 0.008
VOLT = (100.0, 200.0, 300.0)      # anode potential per instance
DENS = (1e21, 2e21, 3e21)         # background density per instance
ME, QE, AMU = 9.10938215e-31, 1.602176565e-19, 1.660538921e-27


def sigma_table():
    E = np.geomspace(0.01, 1e5, 300)
    return E, 6e-20 / np.sqrt(1 + E / 10.0)


def particles(s, n, mass, T, rng):
    pos = np.column_stack([rng.uniform(0, LX, n), rng.uniform(0, LY, n), rng.uniform(2 * DZ, (NKS - 3) * DZ, n)])
    vel = rng.normal(size=(n, 3)) * np.sqrt(1.380648e-23 * T / mass)
    ids = (np.arange(n, dtype=np.uint64) + np.uint64(1_000_000 * (s + 1)))
    return pos, vel, np.full(n, 5e4), ids


def build(pic, nk, zmax, slabs, volts, dens, parts):
    W = pic.World(NI, NJ, nk, (0.0, 0.0, 0.0), (LX, LY, zmax))
    if slabs:
        W.set_boundaries((1, 1, 0), (1,) * 6, (0.0,) * 6)
        W.set_slabs([0.0] * len(volts), volts)
    else:
        W.set_boundaries((1, 1, 0), (1,) * 6, (0, 0, 0, 0, 0.0, volts[0]))
    W.setTime(2e-11, 100)
    e = pic.Species("e-", pic.ME, -pic.QE, W, 5e4, capacity=40000)
    i = pic.Species("O2+", 32 * AMU, pic.QE, W, 5e4, capacity=40000)
    for (sp, key) in ((e, "e"), (i, "i")):
        pos, vel, w, ids = parts[key]
        sp.addParticles(pos, vel, w, ids=ids, rewind=False)
    E, S = sigma_table()
    M = pic.MC_MEX_Ionization(e, i, W, dens[0], 300.0, 32 * AMU, 12.06, E, S, sigma_ion_kind=1,
                              sigma_ion_params=(2.107e-17, 1.0, 0.18, 0.0), seed=77)
    if slabs:
        M.set_slab_density(dens)
    W.configure_loop(solve_each_step=True, sort_every=1000)
    S_ = pic.PotentialSolver(W, 20000, 1e-10, pic.SOLVER_PCG)
    assert S_.solve(raise_on_fail=True)
    S_.computeEF()
    return W, e, i, M


def test_stacked_instances_match_separate_worlds(pic):
    rng = np.random.default_rng(4)
    per = []
    for s in range(len(VOLT)):
        per.append({"e": particles(s, 3000, ME, 2 * 11604.5, rng), "i": particles(s, 3000, 32 * AMU, 300.0, rng)})
    # separate worlds
    sep = [build(pic, NKS, (NKS - 1) * DZ, False, (VOLT[s],), (DENS[s],), per[s]) for s in range(len(VOLT))]
    # one world with the instances stacked along z
    stacked_parts = {}
    for key in ("e", "i"):
        pos = np.concatenate([per[s][key][0] + np.array([0, 0, s * NKS * DZ]) for s in range(len(VOLT))])
        vel = np.concatenate([per[s][key][1] for s in range(len(VOLT))])
        w = np.concatenate([per[s][key][2] for s in range(len(VOLT))])
        ids = np.concatenate([per[s][key][3] for s in range(len(VOLT))])
        stacked_parts[key] = (pos, vel, w, ids)
    nk = NKS * len(VOLT)
    W, e, i, M = build(pic, nk, (nk - 1) * DZ, True, VOLT, DENS, stacked_parts)

    def compare_fields(Wst, sep_worlds):
        phi = Wst.phi.reshape(nk, NJ, NI)
        ef = Wst.ef.reshape(nk, NJ, NI, 3)
        for s, (Ws, *_rest) in enumerate(sep_worlds):
            a, b = phi[s * NKS:(s + 1) * NKS], Ws.phi.reshape(NKS, NJ, NI)
            assert np.max(np.abs(a - b)) <= 1e-6 * np.max(np.abs(b)), s
            ea, eb = ef[s * NKS:(s + 1) * NKS], Ws.ef.reshape(NKS, NJ, NI, 3)
            assert np.max(np.abs(ea - eb)) <= 1e-5 * np.max(np.abs(eb)), s

    compare_fields(W, sep)
    for _ in range(3):
        W.step()
        for Ws, *_rest in sep:
            Ws.step()
    compare_fields(W, sep)
    # particles, by id
    for key, sp_st in (("e", e), ("i", i)):
        got = sp_st.getPartRef()
        for s, (Ws, es, is_, Ms) in enumerate(sep):
            ref = (es if key == "e" else is_).getPartRef()
            lo, hi = 1_000_000 * (s + 1), 1_000_000 * (s + 2)
            mine = got[(got["id"] >= lo) & (got["id"] < hi)]
            ref = ref[(ref["id"] >= lo) & (ref["id"] < hi)]
            mine = mine[np.argsort(mine["id"])]
            ref = ref[np.argsort(ref["id"])]
            assert len(mine) == len(ref)
            assert np.array_equal(mine["id"], ref["id"])
            dpos = mine["pos"] - np.array([0, 0, s * NKS * DZ]) - ref["pos"]
            assert np.max(np.abs(dpos)) <= 1e-7, (key, s)
            assert np.allclose(mine["vel"], ref["vel"], rtol=1e-4, atol=1e-3 * np.abs(ref["vel"]).max())
    # collision counts and densities
    st = M.stats()
    tot = {k: sum(Ms.stats()[k] for _W, _e, _i, Ms in sep) for k in ("candidates", "collisions")}
    assert abs(st["candidates"] - tot["candidates"]) <= 2
    assert abs(st["collisions"] - tot["collisions"]) <= 2
    den = e.den.reshape(nk, NJ, NI)
    for s, (Ws, es, _i, _M) in enumerate(sep):
        ref = es.den.reshape(NKS, NJ, NI)
        assert np.max(np.abs(den[s * NKS:(s + 1) * NKS] - ref)) <= 1e-5 * np.max(ref), s
