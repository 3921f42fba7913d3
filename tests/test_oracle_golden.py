"""The FP64 oracle restatement (oracle/pic_oracle.c) against golden vectors produced by the
reference's own ch4/v3 code (tests/golden/make_golden.py).  Bit-exact: same loop order, same
FP64 operation order, same MT19937 draws."""
import numpy as np
import pytest

import oracle as O
from conftest import golden


def to_parts(d, prefix):
    n = len(d[prefix + "w"])
    p = np.zeros(n, O.PARTICLE)
    p["pos"], p["vel"], p["w"] = d[prefix + "pos"], d[prefix + "vel"], d[prefix + "w"]
    return p


def test_mt19937_canonical_matches_std(port):
    # first outputs of std::mt19937(5489) are published; canonical doubles combine two draws
    r = port.mt(5489)
    first = [port.lib.or_mt_u01(C_byref(r)) for _ in range(2)]
    assert 0.0 <= first[0] < 1.0 and 0.0 <= first[1] < 1.0
    r2 = port.mt(5489)
    import ctypes as C

    port.lib.or_mt_next.restype = C.c_uint32
    port.lib.or_mt_next.argtypes = [C.c_void_p]
    assert port.lib.or_mt_next(C.byref(r2)) == 3499211612  # mt19937 reference output #1
    assert port.lib.or_mt_next(C.byref(r2)) == 581869302


def C_byref(x):
    import ctypes as C

    return C.byref(x)


def test_philox_known_answer(port):
    # Philox-4x32-10 known-answer vectors (Random123 kat_vectors)
    assert list(port.philox([0, 0, 0, 0], [0, 0])) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert list(port.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert list(port.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0])) == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_candidate_draw_restatement_and_statistics(port):
    """The null-collision candidate draw (output step + 1 of a SplitMix64 stream seeded by the
    scrambled id ^ seed): the C restatement equals this numpy one, and the test id draw < T
    selects a fraction T / 2^32 of the particles, independently from step to step."""
    M = np.uint64(0xFFFFFFFFFFFFFFFF)

    def mix(x):
        x = x.astype(np.uint64)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return x ^ (x >> np.uint64(31))

    seed = 0x1234_5678_9ABC_DEF0
    ids = (np.arange(200000, dtype=np.uint64) * np.uint64(7) + np.uint64(3)) & M
    with np.errstate(over="ignore"):
        s = mix(ids ^ np.uint64(seed))
        draws = {st: (mix(s + np.uint64(0x9E3779B97F4A7C15) * np.uint64(st + 1)) >> np.uint64(32)).astype(np.uint32)
                 for st in (0, 1, 2)}
    for k in range(0, 200000, 9973):
        for st in (0, 1, 2):
            assert port.lib.or_cand_draw(int(ids[k]), st, seed & 0xFFFFFFFF, seed >> 32) == draws[st][k]
    p = 0.01
    T = port.lib.or_cand_threshold(p)
    assert T == int(p * 2 ** 32) and port.lib.or_cand_threshold(2.0) == 2 ** 32 - 1
    assert port.lib.or_cand_threshold(0.0) == 0
    n = len(ids)
    sel = [draws[st] < T for st in (0, 1, 2)]
    for a in sel:
        assert abs(a.sum() - n * p) <= 5 * np.sqrt(n * p)
    both = (sel[0] & sel[1]).sum()  # independent steps: n p^2 joint selections
    assert abs(both - n * p * p) <= 5 * np.sqrt(n * p * p) + 1


def test_load_push_deposit_bit_exact(port):
    d = golden("push_deposit")
    g = port.grid(d["nn"], d["x0"], d["xm"])
    # loadParticleBoxThermal with the reference's MT19937 stream
    mt = port.mt(7)
    loaded = port.load_box_thermal_ref(g, mt, 100000, (0, 0.008, 0.015), (0.018, 0.014, 0.028), 1e10, 30000.0, 100.0,
                                       O.ME, -O.QE)
    ref_in = to_parts(d, "in_")
    assert len(loaded) == len(ref_in)
    assert np.array_equal(loaded["pos"], ref_in["pos"]) and np.array_equal(loaded["vel"], ref_in["vel"])
    p = ref_in.copy()
    n = port.push(g, p, d["ef"], float(d["dt"]), -O.QE, O.ME)
    out = to_parts(d, "out_")
    assert n == len(out)
    assert np.array_equal(p[:n]["pos"], out["pos"]) and np.array_equal(p[:n]["vel"], out["vel"])
    den = port.number_density(g, p[:n])
    assert np.array_equal(den, d["den"])


def test_multithreaded_push_same_set(port):
    d = golden("push_deposit")
    g = port.grid(d["nn"], d["x0"], d["xm"])
    a = to_parts(d, "in_")
    b = a.copy()
    ids = np.arange(len(b), dtype=np.uint64)
    na = port.push(g, a, d["ef"], float(d["dt"]), -O.QE, O.ME)
    nb = port.push(g, b, d["ef"], float(d["dt"]), -O.QE, O.ME, ids=ids, threads=4)
    assert na == nb
    ka = np.lexsort(a[:na]["pos"].T)
    kb = np.lexsort(b[:nb]["pos"].T)
    assert np.array_equal(a[:na]["pos"][ka], b[:nb]["pos"][kb])


@pytest.mark.parametrize("mode", ["dirichlet", "v3box"])
def test_poisson_and_efield_bit_exact(port, mode):
    d = golden("poisson")
    boxes = [] if mode == "dirichlet" else [(d["box_c"], d["box_s"])]
    g = port.grid(d["nn"], d["x0"], d["xm"], boxes=boxes)
    kind = port.node_kinds(g, 1 if mode == "dirichlet" else 0)
    phi0 = np.zeros(port.nv(g))
    if mode == "v3box":
        phi0[kind == O.FIXED] = float(d["box_phi"])
    # GS (PotentialSolver::solveGS)
    phi = phi0.copy()
    ok, it, l2 = port.solve_gs(g, kind, phi, d["rho"], 20000, 1e-6)
    assert bool(ok) == bool(d[f"{mode}_gs_ok"])
    assert np.array_equal(phi, d[f"{mode}_gs_phi"])
    assert np.array_equal(port.compute_ef(g, phi), d[f"{mode}_gs_ef"])
    # NR-PCG with the reference's coefficient assignment (PotentialSolver::buildMatrix)
    phi = phi0.copy()
    ok, it, l2 = port.solve_pcg_ref(g, kind, phi, d["rho"], 2000, 1e-6, axis_swap=1)
    assert bool(ok == 1) == bool(d[f"{mode}_pcg_ok"])
    assert np.array_equal(phi, d[f"{mode}_pcg_phi"])
    assert np.array_equal(port.compute_ef(g, phi), d[f"{mode}_pcg_ef"])


@pytest.mark.parametrize("mode", ["dirichlet", "v3box"])
def test_gpu_form_solvers_reach_reference_solution(port, mode):
    """Red-black SOR and flexible PCG on the reduced system converge to the reference GS answer."""
    d = golden("poisson")
    boxes = [] if mode == "dirichlet" else [(d["box_c"], d["box_s"])]
    g = port.grid(d["nn"], d["x0"], d["xm"], boxes=boxes)
    kind = port.node_kinds(g, 1 if mode == "dirichlet" else 0)
    phi0 = np.zeros(port.nv(g))
    if mode == "v3box":
        phi0[kind == O.FIXED] = float(d["box_phi"])
    ref = phi0.copy()
    port.solve_gs(g, kind, ref, d["rho"], 200000, 1e-13)
    for solver in ("rbsor", "fpcg"):
        phi = phi0.copy()
        if solver == "rbsor":
            ok, _, rel = port.solve_rbsor(g, kind, phi, d["rho"], 1.6, 1e-12, 100000)
        else:
            ok, _, rel = port.solve_fpcg(g, kind, phi, d["rho"], 1e-12, 10000)
        assert ok and rel <= 1e-12
        assert np.max(np.abs(phi - ref)) <= 1e-9 * max(1.0, np.max(np.abs(ref)))


def test_ntc_ionization_bit_exact(port):
    d = golden("ntc")
    g = port.grid(d["nn"], d["x0"], d["xm"])
    e_ion = 1313.9 * 1000 / 6.02214076e23 / O.QE
    cp = port.coll_params(d["table_E"], d["table_s"], 16 * O.AMU, e_ion)
    mt = port.mt(int(d["seed"]))
    # replay the two loads to bring the MT19937 stream to the same state
    c, s = (0.002, 0.002, 0.0025), (0.004, 0.004, 0.005)
    e0 = port.load_box_thermal_ref(g, mt, 10 ** 5, c, s, 2.5e12, 11604 * 300.0, 100.0, O.ME, -O.QE)
    n0 = port.load_box_thermal_ref(g, mt, 10 ** 5, c, s, 1.25e22, 300.0, 5e11, 16 * O.AMU, 0.0)
    assert np.array_equal(e0["vel"], d["ele0_vel"]) and np.array_equal(n0["pos"], d["neu0_pos"])
    cap = 20000
    ele = np.zeros(cap, O.PARTICLE)
    neu = np.zeros(cap, O.PARTICLE)
    ion = np.zeros(cap, O.PARTICLE)
    ele[:len(e0)], neu[:len(n0)] = e0, n0
    ne, nn_, ni_ = len(e0), len(n0), 0
    wsv = float(d["wsv0"])
    for it in (1, 2):
        _, nn_, ni_, ne, wsv = port.ntc_ionize_ref(g, cp, mt, neu, nn_, ion, ni_, ele, ne, float(d["dt"]), wsv)
        for nm, arr, n in (("ele", ele, ne), ("neu", neu, nn_), ("ion", ion, ni_)):
            ref = to_parts(d, f"{nm}{it}_")
            assert n == len(ref), (nm, it)
            for f in ("pos", "vel", "w"):
                assert np.array_equal(arr[:n][f], ref[f]), (nm, it, f)


def test_merge_bit_exact(port):
    d = golden("merge")
    g = port.grid(d["nn"], d["x0"], d["xm"])
    mt = port.mt(int(d["seed"]))
    loaded = port.load_box_thermal_ref(g, mt, 10 ** 5, (0.001, 0.0005, 0.0005), (0.002, 0.001, 0.001), 6e13,
                                       11604 * 2.0, 100.0, O.ME, -O.QE)
    ref_in = to_parts(d, "in_")
    assert np.array_equal(loaded["vel"], ref_in["vel"])
    p = np.zeros(4 * len(ref_in), O.PARTICLE)
    p[:len(ref_in)] = ref_in
    n = port.merge_ref(g, mt, p, len(ref_in), d["ef"], -O.QE, O.ME, float(d["dt"]), 10)
    out = to_parts(d, "out_")
    assert n == len(out)
    for f in ("pos", "vel", "w"):
        assert np.array_equal(p[:n][f], out[f]), f


def test_merge_conserves_mass_momentum_energy(port):
    d = golden("merge")
    g = port.grid(d["nn"], d["x0"], d["xm"])
    p0 = to_parts(d, "in_")
    p = np.zeros(4 * len(p0), O.PARTICLE)
    p[:len(p0)] = p0
    mt = port.mt(1)
    zero = np.zeros_like(d["ef"])  # no rewind so the moments must be preserved
    n = port.merge_ref(g, mt, p, len(p0), zero, -O.QE, O.ME, 0.0, 10)
    assert n < len(p0)
    c0, m0, k0 = port.sums(p0, O.ME)
    c1, m1, k1 = port.sums(p[:n], O.ME)
    assert abs(c1 - c0) <= 1e-12 * c0
    assert np.all(np.abs(m1 - m0) <= 1e-9 * np.abs(m0).max())
    assert abs(k1 - k0) <= 1e-9 * k0


def test_moments_and_gas_properties_bit_exact(port):
    d = golden("push_deposit")
    g = port.grid(d["nn"], d["x0"], d["xm"])
    p = to_parts(d, "out_")
    mom = port.sample_moments(g, p)
    mom = port.sample_moments(g, p, mom)  # accumulated twice, as the golden run
    vel, T = port.gas_properties(g, mom, O.ME)
    assert np.array_equal(vel, d["gas_vel"]) and np.array_equal(T, d["gas_T"])


def test_learned_symmetrize_makes_the_preconditioner_symmetric():
    """The trainer's projection (learned_ref.symmetrize, as csrc/pic_learned.cu k_lp_symmetrize)
    turns arbitrary weights into a symmetric B, and leaves the start weights as they are."""
    import learned_ref as LR

    shape, per = (17, 16, 16), (0, 1, 1)
    mask = np.ones(shape)
    mask[0] = mask[-1] = 0
    c = (1e6, 1e6, 1e6)
    nlev = len(LR.level_shapes(shape))
    diags = LR.level_diags(c, nlev)
    W0 = LR.init_weights(diags)
    W1 = LR.symmetrize(LR.init_weights(diags), diags)
    assert np.array_equal(W0["S0"], W1["S0"])
    for a, b in zip(W0["net"], W1["net"]):
        for k in ("Wl", "Wm", "Wp"):
            assert np.allclose(a[k], b[k], rtol=1e-15, atol=0)
    rng = np.random.default_rng(4)
    W = LR.init_weights(diags)
    W["S0"] += rng.normal(size=27) / diags[0]
    for l, w in enumerate(W["net"], start=1):
        for k in ("Wl", "Wm", "Wp"):
            dl = diags[l] if l < len(diags) else 1.0
            w[k] += rng.normal(size=w[k].shape) * (0.3 / dl if k == "Wp" else 0.3)
    x, y = rng.normal(size=shape) * mask, rng.normal(size=shape) * mask
    B = lambda v: LR.apply(v, mask, W, per, diags)
    assert abs(np.vdot(x, B(y)) - np.vdot(y, B(x))) > 1e-3 * abs(np.vdot(x, B(y)))  # not symmetric yet
    LR.symmetrize(W, diags)
    assert abs(np.vdot(x, B(y)) - np.vdot(y, B(x))) <= 1e-10 * abs(np.vdot(x, B(y)))


def test_dsmc_bit_exact(port):
    """DSMC_MEX one species (three applies) and two species (two applies) against the reference."""
    d = golden("dsmc")
    g = port.grid(d["nn"], d["x0"], d["xm"])
    mpw0, dt = float(d["mpw0"]), float(d["dt"])
    a, b = to_parts(d, "a0_"), to_parts(d, "b0_")
    mt = port.mt(int(d["dsmc_seed"]))
    q = port.dsmc_params(g, 16 * O.AMU, 16 * O.AMU, mpw0)
    sv = 1e-14  # DSMC_MEX::sigma_v_rel_max initial value (Interactions.h:58)
    total = 0
    for it in (1, 2, 3):
        nc, pairs, sv = port.dsmc_ref(g, q, mt, a, None, dt, sv)
        total += nc
        assert pairs >= nc and np.array_equal(a["vel"], d[f"one{it}_vel"]), it
        assert sv == float(d[f"one{it}_svmax"])
    assert total > 100  # the case collides
    q2 = port.dsmc_params(g, 16 * O.AMU, 32 * O.AMU, mpw0)
    sv = 1e-14
    for it in (1, 2):
        nc, pairs, sv = port.dsmc_ref(g, q2, mt, a, b, dt, sv)
        assert nc > 10
        assert np.array_equal(a["vel"], d[f"two{it}_vel_a"]) and np.array_equal(b["vel"], d[f"two{it}_vel_b"]), it
        assert sv == float(d[f"two{it}_svmax"])


def test_object_interaction_bit_exact(port):
    """Species::advanceNonElectron with a Rectangle: neutral bounces, ion neutralisation with
    sputtering (Species.cpp:45-256, Object.cpp:231-302), three steps against the reference."""
    d = golden("objects")
    g = port.grid(d["nn"], d["x0"], d["xm"], boxes=[(tuple(d["box_c"]), tuple(d["box_s"]))])
    mt = port.mt(int(d["obj_seed"]))
    cap = 10000
    neu, ion, spu = np.zeros(cap, O.PARTICLE), np.zeros(cap, O.PARTICLE), np.zeros(cap, O.PARTICLE)
    n0, i0 = to_parts(d, "neu0_"), to_parts(d, "ion0_")
    neu[:len(n0)], ion[:len(i0)] = n0, i0
    nn_, ni_, ns_ = len(n0), len(i0), 0
    m = 16 * O.AMU
    for it in (1, 2, 3):
        nn_, _, _ = port.push_nonelectron_ref(g, mt, neu, nn_, d["ef"], float(d["dt_n"]), 0.0, m, neu, nn_, 1e9,
                                              dt_global=float(d["dt_i"]))
        ni_, nn_, ns_ = port.push_nonelectron_ref(g, mt, ion, ni_, d["ef"], float(d["dt_i"]), O.QE, m, neu, nn_, 1e9,
                                                  spu, ns_, 5e8, True)
        for nm, arr, n in (("neu", neu, nn_), ("ion", ion, ni_), ("spu", spu, ns_)):
            ref = to_parts(d, f"{nm}{it}_")
            assert n == len(ref), (nm, it, n, len(ref))
            for f in ("pos", "vel", "w"):
                assert np.array_equal(arr[:n][f], ref[f]), (nm, it, f)


def test_moving_average_bit_exact():
    """oracle.moving_average_update against Species::updateAverages of the reference, over 45
    samples (two restarts of the 20-sample average)."""
    d = golden("averages")
    avg = np.zeros(d["den"].shape[1])
    samples = 0
    for it in range(len(d["den"])):
        samples = O.moving_average_update(avg, samples, d["den"][it])
        assert np.array_equal(avg, d["den_avg"][it]), it


def test_macro_particle_count_matches_reference(port):
    d = golden("averages")
    nn = tuple(int(v) for v in d["nn"])
    g = port.grid(nn, d["x0"], d["xm"])
    p = np.zeros(len(d["last_pos"]), O.PARTICLE)
    p["pos"] = d["last_pos"]
    got = O.macro_particle_count(g, p)
    assert got.sum() == len(p)
    assert np.array_equal(got, d["macro_count"])
