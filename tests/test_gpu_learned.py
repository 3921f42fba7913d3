"""Learned multilevel Poisson preconditioner: hierarchy, apply and solves against the numpy
restatement in oracle/learned_ref.py (FP64), through the C ABI."""
import numpy as np
import pytest

import learned_ref as LR

pytestmark = pytest.mark.gpu

GEOMS = {
    # periodic x, y (distinct 16 x 16), Dirichlet z planes
    "periodic_even": dict(nn=(17, 17, 19), xm=(0.016, 0.016, 0.018), per=(1, 1, 0)),
    # periodic with odd distinct counts (15 and 13) and a non-cubic spacing
    "periodic_odd": dict(nn=(16, 14, 11), xm=(0.015, 0.026, 0.01), per=(1, 1, 0)),
    # all walls Dirichlet, odd extents
    "dirichlet_odd": dict(nn=(13, 11, 9), xm=(0.012, 0.01, 0.008), per=(0, 0, 0)),
}


def make_world(pic, geom, top=0.0):
    g = GEOMS[geom]
    W = pic.World(*g["nn"], (0.0, 0.0, 0.0), g["xm"])
    W.set_boundaries(g["per"], (1,) * 6, (0.0, 0.0, 0.0, 0.0, 0.0, top))
    return W, g


def distinct(a, g):
    """Node array -> [z, y, x] array over the distinct nodes (periodic copies dropped)."""
    ni, nj, nk = g["nn"]
    a = np.asarray(a).reshape(nk, nj, ni)
    return a[:nk - g["per"][2], :nj - g["per"][1], :ni - g["per"][0]]


def free_mask(g):
    ni, nj, nk = g["nn"]
    m = np.ones((nk, nj, ni))
    for d in range(3):  # Dirichlet walls on the non-periodic axes (x = 0, y = 1, z = 2)
        if not g["per"][d]:
            sl = [slice(None)] * 3
            sl[2 - d] = 0
            m[tuple(sl)] = 0
            sl[2 - d] = g["nn"][d] - 1
            m[tuple(sl)] = 0
    return distinct(m.ravel(), g)


def coeffs(g):
    return tuple(((n - 1) / x) ** 2 for n, x in zip(g["nn"], g["xm"]))  # (cx, cy, cz)


def unpack(wflat):
    """Flat parameter array -> the oracle's weight dictionary."""
    W = {"S0": wflat[:27].astype(np.float64), "net": []}
    off = 27
    for C in LR.CHANNELS:
        Wl = wflat[off:off + 27 * C].reshape(C, 27)
        off += 27 * C
        Wm = wflat[off:off + C * C].reshape(C, C)
        off += C * C
        Wp = wflat[off:off + 27 * C].reshape(27, C)
        off += 27 * C
        W["net"].append({"Wl": Wl.astype(np.float64), "Wm": Wm.astype(np.float64), "Wp": Wp.astype(np.float64)})
    assert off == len(wflat)
    return W


@pytest.mark.parametrize("geom", sorted(GEOMS))
def test_levels_and_galerkin_diagonals(pic, geom):
    W, g = make_world(pic, geom)
    dims, diag = pic.LearnedPreconditioner(W).levels()
    shape0 = distinct(np.zeros(int(np.prod(g["nn"]))), g).shape
    shapes = LR.level_shapes(shape0)
    assert [tuple(d[::-1]) for d in dims] == shapes
    assert np.allclose(diag, LR.level_diags(coeffs(g), len(shapes)), rtol=1e-12)


@pytest.mark.parametrize("geom", sorted(GEOMS))
@pytest.mark.parametrize("weights", ["start", "random"])
def test_apply_matches_oracle(pic, geom, weights):
    W, g = make_world(pic, geom)
    lp = pic.LearnedPreconditioner(W)
    w0 = lp.weights()
    rng = np.random.default_rng(11)
    if weights == "random":
        w = w0 + rng.normal(size=w0.size).astype(np.float32) * np.float32(0.2) * np.abs(w0).max()
        lp.set_weights(w)
    else:
        w = w0
    nv = int(np.prod(g["nn"]))
    r = rng.normal(size=nv)
    z = lp.apply(r)
    mask = free_mask(g)
    per = tuple(bool(p) for p in g["per"][::-1])
    _, diag = lp.levels()
    ref = LR.apply(distinct(r, g), mask, unpack(w), per, diag)
    got = distinct(z, g)
    assert np.max(np.abs(got - ref)) <= 2e-5 * np.max(np.abs(ref))
    # periodic copies and non-FREE nodes are zero
    full = np.zeros(nv, bool)
    full[distinct(np.arange(nv), g).ravel()[mask.ravel() > 0]] = True
    assert np.all(z[~full] == 0)


def test_start_weights_are_bpx(pic):
    W, g = make_world(pic, "periodic_even")
    lp = pic.LearnedPreconditioner(W)
    _, diag = lp.levels()
    ref = LR.init_weights(diag)
    got = unpack(lp.weights())
    assert np.allclose(got["S0"], ref["S0"], rtol=1e-7)
    for a, b in zip(got["net"], ref["net"]):
        for k in ("Wl", "Wm", "Wp"):
            assert np.allclose(a[k], b[k], rtol=1e-7, atol=0)


def test_learned_solve_needs_far_fewer_iterations_than_jacobi(pic, port):
    """65^3 nodes, periodic x, y, Dirichlet z at 0 V / 100 V, blob charge: the learned
    preconditioner (BPX start) against Jacobi, both to the same FP64 residual."""
    n = 65
    W = pic.World(n, n, n, (0.0, 0.0, 0.0), (0.02, 0.02, 0.02))
    W.set_boundaries((1, 1, 0), (1,) * 6, (0, 0, 0, 0, 0.0, 100.0))
    rng = np.random.default_rng(3)
    zz, yy, xx = np.meshgrid(*[np.arange(n)] * 3, indexing="ij")
    rho = np.zeros((n, n, n))
    for _ in range(16):
        c = rng.uniform(0, n, 3)
        wd = rng.uniform(2, 10)
        rho += rng.choice([-1, 1]) * 1e-3 * np.exp(-((zz - c[0]) ** 2 + (yy - c[1]) ** 2 + (xx - c[2]) ** 2) / (2 * wd * wd))
    W.rho = rho.ravel()
    phi0 = W.phi
    out = {}
    for name, m in (("pcg", pic.SOLVER_PCG), ("learned", pic.SOLVER_LEARNED)):
        W.phi = phi0
        S = pic.PotentialSolver(W, 20000, 1e-8, m)
        assert S.solve(raise_on_fail=True)
        out[name] = (S.iters, W.phi)
    assert out["learned"][0] * 5 < out["pcg"][0]
    a, b = out["learned"][1], out["pcg"][1]
    assert np.max(np.abs(a - b)) <= 1e-6 * np.max(np.abs(b))


GRAD_GEOM = dict(nn=(33, 33, 35), xm=(0.032, 0.032, 0.034), per=(1, 1, 0))


def test_loss_and_gradients_match_oracle(pic):
    """One forward + backward of the device training path (tensor-core GEMMs on BF16 operands,
    FP32 accumulation) against the FP64 oracle, on perturbed weights so that every channel of the
    four network levels carries signal.  BF16 rounding of the activations bounds the agreement."""
    GEOMS["grad"] = GRAD_GEOM
    try:
        W, g = make_world(pic, "grad")
    finally:
        del GEOMS["grad"]
    lp = pic.LearnedPreconditioner(W)
    dims, diag = lp.levels()
    assert len(dims) >= 5  # all four network levels exist
    rng = np.random.default_rng(5)
    w = lp.weights()
    groups = [(0, 27)]
    off = 27
    for C in LR.CHANNELS:
        groups += [(off, 27 * C), (off + 27 * C, C * C), (off + 27 * C + C * C, 27 * C)]
        off += 54 * C + C * C
    for a, n in groups:
        scale = np.abs(w[a:a + n]).max()
        w[a:a + n] += (rng.normal(size=n) * 0.3 * scale).astype(np.float32)
    lp.set_weights(w)
    nv = int(np.prod(g["nn"]))
    x = rng.normal(size=nv)
    mask = free_mask(g)
    per = tuple(bool(p) for p in g["per"][::-1])
    c = coeffs(g)
    xd = distinct(x, g) * mask
    rd = LR.apply_L(xd, mask, c, per)
    # r on the node array (periodic copies are not read)
    r = np.zeros(nv)
    idx = distinct(np.arange(nv), g)
    r[idx.ravel()] = rd.ravel()
    loss, grad = lp.loss_grad(r, x)
    ref_loss, G = LR.loss_and_grads(rd, xd, mask, unpack(w), c, per, diag, scale_free=False)
    assert abs(loss - ref_loss) <= 0.02 * abs(ref_loss)
    ref = [G["S0"]]
    for lv in G["net"]:
        ref += [lv["Wl"].ravel(), lv["Wm"].ravel(), lv["Wp"].ravel()]
    for (a, n), gr in zip(groups, ref):
        got = grad[a:a + n].astype(np.float64)
        err = np.linalg.norm(got - gr) / np.linalg.norm(gr)
        assert err <= 0.05, (a, n, err)


def test_training_is_judged_by_the_solver_and_keeps_solves_exact(pic):
    """Online learning judged by the solver: level gains calibrated by validation solves on the
    right-hand side of an earlier solve, then gradient rounds on white-noise pairs.  A round is kept
    only if a validation solve needs no more iterations than before it (otherwise it is rolled
    back).  The trained preconditioner needs clearly fewer iterations than its starting (BPX) form on
    a new right-hand side, and still drives the solve to the same FP64 residual, with far fewer
    iterations than Jacobi-PCG."""
    n = 49
    W = pic.World(n, n, n, (0.0, 0.0, 0.0), (0.02, 0.02, 0.02))
    W.set_boundaries((1, 1, 0), (1,) * 6, (0, 0, 0, 0, 0.0, 50.0))
    lp = pic.LearnedPreconditioner(W)
    lp.collect(True)
    rng = np.random.default_rng(9)
    zz, yy, xx = np.meshgrid(*[np.arange(n)] * 3, indexing="ij")

    def blobs():
        rho = np.zeros((n, n, n))
        for _ in range(rng.integers(8, 33)):
            cc = rng.uniform(0, n, 3)
            wd = rng.uniform(2, 8)
            rho += rng.choice([-1, 1]) * 1e-3 * np.exp(
                -((zz - cc[0]) ** 2 + (yy - cc[1]) ** 2 + (xx - cc[2]) ** 2) / (2 * wd * wd))
        return rho.ravel()

    phi0 = W.phi
    S = pic.PotentialSolver(W, 20000, 1e-8, pic.SOLVER_LEARNED)
    for _ in range(4):  # four solves provide training pairs
        W.phi = phi0
        W.rho = blobs()
        assert S.solve(raise_on_fail=True)
    lp.collect(False)
    rho_test = blobs()
    W.phi = phi0
    W.rho = rho_test
    assert S.solve(raise_on_fail=True)
    iters_start = S.iters
    # level gains first: kept only when validation solves get shorter
    cal_before, cal_after = lp.calibrate()
    assert cal_after < cal_before
    rounds = []
    for _ in range(3):
        loss, before, after, kept = lp.train(100, lr=1e-3, pair_every=0)
        assert np.isfinite(loss)
        assert (after <= before) == kept
        rounds.append((before, after, kept))
    # the trainer keeps B symmetric (k_lp_symmetrize): x.By = y.Bx
    mask = (W.node_type == 0).astype(float)
    xv, yv = rng.normal(size=W.nv) * mask, rng.normal(size=W.nv) * mask
    a, b = np.dot(xv, lp.apply(yv)), np.dot(yv, lp.apply(xv))
    assert abs(a - b) <= 1e-4 * max(abs(a), abs(b))
    W.phi = phi0
    W.rho = rho_test
    assert S.solve(raise_on_fail=True)
    learned_iters, phi_l = S.iters, W.phi
    # what training gains over the starting (BPX) preconditioner on a right-hand side it never saw
    assert learned_iters < 0.85 * iters_start, (iters_start, learned_iters, cal_before, cal_after, rounds)
    W.phi = phi0
    P = pic.PotentialSolver(W, 20000, 1e-8, pic.SOLVER_PCG)
    assert P.solve(raise_on_fail=True)
    assert learned_iters * 5 < P.iters
    assert np.max(np.abs(phi_l - W.phi)) <= 1e-6 * np.max(np.abs(W.phi))
