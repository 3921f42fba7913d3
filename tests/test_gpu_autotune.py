"""The launch-shape autotuner leaves the world's state as it was and picks valid shapes."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_keeps_state_and_picks_valid_shapes(pic):
    nn, x0, xm = (48, 48, 96), (0.0, 0.0, 0.0), (0.012, 0.012, 0.024)
    W = pic.World(*nn, x0, xm)
    W.set_boundaries((1, 1, 0), (1,) * 6, (0, 0, 0, 0, 0.0, 100.0))
    W.setTime(1e-12, 100)
    e = pic.Species("e-", pic.ME, -pic.QE, W, 10.0, capacity=600_000)
    i = pic.Species("O2+", 32 * pic.AMU, pic.QE, W, 10.0, capacity=600_000)
    e.loadUniform((0, 0, 0.006), (0.012, 0.012, 0.018), 500_000, 2 * 11604.5, 10.0, 0.5, seed=1)
    i.loadUniform((0, 0, 0.006), (0.012, 0.012, 0.018), 500_000, 0.03 * 11604.5, 10.0, 0.5, seed=2)
    S = pic.PotentialSolver(W, 5000, 1e-6, pic.SOLVER_PCG)
    W.configure_loop(solve_each_step=True, sort_every=20)
    assert S.solve(raise_on_fail=True)
    S.computeEF()
    for _ in range(3):
        W.step()
    before = [sp.getPartRef() for sp in (e, i)]
    rho0, phi0 = W.rho, W.phi
    t = W.autotune()
    assert 1 <= t["push_ctas_per_sm"] <= 4 and t["node_grid"] >= 1 and t["cg_grid"] >= 1
    assert W.launch_shapes() == t
    after = [sp.getPartRef() for sp in (e, i)]
    for a, b in zip(before, after):
        a, b = a[np.argsort(a["id"])], b[np.argsort(b["id"])]
        assert np.array_equal(a["pos"], b["pos"]) and np.array_equal(a["vel"], b["vel"])
    W.computeChargeDensity()
    assert np.array_equal(W.rho, rho0) and np.array_equal(W.phi, phi0)
    # the loop goes on with the tuned shapes and the solver stays exact
    for _ in range(3):
        W.step()
    assert S.solve(raise_on_fail=True) and S.rel <= 1e-6


def test_set_launch_shapes_validates_and_solves(pic):
    """Shapes carried over from an earlier run: range checks, and solves that stay exact with them."""
    nn, x0, xm = (32, 32, 64), (0.0, 0.0, 0.0), (0.008, 0.008, 0.016)
    W = pic.World(*nn, x0, xm)
    W.set_boundaries((1, 1, 0), (1,) * 6, (0, 0, 0, 0, 0.0, 100.0))
    W.setTime(1e-12, 100)
    e = pic.Species("e-", pic.ME, -pic.QE, W, 10.0, capacity=200_000)
    e.loadUniform((0, 0, 0.004), (0.008, 0.008, 0.012), 100_000, 2 * 11604.5, 10.0, 0.5, seed=3)
    W.computeChargeDensity()
    for bad in ((-1, 0, 0), (1000, 0, 0), (0, -5, 0), (0, 0, -2)):
        with pytest.raises(RuntimeError):
            W.set_launch_shapes(*bad)
    for method in (pic.SOLVER_PCG, pic.SOLVER_LEARNED):
        S = pic.PotentialSolver(W, 5000, 1e-6, method)
        phis = []
        for shapes in ((0, 0, 0), (1, 152, 152), (2, 1216, 608)):
            W.set_launch_shapes(*shapes)
            got = W.launch_shapes()
            assert got["node_grid"] == shapes[1] and got["cg_grid"] == shapes[2]
            W.phi = np.zeros(W.nv)
            assert S.solve(raise_on_fail=True) and S.rel <= 1e-6
            phis.append(W.phi)
        # other CTA counts only regroup the partial sums of the dot products
        scale = np.max(np.abs(phis[0]))
        for p in phis[1:]:
            assert np.max(np.abs(p - phis[0])) <= 1e-5 * scale
