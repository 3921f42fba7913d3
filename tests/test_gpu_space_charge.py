"""The space-charge potential of a warm-started discharge loop is resolved.

On an electrode discharge the Dirichlet term of the anode dominates the right-hand side b of the
Poisson system: on 64 x 64 x 256 nodes with a 500 V anode and 2 M + 2 M particles,
||rho/eps0|| is about 1.4e-4 of ||b||, so a residual of 1e-6 ||b|| bounds the potential of the
space charge only to about 1 %.  The stopping rule PIC_STOP_REL_CHARGE measures the residual
against min(||b||, ||rho/eps0||) instead.  Here the loop runs warm-started steps under that rule
and the device potential is compared with the FP64 oracle's converged potential for the device's
final charge density, relative to the space-charge part phi - phi_vacuum (the vacuum potential
is linear in z for periodic x, y and Dirichlet z faces, exactly, on the grid too).
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def test_warm_started_loop_resolves_the_space_charge_potential(pic, port):
    nn, L, V = (64, 64, 256), (0.02, 0.02, 0.08), 500.0
    W = pic.World(*nn, (0.0, 0.0, 0.0), L)
    W.set_boundaries((1, 1, 0), (1,) * 6, (0, 0, 0, 0, 0.0, V))
    W.setTime(2e-12, 1000)
    e = pic.Species("e-", pic.ME, -pic.QE, W, 64.0, capacity=2_200_000)
    i = pic.Species("O2+", 32 * pic.AMU, pic.QE, W, 64.0, capacity=2_200_000)
    lo, hi = (0.0, 0.0, 0.3 * L[2]), (L[0], L[1], 0.7 * L[2])
    e.loadUniform(lo, hi, 2_000_000, 2 * 11604.5, 64.0, 0.5, seed=1)
    i.loadUniform(lo, hi, 2_000_000, 0.03 * 11604.5, 64.0, 0.5, seed=2)
    tol = 1e-7
    S = pic.PotentialSolver(W, 20000, tol, pic.SOLVER_LEARNED, stop=pic.STOP_REL_CHARGE)
    assert S.solve(raise_on_fail=True)
    S.computeEF()
    W.configure_loop(solve_each_step=True, sort_every=5)
    for _ in range(6):
        W.step()
    nr = S.norms()
    assert nr["charge"] < 1e-3 * nr["b"]  # the anode term dominates b
    assert nr["r"] <= tol * nr["charge"] * (1 + 1e-9)
    rho, phi = W.rho, W.phi
    # the oracle's converged potential for the same charge density, from the device's answer
    g = port.grid(nn, (0, 0, 0), L, periodic=(1, 1, 0))
    kind = port.node_kinds(g, 1)
    phi_o = phi.copy()
    ok, its, rel = port.solve_fpcg(g, kind, phi_o, rho, 1e-15, 20000)
    assert ok
    kz = np.arange(W.nv) // (nn[0] * nn[1])
    phi_vac = V * kz / (nn[2] - 1)
    scale = np.max(np.abs(phi_o - phi_vac))
    err = np.max(np.abs(phi - phi_o)) / scale
    print("space-charge potential: max %.3e V, device error %.3e of it, ||rho/eps0||/||b|| = %.3e"
          % (scale, err, nr["charge"] / nr["b"]))
    assert err <= 1e-6


def discharge_world(pic, warm):
    nn, L, V = (64, 64, 128), (0.02, 0.02, 0.04), 500.0
    W = pic.World(*nn, (0.0, 0.0, 0.0), L)
    W.set_boundaries((1, 1, 0), (1,) * 6, (0, 0, 0, 0, 0.0, V))
    W.setTime(2e-12, 1000)
    e = pic.Species("e-", pic.ME, -pic.QE, W, 32.0, capacity=1_100_000)
    i = pic.Species("O2+", 32 * pic.AMU, pic.QE, W, 32.0, capacity=1_100_000)
    lo, hi = (0.0, 0.0, 0.3 * L[2]), (L[0], L[1], 0.7 * L[2])
    e.loadUniform(lo, hi, 1_000_000, 2 * 11604.5, 32.0, 0.5, seed=3)
    i.loadUniform(lo, hi, 1_000_000, 0.03 * 11604.5, 32.0, 0.5, seed=4)
    S = pic.PotentialSolver(W, 20000, 1e-6, pic.SOLVER_LEARNED, stop=pic.STOP_REL_CHARGE)
    S.setWarmStart(warm)
    assert S.solve(raise_on_fail=True)
    S.computeEF()
    W.configure_loop(solve_each_step=True, sort_every=10)
    return W, S


def test_extrapolated_warm_start_cuts_iterations_and_keeps_the_answer(pic):
    """The same discharge twice, the Poisson solve of every step warm-started from the last
    potential or from its linear extrapolation in time; both end at the same certified residual,
    the extrapolated start needs fewer inner iterations."""
    out = {}
    for name, mode in (("previous", pic.WARM_PREVIOUS), ("extrapolate", pic.WARM_EXTRAPOLATE)):
        W, S = discharge_world(pic, mode)
        W.step()
        W.step()  # the first warm solve provides the change that the second extrapolates
        st0 = S.stats()
        for _ in range(10):
            W.step()
            nr = S.norms()
            assert nr["r"] <= 1e-6 * min(nr["b"], nr["charge"]) * (1 + 1e-9)
        st1 = S.stats()
        out[name] = (st1["inner"] - st0["inner"], W.phi, W.rho)
        W.close()
    print("inner iterations over 10 steps: previous %d, extrapolated %d" % (out["previous"][0], out["extrapolate"][0]))
    assert out["extrapolate"][0] <= 0.9 * out["previous"][0]
    # the two runs push in fields that agree within the tolerance: the potentials stay together
    pa, pb = out["previous"][1], out["extrapolate"][1]
    assert np.max(np.abs(pa - pb)) <= 1e-6 * np.max(np.abs(pa))
