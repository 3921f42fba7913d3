"""Beam sources (ColdBeamSource / WarmBeamSource, ch4/v3/src/Source.cpp) against the oracle's
restatement on the same Philox streams, plus their injection statistics."""
import numpy as np
import pytest

import oracle as O
import source_ref

pytestmark = pytest.mark.gpu


def smooth_field(nn, amp, seed):
    rng = np.random.default_rng(seed)
    k, j, i = np.meshgrid(np.arange(nn[2]), np.arange(nn[1]), np.arange(nn[0]), indexing="ij")
    ef = np.zeros((int(np.prod(nn)), 3))
    for d in range(3):
        a = rng.uniform(0.5, 1.5, 3)
        ef[:, d] = (amp * np.sin(a[0] * i * 0.3 + d) * np.cos(a[1] * j * 0.25) * np.sin(a[2] * k * 0.2 + 1)).ravel()
    return ef


@pytest.mark.parametrize("face,T", [(4, 0.0), (5, 0.0), (0, 2.0 * 11604.5), (3, 1.0 * 11604.5)])
def test_source_particles_match_oracle(pic, port, face, T):
    nn, x0, xm = (9, 11, 13), (0.0, -0.001, 0.002), (0.008, 0.009, 0.014)
    dx = [(xm[d] - x0[d]) / (nn[d] - 1) for d in range(3)]
    g = port.grid(nn, x0, xm)
    dt = 1e-11
    W = pic.World(*nn, x0, xm)
    W.set_boundaries((0, 0, 0), (0,) * 6, (5.0,) * 6)
    W.setTime(dt, 100)
    ef = smooth_field(nn, 2e3, 3)
    W.ef = ef
    s = pic.Species("e-", pic.ME, -pic.QE, W, 1e4, capacity=20000)
    v_drift, den, seed = 3e5, 1e16, 0x1234_5678_9A
    cls = pic.WarmBeamSource if T > 0 else pic.ColdBeamSource
    args = (s, W, v_drift, den, T) if T > 0 else (s, W, v_drift, den)
    src = cls(*args, inlet_face=["x-", "x+", "y-", "y+", "z-", "z+"][face], seed=seed)
    # World::addInlet: the inlet face is Dirichlet at 0 V
    ntype = W.node_type.reshape(nn[2], nn[1], nn[0])
    phi = W.phi.reshape(nn[2], nn[1], nn[0])
    sl = [slice(None)] * 3
    sl[2 - face // 2] = -1 if face & 1 else 0
    assert np.all(ntype[tuple(sl)] == 2) and np.all(phi[tuple(sl)] == 0.0)
    total = 0
    for step in range(3):
        W.advanceTime()
        n0 = s.getNumParticles()
        src.sample()
        p = s.getPartRef()
        new = p[p["id"] >= total]
        new = new[np.argsort(new["id"])]
        pos, vel, n = source_ref.sample(port, g, nn, x0, dx, face, v_drift, den, T, O.ME, -O.QE, 1e4, dt, W.getTs(),
                                        src.id, seed, ef=ef)
        assert n > 50
        total += n
        assert len(new) == len(pos) == s.getNumParticles() - n0
        assert np.max(np.abs(new["pos"] - pos)) <= 1e-6 * min(dx)
        assert np.all(np.abs(new["vel"] - vel) <= 1e-6 * np.abs(vel) + 1e-3 * v_drift * 1e-3)
        assert np.all(new["w"] == 1e4)


def test_source_injection_statistics(pic):
    nn, x0, xm = (17, 17, 17), (0.0, 0.0, 0.0), (0.01, 0.01, 0.01)
    W = pic.World(*nn, x0, xm)
    W.set_boundaries((1, 1, 0), (1,) * 6, (0.0,) * 6)
    dt = 1e-11
    W.setTime(dt, 1000)
    mpw0 = 1e3
    s = pic.Species("O+", 16 * pic.AMU, pic.QE, W, mpw0, capacity=2_000_000)
    T = 0.5 * 11604.5
    v_drift, den = 2e4, 5.17e15
    src = pic.WarmBeamSource(s, W, v_drift, den, T, inlet_face="-z", seed=5)
    expect = den * v_drift * 0.01 * 0.01 * dt / mpw0  # n v A dt / mpw0, not an integer
    counts = []
    for _ in range(200):
        W.advanceTime()
        n0 = s.getNumParticles()
        src.sample()
        counts.append(s.getNumParticles() - n0)
    counts = np.array(counts)
    # (int)(x + u) is an unbiased rounding: mean x, each count floor(x) or floor(x) + 1
    assert set(np.unique(counts)) <= {int(expect), int(expect) + 1}
    assert abs(counts.mean() - expect) <= 4 * 0.5 / np.sqrt(len(counts))
    p = s.getPartRef()
    v = p["vel"]
    # drift along +z; Species::sampleV3th: isotropic, E[v^2] = 3 Var(u1+u2+u3) v_th^2 = 0.75 v_th^2
    vth2 = 2 * pic.KB * T / (16 * pic.AMU)
    n = len(v)
    assert abs(v[:, 2].mean() - v_drift) <= 5 * np.sqrt(0.25 * vth2 / n)
    assert abs(v[:, 0].mean()) <= 5 * np.sqrt(0.25 * vth2 / n)
    v2 = ((v - np.array([0, 0, v_drift])) ** 2).sum(1)
    assert abs(v2.mean() / (0.75 * vth2) - 1.0) <= 0.03
    # positions on the inlet plane z = 0, spread over the face
    assert np.all(p["pos"][:, 2] >= 0) and p["pos"][:, 2].max() < 0.01 / 16 * 5
    assert p["pos"][:, 0].std() > 0.0025
