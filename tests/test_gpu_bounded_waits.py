"""Bounded device waits: a wait that runs out is reported to the host and leaves the world usable.

Every mbarrier wait in the library's kernels polls a bounded number of times; when the limit
runs out the kernel records the fault in the world's error word, waits (with the full limit) for
the copies or tensor-core MMAs it still has in flight, frees its TMEM and returns.  The test hook
pic_debug_set_wait_polls(w, 0) makes the first wait give up at once, without a poll: nothing
faults, traps or hangs, and the drain keeps its full limit.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def last_error(L):
    buf = C.create_string_buffer(512)
    L.pic_last_error(buf, 512)
    return buf.value.decode()


def test_push_wait_that_runs_out_is_reported_and_world_stays_usable(pic, port):
    nn, x0, xm = (33, 17, 25), (0.0, 0.0, 0.0), (0.032, 0.016, 0.024)
    g = port.grid(nn, x0, xm)
    nv = int(np.prod(nn))
    rng = np.random.default_rng(4)
    n = 40_000  # many 1 024-particle chunks: the push stages them with bulk copies
    p = np.zeros(n, O.PARTICLE)
    p["pos"] = rng.uniform(0, 1, (n, 3)) * np.array(xm) * 0.999999
    p["vel"] = rng.normal(size=(n, 3)) * 2e5
    p["w"] = 7.0
    ef = rng.normal(size=(nv, 3)) * 1e3
    dt = 1e-11
    W = pic.World(*nn, x0, xm)
    W.dirichletBoundries(0.0)
    W.setTime(dt, 10)
    W.ef = ef
    e = pic.Species("e-", pic.ME, -pic.QE, W, 7.0, capacity=n + 64)
    ids = np.arange(n, dtype=np.uint64)
    e.addParticles(p["pos"], p["vel"], p["w"], ids=ids, rewind=False)
    e.sortIndexes()
    before = e.getPartRef()
    L = W._L
    assert L.pic_debug_set_wait_polls(W._h, 0) == pic.PIC_OK
    try:
        assert L.pic_species_push(W._h, e.id, dt, 1) == pic.PIC_OK  # queued; the fault shows at the sync
        assert L.pic_synchronize(W._h) == pic.PIC_ERR_DEVICE
        assert "bounded wait" in last_error(L)
        # every block gave up before it touched a particle
        after = e.getPartRef()
        assert np.array_equal(after["id"], before["id"])
        assert np.array_equal(after["pos"], before["pos"]) and np.array_equal(after["vel"], before["vel"])
    finally:
        assert L.pic_debug_set_wait_polls(W._h, -1) == pic.PIC_OK
    assert L.pic_synchronize(W._h) == pic.PIC_OK  # the error word was cleared when it was read
    # the world still works: one push + deposit against the oracle
    e.advance(dt, deposit=True)
    W.computeChargeDensity()
    po, oid = p.copy(), ids.copy()
    m = port.push(g, po, ef, dt, -O.QE, O.ME, ids=oid)
    gp = e.getPartRef()
    assert len(gp) == m
    a, b = np.argsort(gp["id"]), np.argsort(oid[:m])
    dx = (np.array(xm) - np.array(x0)) / (np.array(nn) - 1)
    assert np.max(np.abs(gp["pos"][a] - po[:m]["pos"][b])) <= 1e-5 * dx.min()
    den = port.number_density(g, po[:m])
    assert np.max(np.abs(e.den - den)) <= 1e-6 * np.max(den)


def test_tensor_core_wait_that_runs_out_is_reported_and_training_recovers(pic):
    n = 33
    W = pic.World(n, n, n, (0.0, 0.0, 0.0), (0.032, 0.032, 0.032))
    W.set_boundaries((1, 1, 0), (1,) * 6, (0.0,) * 6)
    lp = pic.LearnedPreconditioner(W)
    rng = np.random.default_rng(9)
    nv = n ** 3
    x = rng.normal(size=nv)
    r = rng.normal(size=nv)
    loss0, g0 = lp.loss_grad(r, x)
    L = W._L
    assert L.pic_debug_set_wait_polls(W._h, 0) == pic.PIC_OK
    try:
        with pytest.raises(pic.PicError) as ei:
            lp.loss_grad(r, x)
        assert ei.value.code == pic.PIC_ERR_DEVICE
        assert "tensor-core wait" in last_error(L)
    finally:
        assert L.pic_debug_set_wait_polls(W._h, -1) == pic.PIC_OK
    loss1, g1 = lp.loss_grad(r, x)
    assert abs(loss1 - loss0) <= 1e-9 * abs(loss0)
    assert np.allclose(g1, g0, rtol=1e-5, atol=1e-7 * np.abs(g0).max())
