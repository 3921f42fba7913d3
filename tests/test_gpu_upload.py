"""Species::addParticle semantics are the same whichever memory the host arrays live in: pageable
arrays go through the staging buffer, pinned host and device arrays are read in place by the
conversion kernel."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_pinned_and_device_arrays_upload_like_pageable(pic):
    torch = pytest.importorskip("torch")
    nn, x0, xm = (17, 17, 17), (0.0, 0.0, 0.0), (0.01, 0.01, 0.01)
    rng = np.random.default_rng(3)
    n = 60000
    pos = rng.uniform(0, 0.01, (n, 3)) * 0.999999
    pos[::97] = 0.02  # out of bounds: dropped by the rewind path
    vel = rng.normal(size=(n, 3)) * 1e5
    w = rng.uniform(1.0, 2.0, n)
    ids = np.arange(n, dtype=np.uint64) * 7 + 3
    ef = rng.normal(size=(int(np.prod(nn)), 3)) * 1e3
    W = pic.World(*nn, x0, xm)
    W.setTime(1e-11, 10)
    W.ef = ef
    sps = [pic.Species("e%d" % k, pic.ME, -pic.QE, W, 1.5, capacity=2 * n) for k in range(3)]
    sps[0].addParticles(pos, vel, w, ids=ids, rewind=True)  # pageable
    t_pos, t_vel, t_w = (torch.from_numpy(a).pin_memory() for a in (pos, vel, w))
    t_ids = torch.from_numpy(ids.view(np.int64)).pin_memory()
    d_pos, d_vel, d_w, d_ids = (t.cuda() for t in (t_pos, t_vel, t_w, t_ids))
    torch.cuda.synchronize()
    for sp, arrs in ((sps[1], (t_pos, t_vel, t_w, t_ids)), (sps[2], (d_pos, d_vel, d_w, d_ids))):
        rc = W._L.pic_species_add_particles(W.handle, sp.id, *[C.c_void_p(a.data_ptr()) for a in arrs], n, 1)
        assert rc == 0
    ref = sps[0].getPartRef()
    ref = ref[np.argsort(ref["id"])]
    assert 0 < len(ref) < n  # the out-of-bounds particles are gone
    for sp in sps[1:]:
        p = sp.getPartRef()
        p = p[np.argsort(p["id"])]
        assert len(p) == len(ref)
        for f in ("id", "pos", "vel", "w"):
            assert np.array_equal(p[f], ref[f]), (sp.name, f)


def test_batch_upload_matches_species_by_species(pic):
    """pic_species_add_particles_batch (uploads on a side stream, each species sorted as soon as its
    upload is done) leaves the same particles and the same cell occupancy as one call per species
    followed by a sort, for pinned arrays (read in place) and pageable ones (one species at a time)."""
    torch = pytest.importorskip("torch")
    nn, x0, xm = (17, 17, 33), (0.0, 0.0, 0.0), (0.01, 0.01, 0.02)
    rng = np.random.default_rng(11)
    n = (50000, 30000)
    data = []
    for k in range(2):
        pos = rng.uniform(x0, xm, (n[k], 3)) * 0.999999
        pos[::101] = 0.05  # out of bounds: dropped by the rewind path
        data.append((pos, rng.normal(size=(n[k], 3)) * 1e5, rng.uniform(1.0, 2.0, n[k])))
    ef = rng.normal(size=(int(np.prod(nn)), 3)) * 1e3

    def world():
        W = pic.World(*nn, x0, xm)
        W.setTime(1e-11, 10)
        W.ef = ef
        sps = [pic.Species("s%d" % k, pic.ME * (1 + 40 * k), -pic.QE, W, 1.5, capacity=2 * n[k]) for k in range(2)]
        return W, sps

    W0, ref = world()
    for sp, (pos, vel, w) in zip(ref, data):
        sp.addParticles(pos, vel, w, rewind=True)
        sp.sortIndexes()
    W1, pinned = world()
    tensors = [[torch.from_numpy(a).pin_memory() for a in d] for d in data]
    torch.cuda.synchronize()
    W1.add_particles_batch(pinned, *[[t[j] for t in tensors] for j in range(3)])
    W2, pageable = world()
    W2.add_particles_batch(pageable, *[[d[j] for d in data] for j in range(3)])
    for k in range(2):
        r = ref[k].getPartRef()
        r = r[np.argsort(r["id"])]
        assert 0 < len(r) < n[k]
        counts = ref[k].sortIndexes(counts=True)
        for sp in (pinned[k], pageable[k]):
            p = sp.getPartRef()
            p = p[np.argsort(p["id"])]
            for f in ("id", "pos", "vel", "w"):
                assert np.array_equal(p[f], r[f]), (sp.name, f)
            assert np.array_equal(sp.sortIndexes(counts=True), counts)
    bad = W2.add_particles_batch
    with pytest.raises(RuntimeError):
        bad([pageable[0], pageable[0]], [data[0][0]] * 2, [data[0][1]] * 2, [data[0][2]] * 2)
