"""The GPU form of the object interaction (Philox streams, or_push_nonelectron_gpuform) against the
reference's own form (MT19937, or_push_nonelectron_ref, pinned bit-exactly by
tests/golden/objects.npz): both start from the same particles, so the same particles hit the
box; the bounces they draw must have the same distribution."""
import numpy as np

import oracle as O


def setup(n, seed):
    rng = np.random.default_rng(seed)
    c, half = 0.01, 0.004
    pos = rng.uniform(0, 0.02, (3 * n, 3)) * 0.999999
    pos = pos[~np.all(np.abs(pos - c) <= half, axis=1)][:n]
    vel = rng.normal(size=(n, 3)) * np.sqrt(O.KB * 3000.0 / (16 * O.AMU))
    p = np.zeros(n, O.PARTICLE)
    p["pos"], p["vel"], p["w"] = pos, vel, 1e9
    return p


def bounce_stats(p0, p, ids):
    """speeds of the particles whose velocity changed, and the fraction of them moving away from
    the box centre"""
    v0 = p0["vel"][ids]
    changed = np.any(p["vel"] != v0, axis=1)
    v = p["vel"][changed]
    r = p["pos"][changed] - 0.01
    return np.linalg.norm(v, axis=1), np.mean(np.sum(v * r, axis=1) > 0), int(changed.sum())


def test_gpu_form_bounces_match_reference_form(port):
    n = 40000
    g = port.grid((21, 21, 21), (0, 0, 0), (0.02, 0.02, 0.02), boxes=[((0.01,) * 3, (0.008,) * 3)])
    ef = np.zeros((21 ** 3, 3))
    m, dt = 16 * O.AMU, 2e-6
    p0 = setup(n, 1)
    speeds = {"ref": [], "gpu": []}
    away = {"ref": [], "gpu": []}
    counts = {"ref": [], "gpu": []}
    neu = np.zeros(10, O.PARTICLE)
    for k in range(6):
        # reference form: swap-with-last deletion, ids tracked through the weights' order
        p = p0.copy()
        p["w"] = np.arange(n) + 1.0  # the weight carries the index (neutrals never use it)
        nr, _, _ = port.push_nonelectron_ref(g, port.mt(100 + k), p, n, ef, dt, 0.0, m, neu, 0, 1e9)
        idx = (p["w"][:nr] - 1).astype(int)
        s, a, c = bounce_stats(p0, p[:nr], idx)
        speeds["ref"].append(s)
        away["ref"].append(a)
        counts["ref"].append((c, nr))
        # GPU form
        q = p0.copy()
        ids = np.arange(n, dtype=np.uint64)
        ng, _, _, st = port.push_nonelectron_gpuform(g, q, ids, n, ef, dt, 0.0, m, neu, np.zeros(10, np.uint64), 0,
                                                     1e9, neu, np.zeros(10, np.uint64), 0, 1.0, False, 500 + k, 1)
        s, a, c = bounce_stats(p0, q[:ng], ids[:ng].astype(int))
        speeds["gpu"].append(s)
        away["gpu"].append(a)
        counts["gpu"].append((c, ng))
        assert st[0] > 1000 and st[1] >= st[0]
    for key in ("ref", "gpu"):
        speeds[key] = np.concatenate(speeds[key])
    sr, sg = speeds["ref"], speeds["gpu"]
    # full accommodation at 300 K: sampleVth(300) speeds, the same in both forms
    se = np.sqrt(sr.var() / len(sr) + sg.var() / len(sg))
    assert abs(sr.mean() - sg.mean()) <= 4 * se
    assert abs(sr.std() / sg.std() - 1) <= 0.03
    # (the reference's tangent t1 = n x (1,0,0) if n_x != 0 else n x (0,1,0) vanishes on the x and
    # y faces, so those bounces leave along the normal with v_th cos(theta): both forms keep that)
    # survivors and bounced counts agree (the same particles hit the box in both forms)
    cr, cg = np.array(counts["ref"]), np.array(counts["gpu"])
    assert np.all(np.abs(cr[:, 0] - cg[:, 0]) <= 0.05 * cr[:, 0] + 20)
    assert np.all(np.abs(cr[:, 1] - cg[:, 1]) <= 0.01 * n)
    assert min(away["ref"]) > 0.9 and min(away["gpu"]) > 0.9
