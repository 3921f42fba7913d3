"""The conservation sums' per-thread accumulation, emulated exactly in FP32 on the CPU: a TwoSum of
each term into the running sum, with the rounding error and the exact error of the product w v
collected in a second word, then FP64 per-thread totals.  The totals agree with FP64 sums to about
1e-14 and do not depend on the particle order beyond that, which is what the loop tests' 1e-9
conservation checks rely on."""
import numpy as np

f32 = np.float32


def two_sum(a, b):
    s = (a + b).astype(f32)
    bb = (s - a).astype(f32)
    e = ((a - (s - bb).astype(f32)).astype(f32) + (b - bb).astype(f32)).astype(f32)
    return s, e


def two_prod(a, b):
    p = (a * b).astype(f32)
    # the FMA residual a*b - p: exact in FP64 for FP32 operands, then rounded once to FP32
    e = (a.astype(np.float64) * b.astype(np.float64) - p.astype(np.float64)).astype(f32)
    return p, e


def thread_sums(vel, w, threads):
    """k_sums: thread t takes particles t, t + threads, ...; returns the FP64 totals of
    w, w vx, w vy, w vz, w |v|^2 (|v|^2 rounded once in FP32)."""
    n = len(w)
    steps = (n + threads - 1) // threads
    pad = steps * threads - n
    vel = np.concatenate([vel, np.zeros((pad, 3), f32)]).reshape(steps, threads, 3)
    w = np.concatenate([w, np.zeros(pad, f32)]).reshape(steps, threads)
    hi = np.zeros((5, threads), f32)
    lo = np.zeros((5, threads), f32)
    for k in range(steps):
        v, ww = vel[k], w[k]
        terms = [(ww, np.zeros_like(ww))]
        for ax in range(3):
            terms.append(two_prod(ww, v[:, ax]))
        v2 = (v[:, 0] * v[:, 0]).astype(f32)
        v2 = (v[:, 1].astype(np.float64) * v[:, 1] + v2).astype(f32)  # fmaf: one rounding
        v2 = (v[:, 2].astype(np.float64) * v[:, 2] + v2).astype(f32)
        terms.append(two_prod(ww, v2))
        for c, (x, ex) in enumerate(terms):
            s, e = two_sum(hi[c], x)
            hi[c] = s
            lo[c] = (lo[c] + (e + ex).astype(f32)).astype(f32)
    return (hi.astype(np.float64) + lo.astype(np.float64)).sum(axis=1)


def test_compensated_sums_match_fp64_and_ignore_order():
    rng = np.random.default_rng(5)
    n = 200_000
    vel = (rng.normal(size=(n, 3)) * 3e5).astype(f32)
    w = rng.lognormal(np.log(64.0), 0.5, n).astype(f32)
    exact_w = np.sum(w.astype(np.float64))
    exact_p = np.sum(w.astype(np.float64)[:, None] * vel.astype(np.float64), axis=0)
    exact_k = np.sum(w.astype(np.float64) * np.sum(vel.astype(np.float64) ** 2, axis=1))
    a = thread_sums(vel, w, 4096)
    perm = rng.permutation(n)
    b = thread_sums(vel[perm], w[perm], 4096)
    scale_p = np.sum(w.astype(np.float64)[:, None] * np.abs(vel.astype(np.float64)), axis=0)
    for t in (a, b):
        assert abs(t[0] - exact_w) <= 1e-14 * exact_w
        assert np.all(np.abs(t[1:4] - exact_p) <= 1e-13 * scale_p)
        # |v|^2 is rounded once per particle (relative 6e-8, unbiased), so the kinetic sum is
        # within that of the FP64 one
        assert abs(t[4] - exact_k) <= 1e-7 * exact_k
    assert abs(a[0] - b[0]) <= 1e-14 * exact_w
    assert np.all(np.abs(a[1:4] - b[1:4]) <= 1e-13 * scale_p)
    assert abs(a[4] - b[4]) <= 1e-12 * exact_k
