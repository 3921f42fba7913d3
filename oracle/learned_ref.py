"""CPU reference of the learned Poisson preconditioner -- TEST INFRASTRUCTURE ONLY.

Restates, in numpy FP64, the preconditioner the CUDA library applies and trains
(csrc/pic_learned.cu), so the device apply, forward pass and gradients can be checked element by
element.  Nothing in the library calls this file.

The preconditioner is additive multilevel with a small linear convolutional network per level:

    B r = mask * sum_l P^l o_l,   z_0 = mask * r,   z_{l+1} = R z_l,   R = P^T
    o_0     = S_0 * z_0                                    (3x3x3 stencil, level 0)
    o_l     = N_l(z_l)                for l = 1 .. 4       (network level, channels 16/32/64/64)
    o_l     = z_l / diag_l            for l >= 5           (fixed diagonal scaling)
    N_l(z)[v] = sum_t sum_c Wp[t, c] h2[v + o_t, c],  h2 = h1 Wm^T,
    h1[v, c]  = sum_t Wl[c, t] z[v + o_t]                  (3x3x3 lift 1 -> C, mix C -> C, 3x3x3 proj C -> 1)

P is cell-centred trilinear prolongation (per axis: fine 2c <- 3/4 a[c] + 1/4 a[c-1],
fine 2c+1 <- 3/4 a[c] + 1/4 a[c+1]), R its exact transpose.  Level sizes halve rounding up;
periodic axes wrap at every level, other axes read zero outside the level box (also the
network's intermediate h2).  With weights at their initial values (S_0, N_l the identity
scaled by 1/diag_l, diag_l the interior diagonal of the Galerkin operator P^l^T A P^l) this is
the BPX preconditioner.  Training minimises |A B r - r|^2 / |r|^2 over residual samples r.
Arrays are [z, y, x] (x fastest) over the distinct nodes of each axis; channels last.
"""
import numpy as np

CHANNELS = (16, 32, 64, 64)  # network levels 1 .. 4
NET_LEVELS = len(CHANNELS)
TAPS = [(dz, dy, dx) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]  # t = 9(dz+1)+3(dy+1)+(dx+1)
MAX_LEVELS = 12


def level_shapes(shape0):
    """Level l+1 halves every axis of level l (rounding up) while all axes stay >= 2."""
    shapes = [tuple(shape0)]
    while len(shapes) < MAX_LEVELS:
        nxt = tuple((s + 1) // 2 for s in shapes[-1])
        if min(nxt) < 2 or nxt == shapes[-1]:
            break
        shapes.append(nxt)
    return shapes


def shift(a, d, per):
    """b[v] = a[v + d]: zero outside the box, or wrapped on periodic axes; d and per are (z, y, x)."""
    out = a
    for ax, (dd, p) in enumerate(zip(d, per)):
        if dd == 0:
            continue
        out = np.roll(out, -dd, axis=ax)
        if not p:
            sl = [slice(None)] * out.ndim
            sl[ax] = slice(-dd, None) if dd > 0 else slice(0, -dd)
            out[tuple(sl)] = 0
    return out


def _up1(a, ax, nf, per):
    a = np.moveaxis(a, ax, 0)
    if per:
        am, ap = np.roll(a, 1, 0), np.roll(a, -1, 0)
    else:
        z = np.zeros_like(a[:1])
        am, ap = np.concatenate([z, a[:-1]]), np.concatenate([a[1:], z])
    f = np.empty((2 * a.shape[0],) + a.shape[1:])
    f[0::2] = 0.75 * a + 0.25 * am
    f[1::2] = 0.75 * a + 0.25 * ap
    return np.moveaxis(f[:nf], 0, ax)


def _dn1(f, ax, per):
    f = np.moveaxis(f, ax, 0)
    nf = f.shape[0]
    nc = (nf + 1) // 2
    g = np.zeros((2 * nc,) + f.shape[1:])
    g[:nf] = f
    ev, od = g[0::2], g[1::2]
    c = 0.75 * (ev + od)
    if per:
        c += 0.25 * (np.roll(ev, -1, 0) + np.roll(od, 1, 0))
    else:
        c[:-1] += 0.25 * ev[1:]
        c[1:] += 0.25 * od[:-1]
    return np.moveaxis(c, 0, ax)


def prolong(a, fine_shape, per):
    for ax in range(3):
        a = _up1(a, ax, fine_shape[ax], per[ax])
    return a


def restrict(f, per):
    for ax in range(3):
        f = _dn1(f, ax, per[ax])
    return f


def galerkin_factors(levels):
    """1-D interior diagonals of P^l^T T P^l (T = tridiag(-1, 2, -1)) and of P^l^T P^l."""
    n = 2 ** (levels + 3)
    t, m = [], []
    for l in range(levels):
        nc = n >> l
        a = np.zeros(nc)
        a[nc // 2] = 1.0
        f = a
        for k in range(l):
            f = _up1(f[:, None, None], 0, 2 * f.shape[0], False)[:, 0, 0]
        tf = 2 * f - np.concatenate([[0.0], f[:-1]]) - np.concatenate([f[1:], [0.0]])
        mf = f.copy()
        for k in range(l):
            tf = _dn1(tf[:, None, None], 0, False)[:, 0, 0]
            mf = _dn1(mf[:, None, None], 0, False)[:, 0, 0]
        t.append(tf[nc // 2])
        m.append(mf[nc // 2])
    return np.array(t), np.array(m)


def level_diags(c, nlev):
    """Interior diagonal of the Galerkin operator at each level for coefficients c = (cx, cy, cz)."""
    t, m = galerkin_factors(nlev)
    return (c[0] + c[1] + c[2]) * t * m * m


def init_weights(diags, channels=CHANNELS):
    W = {"S0": np.zeros(27), "net": []}
    W["S0"][13] = 1.0 / diags[0]
    for l, C in enumerate(channels, start=1):
        d = diags[l] if l < len(diags) else 1.0
        Wl = np.zeros((C, 27))
        Wl[0, 13] = 1.0
        Wp = np.zeros((27, C))
        Wp[13, 0] = 1.0 / d
        W["net"].append({"Wl": Wl, "Wm": np.eye(C), "Wp": Wp})
    return W


def symmetrize(W, diags):
    """The projection the trainer applies after every optimiser step (csrc/pic_learned.cu
    k_lp_symmetrize): S0 even, each network level's projection the adjoint of its lift scaled by
    1 / diag_l, its mix symmetric; every tied pair replaced by its mean.  B is then symmetric."""
    W["S0"][:] = 0.5 * (W["S0"] + W["S0"][::-1])
    for l, w in enumerate(W["net"], start=1):
        sc = 1.0 / diags[l] if l < len(diags) else 1.0
        a = 0.5 * (w["Wl"] + w["Wp"][::-1].T / sc)
        w["Wl"][:] = a
        w["Wp"][:] = sc * a[:, ::-1].T
        w["Wm"][:] = 0.5 * (w["Wm"] + w["Wm"].T)
    return W


def stencil27(z, S, per):
    out = np.zeros_like(z)
    for t, d in enumerate(TAPS):
        out += S[t] * shift(z, d, per)
    return out


def net_forward(z, w, per):
    h1 = np.zeros(z.shape + (w["Wl"].shape[0],))
    for t, d in enumerate(TAPS):
        h1 += shift(z, d, per)[..., None] * w["Wl"][:, t]
    h2 = h1 @ w["Wm"].T
    o = np.zeros(z.shape)
    for t, d in enumerate(TAPS):
        o += shift(h2, d, per) @ w["Wp"][t]
    return o, (h1, h2)


def apply(r, mask, W, per, diags, keep=False):
    """B r over the level-0 box [z, y, x]; per = periodic flags (z, y, x)."""
    shapes = level_shapes(r.shape)
    zs = [mask * r]
    for l in range(1, len(shapes)):
        zs.append(restrict(zs[-1], per))
    outs, caches = [], []
    for l, z in enumerate(zs):
        if l == 0:
            o = stencil27(z, W["S0"], per)
            cache = None
        elif l <= NET_LEVELS:
            o, cache = net_forward(z, W["net"][l - 1], per)
        else:
            o = z / diags[l]
            cache = None
        outs.append(o)
        caches.append(cache)
    e = outs[-1]
    for l in range(len(zs) - 2, -1, -1):
        e = outs[l] + prolong(e, shapes[l], per)
    e = mask * e
    if keep:
        return e, (zs, caches)
    return e


def apply_L(e, mask, c, per):
    """(L e)_p = sum_axes c ((e_p - e_-) + (e_p - e_+)) on masked nodes (e read as zero off the mask)."""
    e = mask * e
    out = np.zeros_like(e)
    for ax, cc in zip((2, 1, 0), c):  # x, y, z coefficients
        dp = [0, 0, 0]
        dp[ax] = 1
        dm = [0, 0, 0]
        dm[ax] = -1
        out += cc * (2 * e - shift(e, tuple(dp), per) - shift(e, tuple(dm), per))
    return mask * out


def backward(r, mask, W, per, diags, ge):
    """Gradients of sum(ge * B r) with respect to every weight (ge: the loss gradient at e = B r)."""
    shapes = level_shapes(r.shape)
    _, (zs, caches) = apply(r, mask, W, per, diags, keep=True)
    gs = [mask * ge]
    for l in range(1, len(shapes)):
        gs.append(restrict(gs[-1], per))
    G = {"S0": np.array([np.sum(gs[0] * shift(zs[0], d, per)) for d in TAPS]), "net": []}
    for l in range(1, min(NET_LEVELS, len(shapes) - 1) + 1):
        w = W["net"][l - 1]
        z, (h1, h2), g = zs[l], caches[l], gs[l]
        dWp = np.zeros_like(w["Wp"])
        dh2 = np.zeros_like(h2)
        for t, d in enumerate(TAPS):
            dWp[t] = np.tensordot(g, shift(h2, d, per), axes=([0, 1, 2], [0, 1, 2]))
            dh2 += shift(g, tuple(-x for x in d), per)[..., None] * w["Wp"][t]
        dWm = np.tensordot(dh2, h1, axes=([0, 1, 2], [0, 1, 2]))
        dh1 = dh2 @ w["Wm"]
        dWl = np.zeros_like(w["Wl"])
        for t, d in enumerate(TAPS):
            dWl[:, t] = np.tensordot(dh1, shift(z, d, per), axes=([0, 1, 2], [0, 1, 2]))
        G["net"].append({"Wl": dWl, "Wm": dWm, "Wp": dWp})
    return G


def loss_and_grads(r, x, mask, W, c, per, diags, scale_free=True):
    """Loss of one pair (r, x) with L x = r, and its gradients with respect to every weight.

    scale_free: the squared sine of the energy-norm angle between e = B r and x,
        1 - <e, x>_L^2 / (<e, e>_L <x, x>_L)   (CG does not see the scale of B);
    otherwise the energy-norm error (e - x)^T L (e - x) / x^T L x."""
    e = apply(r, mask, W, per, diags)
    x = mask * x
    lx = apply_L(x, mask, c, per)
    le = apply_L(e, mask, c, per)
    q = np.sum(x * lx)
    if scale_free:
        a = np.sum(e * lx)
        p = np.sum(e * le)
        loss = 1.0 - a * a / (p * q)
        ge = (2.0 * a / (p * q)) * ((a / p) * le - lx)
    else:
        lerr = le - lx
        loss = np.sum((e - x) * lerr) / q
        ge = 2.0 * lerr / q
    return loss, backward(r, mask, W, per, diags, ge)


def fpcg(b, mask, c, per, precond, tol=1e-6, maxit=5000):
    """Flexible CG (beta = z_new.(r_new - r_old) / z_old.r_old) on L x = b; returns (x, iterations)."""
    x = np.zeros_like(b)
    r = mask * b
    z = precond(r)
    p = z.copy()
    rz = np.vdot(r, z)
    nb = np.linalg.norm(r)
    for it in range(1, maxit + 1):
        q = apply_L(p, mask, c, per)
        alpha = rz / np.vdot(p, q)
        x += alpha * p
        r_new = r - alpha * q
        if np.linalg.norm(r_new) <= tol * nb:
            return x, it
        z = precond(r_new)
        beta = np.vdot(z, r_new - r) / rz
        rz = np.vdot(r_new, z)
        r = r_new
        p = z + beta * p
    return x, maxit
