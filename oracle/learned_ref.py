"""CPU reference of the learned Poisson preconditioner -- TEST INFRASTRUCTURE ONLY.

Restates, in numpy FP64, the network the CUDA library applies and trains (csrc/pic_learned.cu),
so the device forward pass and the device gradients can be checked element by element.

Network (linear, four levels l = 0..3, channels C_l = 16, 32, 64, 64):
    z_0 = r / rms(r);  z_{l+1} = 2x2x2 block sum of z_l
    h1_l[v, c] = sum_t Wl_l[c, t] z_l[v + o_t]                 (3x3x3 lift, 1 -> C_l)
    h2_l[v, c] = sum_c' Wm_l[c, c'] h1_l[v, c']                 (channel mix, C_l -> C_l)
    o_l[v]     = sum_t sum_c Wp_l[t, c] h2_l[v + o_t, c]        (3x3x3 projection, C_l -> 1)
    e_3 = o_3;  e_l = o_l + nearest-neighbour upsampling of e_{l+1};  e = mask * e_0 * rms(r)
Neighbours outside the grid read zero, except along periodic axes, which wrap.
Training loss for a residual r:  |L e - r|^2 / |r|^2 with L the (masked) 7-point operator.
Arrays are indexed [z, y, x] (x fastest), channels last.
"""
import numpy as np

CHANNELS = (16, 32, 64, 64)
TAPS = [(dz, dy, dx) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]  # t = 9(dz+1)+3(dy+1)+(dx+1)


def shift(a, d, periodic):
    """b[v] = a[v + d] with zero fill (or wrap on periodic axes), d = (dz, dy, dx)."""
    out = a
    for ax, (dd, per) in enumerate(zip(d, periodic)):
        if dd == 0:
            continue
        out = np.roll(out, -dd, axis=ax)
        if not per:
            sl = [slice(None)] * out.ndim
            sl[ax] = slice(-dd, None) if dd > 0 else slice(0, -dd)
            out[tuple(sl)] = 0
    return out


def block_sum(a):
    nz, ny, nx = a.shape[:3]
    return a.reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2, *a.shape[3:]).sum(axis=(1, 3, 5))


def upsample(a):
    return a.repeat(2, axis=0).repeat(2, axis=1).repeat(2, axis=2)


def init_weights(c_diag, levels=4, channels=CHANNELS):
    """Weights making the network a multilevel diagonal-scaling (BPX-like) preconditioner."""
    W = []
    for l in range(levels):
        C = channels[l]
        Wl = np.zeros((C, 27))
        Wl[0, 13] = 1.0
        Wm = np.eye(C)
        Wp = np.zeros((27, C))
        Wp[13, 0] = 1.0 / (c_diag * 2.0 ** l)
        W.append({"Wl": Wl, "Wm": Wm, "Wp": Wp})
    return W


def forward(r, mask, W, periodic=(0, 0, 0), keep=False):
    rms = np.sqrt(np.mean(r ** 2)) or 1.0
    z = [r / rms]
    for l in range(1, len(W)):
        z.append(block_sum(z[-1]))
    per = periodic[::-1]  # arrays are [z, y, x]
    cache = []
    o = []
    for l, w in enumerate(W):
        zl = z[l]
        h1 = np.zeros(zl.shape + (w["Wl"].shape[0],))
        for t, d in enumerate(TAPS):
            h1 += shift(zl, d, per)[..., None] * w["Wl"][:, t]
        h2 = h1 @ w["Wm"].T
        ol = np.zeros(zl.shape)
        for t, d in enumerate(TAPS):
            ol += shift(h2, d, per) @ w["Wp"][t]
        cache.append((zl, h1, h2))
        o.append(ol)
    e = o[-1]
    for l in range(len(W) - 2, -1, -1):
        e = o[l] + upsample(e)
    e = mask * e
    if keep:
        return e * rms, (z, cache, rms)
    return e * rms


def apply_L(e, mask, c, periodic=(0, 0, 0)):
    """(L e)_p = sum_axes c ((e_p - e_-) + (e_p - e_+)) on masked nodes, zero elsewhere."""
    per = periodic[::-1]
    out = np.zeros_like(e)
    for ax, cc in zip((2, 1, 0), c):  # x, y, z coefficients
        d = [0, 0, 0]
        d[ax] = 1
        dm = [0, 0, 0]
        dm[ax] = -1
        out += cc * (2 * e - shift(e, tuple(d), per) - shift(e, tuple(dm), per))
    return mask * out


def loss_and_grads(r, mask, W, c, periodic=(0, 0, 0)):
    """Loss |L e - r|^2/|r|^2 on the normalised residual and its gradients wrt all weights."""
    rms = np.sqrt(np.mean(r ** 2)) or 1.0
    e, (z, cache, _) = forward(r, mask, W, periodic, keep=True)
    en = e / rms
    rn = r / rms
    res = apply_L(en, mask, c, periodic) - rn * mask
    denom = np.sum((rn * mask) ** 2)
    loss = np.sum(res ** 2) / denom
    ge = mask * apply_L(2.0 * res / denom, mask, c, periodic)
    per = periodic[::-1]
    grads = []
    g = [ge]
    for l in range(1, len(W)):
        g.append(block_sum(g[-1]))
    for l, w in enumerate(W):
        zl, h1, h2 = cache[l]
        dO = g[l]
        dWp = np.zeros_like(w["Wp"])
        dh2 = np.zeros_like(h2)
        for t, d in enumerate(TAPS):
            sh2 = shift(h2, d, per)
            dWp[t] = np.tensordot(dO, sh2, axes=([0, 1, 2], [0, 1, 2]))
            dh2 += shift(dO, tuple(-x for x in d), per)[..., None] * w["Wp"][t]
        dWm = np.tensordot(dh2, h1, axes=([0, 1, 2], [0, 1, 2]))
        dh1 = dh2 @ w["Wm"]
        dWl = np.zeros_like(w["Wl"])
        for t, d in enumerate(TAPS):
            dWl[:, t] = np.tensordot(dh1, shift(zl, d, per), axes=([0, 1, 2], [0, 1, 2]))
        grads.append({"Wl": dWl, "Wm": dWm, "Wp": dWp})
    return loss, grads
