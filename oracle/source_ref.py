"""CPU restatement of the beam sources -- TEST INFRASTRUCTURE ONLY.

Restates, in numpy FP64, ColdBeamSource / WarmBeamSource::sample (ch4/v3/src/Source.cpp:35-192)
in the GPU form the library implements (csrc/pic_particles.cu k_source, csrc/pic_capi.cu
pic_source_sample): the reference's MT19937 calls are replaced by Philox-4x32-10 streams keyed by
(seed, step, source, particle), so the library's particles can be checked one by one.  Nothing in
the library calls this file.

  count     (int)(den v_drift A dt / mpw0 + u)                       Source.cpp:27, 41
  position  the inlet face plane (the + faces one cell in: Source.cpp:55, 74, 93), the two other
            coordinates uniform over the face                          Source.cpp:42-98
  velocity  v_drift along the inward normal; a warm beam adds Species::sampleV3th(T)
            (speed from three per-axis sums of three uniforms with v_th = sqrt(2kT/m), isotropic
            direction from theta = 2 pi u, r = 2u - 1)                 Species.cpp:855-869
  adding    Species::addParticle: out-of-bounds positions are dropped and v -= q/m E dt/2
            (Species.cpp:420-434)
"""
import ctypes as C

import numpy as np

import oracle as O

TAG = 0x5C000000


def u01(x):
    return ((np.asarray(x, np.uint32) >> 9).astype(np.float32) + np.float32(0.5)) * np.float32(1.0 / 8388608.0)


def _block(port, p, step, src, b, key):
    return port.philox([p, step, TAG + src, b], key)


def sample(port, g, nn, x0, dx, face, v_drift, den, T, mass, charge, mpw0, dt, step, src, seed, ef=None):
    """Particles one source injects at a step: (pos [n,3], vel [n,3]) after addParticle, and n drawn."""
    key = [seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF]
    L = np.array([dx[d] * (nn[d] - 1) for d in range(3)], float)
    ax = face // 2
    A = np.prod(L) / L[ax]
    if face & 1:
        L[ax] -= dx[ax]
    ru = port.philox([0xFFFFFFFF, step, TAG + src, 7], key)
    n = int(den * v_drift * A * dt / mpw0 + float(u01(ru[0])))
    e1 = 1 if ax == 0 else 0
    e2 = 1 if ax == 2 else 2
    vth = np.sqrt(2 * O.KB * T / mass) if T > 0 else 0.0
    pos = np.zeros((n, 3))
    vel = np.zeros((n, 3))
    for p in range(n):
        r0 = _block(port, p, step, src, 0, key)
        x = np.zeros(3)
        x[ax] = x0[ax] + (L[ax] if face & 1 else 0.0)
        x[e1] = x0[e1] + float(u01(r0[0])) * L[e1]
        x[e2] = x0[e2] + float(u01(r0[1])) * L[e2]
        v = np.zeros(3)
        if vth > 0:
            r1 = _block(port, p, step, src, 1, key)
            r2 = _block(port, p, step, src, 2, key)
            r3 = _block(port, p, step, src, 3, key)
            f = [float(u01(q)) for q in (r0[2], r0[3], r1[0], r1[1], r1[2], r1[3], r2[0], r2[1], r2[2])]
            v1 = vth * (f[0] + f[1] + f[2] - 1.5)
            v2 = vth * (f[3] + f[4] + f[5] - 1.5)
            v3 = vth * (f[6] + f[7] + f[8] - 1.5)
            sp = np.sqrt(v1 * v1 + v2 * v2 + v3 * v3)
            th = 2 * np.pi * float(u01(r2[3]))
            r = -1.0 + 2.0 * float(u01(r3[0]))
            a = np.sqrt(max(1.0 - r * r, 0.0))
            v = np.array([sp * r, sp * np.cos(th) * a, sp * np.sin(th) * a])
        v[ax] += -v_drift if face & 1 else v_drift
        pos[p], vel[p] = x, v
    # Species::addParticle: bounds (World::inBounds, World.cpp:201-205) and the half-step rewind
    xm = np.array(x0) + np.array([dx[d] * (nn[d] - 1) for d in range(3)])
    keep = np.all((pos >= np.array(x0)) & (pos < xm), axis=1)
    pos, vel = pos[keep], vel[keep]
    if ef is not None:
        port.lib.or_gather3_ref.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        efc = np.ascontiguousarray(ef, np.float64)
        for q in range(len(pos)):
            lc = np.ascontiguousarray((pos[q] - np.array(x0)) / np.array(dx))
            e = np.zeros(3)
            port.lib.or_gather3_ref(C.byref(g), efc.ctypes.data, lc.ctypes.data, e.ctypes.data)
            vel[q] -= charge / mass * e * 0.5 * dt
    return pos, vel, n
