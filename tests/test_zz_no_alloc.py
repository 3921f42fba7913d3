"""pic_number_density_noalloc: the number density for callers that cannot allocate device memory.

Those callers (plugins whose host application owns all device memory through its own
allocator, real-time loops that forbid allocation after start-up) pass particle arrays and the
output field they already hold; the entry point works in a library-owned device array instead
of allocating.
It is checked through the C ABI against the existing path (pic_species_number_density +
pic_charge_density) on two calls in a row, within the deposit tolerance of the other tests.
This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NN, X0, XM, PER = (33, 29, 41), (0.0, -0.01, 0.0), (0.016, 0.004, 0.02), (1, 1, 0)


def library_layout(pos, w, torch):
    """Particles in the library's device layout: float4 {offsets, packed cell}, float4 {v, w}."""
    x0, xm, nn = np.array(X0), np.array(XM), np.array(NN)
    dx = (xm - x0) / (nn - 1)
    lc = (pos - x0) / dx
    c = np.minimum(np.maximum(lc.astype(np.int64), 0), nn - 2)
    off = np.minimum((lc - c).astype(np.float32), np.float32(np.nextafter(np.float32(1), np.float32(0))))
    cell = (c[:, 0] | (c[:, 1] << 9) | (c[:, 2] << 18)).astype(np.int32)
    p4 = np.zeros((len(w), 4), np.float32)
    p4[:, :3] = off
    p4[:, 3] = cell.view(np.float32)
    v4 = np.zeros((len(w), 4), np.float32)
    v4[:, 3] = w
    return torch.from_numpy(p4).cuda(), torch.from_numpy(v4).cuda()


def test_noalloc_density_matches_existing_entry_point(pic):
    torch = pytest.importorskip("torch")
    L = pic.library()
    rng = np.random.default_rng(21)
    W = pic.World(*NN, X0, XM)
    W.set_boundaries(PER, (1,) * 6, (0.0,) * 6)
    nv = int(np.prod(NN))
    x0, xm = np.array(X0, np.float64), np.array(XM, np.float64)
    per = np.array(PER, np.int32)
    out = torch.zeros(nv, dtype=torch.float32, device="cuda")
    for call, n in enumerate((250000, 97000)):
        pos = rng.uniform(X0, XM, (n, 3)) * 0.999999 + np.array(X0) * 0.000001
        w = rng.lognormal(np.log(64) - 0.125, 0.5, n).astype(np.float32).astype(np.float64)
        # existing entry point: a species in the world
        s = pic.Species("s%d" % call, pic.ME, -pic.QE, W, 64.0, capacity=n)
        s.addParticles(pos, np.zeros((n, 3)), w, rewind=False)
        s.computeNumberDensity()
        W.computeChargeDensity()
        ref = s.den
        # the no-allocation entry point on the same particles
        p4, v4 = library_layout(pos, w, torch)
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        rc = L.pic_number_density_noalloc(NN[0], NN[1], NN[2], x0.ctypes.data_as(C.c_void_p),
                                          xm.ctypes.data_as(C.c_void_p), per.ctypes.data_as(C.c_void_p),
                                          C.c_void_p(p4.data_ptr()), C.c_void_p(v4.data_ptr()), n, 2.0 ** 30,
                                          C.c_void_p(out.data_ptr()), None)
        assert rc == pic.PIC_OK
        torch.cuda.synchronize()
        if call > 0:  # the first call on a device may load the library's module (its device array)
            assert torch.cuda.mem_get_info()[0] == free0, "device memory changed during the call"
        got = out.cpu().numpy().astype(np.float64)
        assert np.max(np.abs(got - ref)) <= 1e-6 * np.max(ref), call


def test_noalloc_rejects_grids_beyond_its_accumulator(pic):
    L = pic.library()
    x0 = np.zeros(3)
    xm = np.ones(3)
    rc = L.pic_number_density_noalloc(129, 129, 129, x0.ctypes.data_as(C.c_void_p), xm.ctypes.data_as(C.c_void_p),
                                      None, None, None, 0, 1.0, C.c_void_p(1), None)
    assert rc == pic.PIC_ERR_ARG
    buf = C.create_string_buffer(256)
    L.pic_last_error(buf, 256)
    assert b"exceed" in buf.value


@pytest.mark.parametrize("nn,per", [((514, 4, 4), None), ((4, 514, 4), None), ((3, 8, 8), (1, 0, 0))])
def test_noalloc_rejects_grids_the_world_rejects(pic, nn, per):
    """A 513-cell axis does not fit the packed particle cell, and a periodic axis needs 4 nodes."""
    L = pic.library()
    x0 = np.zeros(3)
    xm = np.ones(3)
    p = np.array(per, np.int32) if per else None
    rc = L.pic_number_density_noalloc(nn[0], nn[1], nn[2], x0.ctypes.data_as(C.c_void_p),
                                      xm.ctypes.data_as(C.c_void_p),
                                      p.ctypes.data_as(C.c_void_p) if p is not None else None, None, None, 0, 1.0,
                                      C.c_void_p(1), None)
    assert rc == pic.PIC_ERR_ARG
