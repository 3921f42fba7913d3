"""Diagnostics and output writers (ch4/v3/src/Outputs.cpp, World.cpp:108-119, 277-293, 331-341).

The device sums and exports are checked against numpy restatements of the reference's loops;
the C++ writers are run through the example driver and their files parsed back."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, PKG_NAME

pytestmark = pytest.mark.gpu

EPS0 = 8.85418782e-12  # ch4/v3/src/all.h:16


def _pe_oracle(W, nn, periodic, zslab=0):
    """World::getPE: 0.5 eps0 sum |E|^2 node_vol over the distinct nodes."""
    ef = W.ef.reshape(nn[2], nn[1], nn[0], 3)
    vol = W.node_vol.reshape(nn[2], nn[1], nn[0])
    keep = np.ones((nn[2], nn[1], nn[0]), bool)
    for ax, p in zip((2, 1, 0), periodic):
        if p:
            sl = [slice(None)] * 3
            sl[ax] = -1
            keep[tuple(sl)] = False
    return 0.5 * EPS0 * np.sum((ef ** 2).sum(-1) * vol * keep)


@pytest.mark.parametrize("periodic", [(0, 0, 0), (1, 1, 0)])
def test_potential_energy_matches_reference_sum(pic, periodic):
    nn, x0, xm = (33, 29, 41), (0.0, 0.0, 0.0), (0.0128, 0.0112, 0.016)
    W = pic.World(*nn, x0, xm)
    W.set_boundaries(periodic, (1,) * 6, (0, 0, 0, 0, 0.0, 100.0))
    rng = np.random.default_rng(5)
    W.ef = rng.normal(scale=1e4, size=(W.nv, 3))
    pe = W.getPE()
    ref = _pe_oracle(W, nn, periodic)
    assert pe > 0 and abs(pe - ref) <= 1e-9 * ref


def test_potential_energy_after_solve_and_slabs(pic):
    nn, x0, xm = (17, 17, 48), (0.0, 0.0, 0.0), (0.008, 0.008, 0.0235)
    W = pic.World(*nn, x0, xm)
    W.set_boundaries((1, 1, 0), (1,) * 6, (0,) * 6)
    W.set_slabs([0.0, 0.0, 0.0], [100.0, 200.0, 300.0])
    S = pic.PotentialSolver(W, 5000, 1e-8, pic.SOLVER_PCG)
    assert S.solve(raise_on_fail=True)
    S.computeEF()
    vol = W.node_vol.reshape(nn[2], nn[1], nn[0])
    # node volumes halve on the first and last plane of every slab (16 planes each)
    dv = np.prod((np.array(xm) - np.array(x0)) / (np.array(nn) - 1))
    for k in (0, 15, 16, 31, 32, 47):
        assert np.allclose(vol[k, 3, 3], dv / 2)
    assert np.allclose(vol[7, 3, 3], dv)
    pe = W.getPE()
    ref = _pe_oracle(W, nn, (1, 1, 0))
    assert abs(pe - ref) <= 1e-9 * ref
    # a vacuum capacitor per slab: PE = eps0/2 (V/d)^2 * volume, V = 100, 200, 300
    lx, ly, d = 0.008 * 16 / 16, 0.008, 0.0235 / 47 * 15
    analytic = sum(0.5 * EPS0 * (v / d) ** 2 * lx * ly * d for v in (100.0, 200.0, 300.0))
    assert abs(pe - analytic) <= 2e-3 * analytic


def test_node_type_object_id_and_box_order(pic):
    nn, x0, xm = (21, 19, 23), (0.0, 0.0, 0.0), (0.02, 0.018, 0.022)
    W = pic.World(*nn, x0, xm)
    mode = (1, 0, 0, 1, 1, 1)
    phi = (5.0, 0.0, 0.0, 7.0, 0.0, 50.0)
    W.set_boundaries((0, 1, 0), mode, phi)
    boxes = [((0.008, 0.009, 0.011), (0.006, 0.006, 0.006), 20.0),
             ((0.011, 0.009, 0.011), (0.006, 0.004, 0.004), -30.0)]
    for c, s, p in boxes:
        W.addBox(c, s, p)
    dx = (np.array(xm) - np.array(x0)) / (np.array(nn) - 1)
    k, j, i = np.meshgrid(*(np.arange(n) for n in nn[::-1]), indexing="ij")
    x = np.stack([x0[0] + i * dx[0], x0[1] + j * dx[1], x0[2] + k * dx[2]], -1)
    inside = [np.all(np.abs(x - np.array(c)) <= np.array(s) / 2, -1) for c, s, _ in boxes]
    alias = j == nn[1] - 1
    ntype = np.zeros(x.shape[:3], int)
    ijk = (i, j, k)
    wall = np.zeros_like(alias)
    fixed = np.zeros_like(alias)
    for d in (0, 2):
        for s in (0, 1):
            face = ijk[d] == (0 if s == 0 else nn[d] - 1)
            wall |= face
            if mode[2 * d + s]:
                fixed |= face
    ntype[wall] = 1
    ntype[fixed] = 2
    ntype[inside[0] | inside[1]] = 2
    ntype[:, -1, :] = ntype[:, 0, :]  # the duplicate periodic plane reports its source node
    assert np.array_equal(W.node_type.reshape(ntype.shape), ntype)
    assert np.array_equal(W.object_id.reshape(ntype.shape), (inside[0] | inside[1]).astype(int))
    ph = W.phi.reshape(ntype.shape)
    # World::computeObjectID visits the objects in order: the later box sets the overlap
    both = inside[0] & inside[1] & ~alias
    assert both.any()
    assert np.all(ph[both] == -30.0)
    assert np.all(ph[inside[0] & ~inside[1] & ~alias] == 20.0)


def test_time_and_particle_sample(pic):
    nn, x0, xm = (17, 17, 17), (0.0, 0.0, 0.0), (0.01, 0.01, 0.01)
    W = pic.World(*nn, x0, xm)
    W.setTime(3e-12, 5)
    t = 0.0
    for _ in range(3):
        W.advanceTime()
        t += 3e-12
    assert W.getTime() == t and W.getTs() == 2
    s = pic.Species("e-", pic.ME, -pic.QE, W, 1.0, capacity=10000)
    pos, vel = s.sample_particles(1000)
    assert len(pos) == 0
    s.loadUniform(x0, xm, 9001, 1e4, 1.0, 0.0, seed=3)
    s.sortIndexes()
    p = s.getPartRef()
    for num in (1000, 9001, 20000, 7):
        pos, vel = s.sample_particles(num)
        step = 1 if num > len(p) else len(p) // num
        m = min(num, len(p))
        assert len(pos) == m
        assert np.array_equal(pos, p["pos"][::step][:m]) and np.array_equal(vel, p["vel"][::step][:m])
    with pytest.raises(pic.PicError):
        s.sample_particles(0)


def _arrays(text):
    out = {}
    for m in re.finditer(r'<DataArray Name="([^"]+)" NumberOfComponents="(\d)" format="ascii" type="Float64">\n(.*?)'
                         r'</DataArray>', text, re.S):
        out[m.group(1)] = (int(m.group(2)), np.array(m.group(3).split(), float))
    return out


def test_reference_outputs_from_cpp_driver(pic, tmp_path):
    pic.library()
    pkg = os.path.join(ROOT, PKG_NAME)
    exe = str(tmp_path / "v3_loop")
    r = subprocess.run(["g++", "-std=c++17", "-O2", os.path.join(pkg, "examples", "v3_loop.cpp"),
                        "-I", os.path.join(ROOT, "include"), "-L", os.path.join(pkg, "lib"), "-lpic_gb300",
                        "-Wl,-rpath," + os.path.join(pkg, "lib"), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = tmp_path / "run"
    (run / "results").mkdir(parents=True)
    num_ts = 12
    r = subprocess.run([exe, str(num_ts), "all"], capture_output=True, text=True, timeout=300, cwd=run)
    assert r.returncode == 0, r.stderr
    res = run / "results"
    nn = (33, 33, 65)
    nv, nc = nn[0] * nn[1] * nn[2], (nn[0] - 1) * (nn[1] - 1) * (nn[2] - 1)
    names = sorted(os.listdir(res))
    for ts in ("000-1", "00000", "00010", "00011"):  # before the loop, every 10 steps and the last step
        assert f"fields_{ts}.vti" in names, names
    for ts in ("00000", "00010", "00011"):
        for sp in ("O2+", "e-"):
            assert f"parts_{sp}_{ts}.vtp" in names
    assert "fields_00005.vti" not in names
    # runtime_diags.csv
    lines = (res / "runtime_diags.csv").read_text().strip().splitlines()
    cols = lines[0].split(",")
    assert cols == ["ts", "time", "wall_time", "mp_count.O2+", "real_count.O2+", "px.O2+", "py.O2+", "pz.O2+", "KE.O2+",
                    "mp_count.e-", "real_count.e-", "px.e-", "py.e-", "pz.e-", "KE.e-", "PE", "E_total"]
    rows = np.array([[float(v) for v in ln.split(",")] for ln in lines[1:]])
    assert len(rows) == num_ts + 1 and np.array_equal(rows[:, 0], np.arange(num_ts + 1))
    assert np.allclose(rows[:, 1], (rows[:, 0] + 1) * 2e-12, rtol=1e-5)
    ke = rows[:, cols.index("KE.O2+")] + rows[:, cols.index("KE.e-")]
    pe = rows[:, cols.index("PE")]
    assert np.all(pe > 0)
    assert np.allclose(rows[:, cols.index("E_total")], ke + pe, rtol=1e-5)
    # fields at ts 10
    text = (res / "fields_00010.vti").read_text()
    assert text.startswith('<VTKFile type="ImageData">\n<ImageData Origin="0 0 0" Spacing="0.0003125 0.0003125 0.0003125" '
                           'WholeExtent="0 32 0 32 0 64">\n')
    arr = _arrays(text)
    expect = ["NodeVol", "ObjectID", "NodeType", "phi", "rho", "nd.O2+", "nd.e-", "avg_nd.O2+", "avg_nd.e-", "vel.O2+",
              "vel.e-", "T.O2+", "T.e-", "ef", "mpc.O2+", "mpc.e-"]
    assert list(arr) == expect
    for name, (comps, v) in arr.items():
        n = nc if name.startswith("mpc.") else nv
        assert comps == (3 if name.startswith("vel.") or name == "ef" else 1) and v.size == comps * n, name
    phi = arr["phi"][1].reshape(nn[2], nn[1], nn[0])
    assert np.all(phi[0] == 0) and np.all(phi[-1] == 500)
    ntype = arr["NodeType"][1].reshape(nn[2], nn[1], nn[0])
    assert np.all(ntype[0] == 2) and np.all(ntype[-1] == 2) and np.all(ntype[1:-1] == 0)
    assert np.all(arr["ObjectID"][1] == 0)
    row = rows[10]
    for sp in ("O2+", "e-"):
        assert arr["mpc." + sp][1].sum() == row[cols.index("mp_count." + sp)]
        T = arr["T." + sp][1]
        assert T.max() > 0 and T.min() >= -1e-3 * T.max()  # <v^2> - <v>^2 in FP32 may round below 0
        assert np.all(arr["nd." + sp][1] >= 0)
    # one line per z plane (Field.h:676-692)
    block = text.split('<DataArray Name="phi" NumberOfComponents="1" format="ascii" type="Float64">\n')[1]
    block = block.split("</DataArray>")[0]
    assert block.count("\n") == nn[2]
    # particle sample
    vtp = (res / "parts_e-_00010.vtp").read_text()
    assert '<Piece NumberOfPoints="1000" ' in vtp
    pts = vtp.split('format="ascii">\n')[1].split("</DataArray>")[0].split()
    p = np.array(pts, float).reshape(-1, 3)
    assert p.shape == (1000, 3)
    assert np.all(p >= 0) and np.all(p[:, :2] <= 0.01) and np.all(p[:, 2] <= 0.02)
