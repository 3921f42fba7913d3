"""The step loop and its diagnostics against the reference's algorithms at the reference's own
settings, through the C ABI:

* the plain electrostatic PIC case at full size (21^3 nodes over a 0.2 m box, Dirichlet 0 V
  walls, 80 000 electrons + 80 000 O+ ions, dt = 5e-12 s) with the reference's Poisson rule
  (SOR weight 1.4, absolute RMS residual 1e-4, PotentialSolver.cpp:69-166) on both sides,
  compared with the FP64 oracle one step at a time for 100 steps;
* Species::updateAverages (Field.h:245-261) over more than 20 samples and
  Species::computeMacroParticlesCount (Species.cpp:813-819) per cell;
* Species::merge (Species.cpp:981-1145) against the oracle's reference restatement or_merge_ref
  (pinned bit-exactly to the reference by tests/golden/merge.npz).

Tolerances, one step at a time on identical inputs: rho within 1e-6 of its maximum magnitude,
E within 1e-6 of the step's exact FP64 answer (the device meeting the reference's residual rule),
phi within 4e-6; positions within 1e-5 of a cell.
"""
import numpy as np
import pytest

import oracle as O
from conftest import golden

pytestmark = pytest.mark.gpu

EV = 11604.518  # K per eV


def plain_pic_case(port, n_each=80_000):
    nn, x0, xm = (21, 21, 21), (0.0, 0.0, 0.0), (0.2, 0.2, 0.2)
    g = port.grid(nn, x0, xm)
    den = 1e11
    w = den * 0.2 ** 3 / n_each
    ele = port.load_box_thermal_ref(g, port.mt(1), 10 ** 6, (0.1,) * 3, (0.2,) * 3, den, 1.0 * EV, w, O.ME, -O.QE)
    ion = port.load_box_thermal_ref(g, port.mt(2), 10 ** 6, (0.1,) * 3, (0.2,) * 3, den, 0.1 * EV, w, 16 * O.AMU,
                                    O.QE)
    return nn, x0, xm, g, w, ele, ion


def gpu_parts(sp):
    """The species' particles as FP64 oracle particles (positions from cell + FP32 offset) and ids."""
    gp = sp.getPartRef()
    p = np.zeros(len(gp), O.PARTICLE)
    p["pos"], p["vel"], p["w"] = gp["pos"], gp["vel"], gp["w"]
    return p, gp["id"].copy()


def test_plain_pic_full_size_each_step_matches_oracle(pic, port):
    """100 steps of push -> density -> rho -> Poisson (RMS 1e-4, SOR weight 1.4) -> E.

    One step at a time on identical inputs: before every step the device's particles, E and phi
    are handed to the oracle, which runs the same step in FP64.  Its Poisson solve runs twice
    from that phi: the reference's lexicographic GS-SOR to the reference's own rule (absolute RMS
    residual 1e-4, warm-started as solveGS is), and a tight FP64 solve (the exact answer of the
    step).  The device must meet the same RMS rule; rho within 1e-6 of its maximum; E within
    1e-6 of the exact answer's maximum (the reference GS stops within about 2e-7 of it, printed);
    phi within 4e-6 of the exact answer; positions within 1e-5 of a cell.  Beside it a
    free-running oracle loop from the same start shows how far FP32 and FP64 loops drift apart
    over the 100 steps (E bounded at 1e-5)."""
    nn, x0, xm, g, w, ele, ion = plain_pic_case(port)
    assert len(ele) == 80_000 and len(ion) == 80_000
    kind = port.node_kinds(g, 1)
    nv = int(np.prod(nn))
    dt = 5e-12
    W = pic.World(*nn, x0, xm)
    W.dirichletBoundries(0.0)
    W.setTime(dt, 1000)
    E = pic.Species("e-", pic.ME, -pic.QE, W, w, capacity=len(ele) + 64)
    I = pic.Species("O+", 16 * pic.AMU, pic.QE, W, w, capacity=len(ion) + 64)
    E.addParticles(ele["pos"], ele["vel"], ele["w"], ids=np.arange(len(ele), dtype=np.uint64), rewind=False)
    I.addParticles(ion["pos"], ion["vel"], ion["w"], ids=np.arange(len(ion), dtype=np.uint64), rewind=False)
    S = pic.PotentialSolver(W, 200000, 1e-4, pic.SOLVER_RBSOR, omega=1.4, stop=pic.STOP_ABS_RMS)
    W.configure_loop(solve_each_step=True, sort_every=20)
    # free-running oracle loop
    fe, fi = ele.copy(), ion.copy()
    fide, fidi = np.arange(len(fe), dtype=np.uint64), np.arange(len(fi), dtype=np.uint64)
    fne, fni = len(fe), len(fi)
    fef, fphi = np.zeros((nv, 3)), np.zeros(nv)
    errs = []
    dx = 0.01
    for step in range(100):
        # the step's inputs, as the device holds them
        pe, ide = gpu_parts(E)
        pi_, idi = gpu_parts(I)
        ef0, phi0 = W.ef, W.phi
        W.step()
        n_e = port.push(g, pe, ef0, dt, -O.QE, O.ME, ids=ide)
        n_i = port.push(g, pi_, ef0, dt, O.QE, 16 * O.AMU, ids=idi)
        rho = -O.QE * port.number_density(g, pe[:n_e]) + O.QE * port.number_density(g, pi_[:n_i])
        phi_gs = phi0.copy()
        ok, _, l2 = port.solve_gs(g, kind, phi_gs, rho, 200000, 1e-4)
        assert ok and l2 < 1e-4
        phi_x = phi0.copy()
        port.solve_fpcg(g, kind, phi_x, rho, 1e-13, 20000)
        ef_gs, ef_x = port.compute_ef(g, phi_gs), port.compute_ef(g, phi_x)
        nr = S.norms()
        emax, pmax = np.max(np.abs(ef_x)), np.max(np.abs(phi_x))
        err = dict(step=step, rms=np.sqrt(nr["r"] ** 2 / nv),
                   rho=np.max(np.abs(W.rho - rho)) / np.max(np.abs(rho)),
                   ef=np.max(np.abs(W.ef - ef_x)) / emax, phi=np.max(np.abs(W.phi - phi_x)) / pmax,
                   ef_vs_gs=np.max(np.abs(W.ef - ef_gs)) / emax, gs_ef=np.max(np.abs(ef_gs - ef_x)) / emax,
                   n=(len(E.getPartRef()) - n_e, len(I.getPartRef()) - n_i))
        for sp, p, ids, n in ((E, pe, ide, n_e), (I, pi_, idi, n_i)):
            gp = sp.getPartRef()
            if len(gp) != n:
                continue
            a_, b_ = np.argsort(gp["id"]), np.argsort(ids[:n])
            err["pos"] = max(err.get("pos", 0.0), np.max(np.abs(gp["pos"][a_] - p[:n]["pos"][b_])) / dx)
        # free-running FP64 loop
        fne = port.push(g, fe[:fne], fef, dt, -O.QE, O.ME, ids=fide[:fne])
        fni = port.push(g, fi[:fni], fef, dt, O.QE, 16 * O.AMU, ids=fidi[:fni])
        frho = -O.QE * port.number_density(g, fe[:fne]) + O.QE * port.number_density(g, fi[:fni])
        port.solve_gs(g, kind, fphi, frho, 200000, 1e-4)
        fef = port.compute_ef(g, fphi)
        err["drift_rho"] = np.max(np.abs(W.rho - frho)) / np.max(np.abs(frho))
        err["drift_ef"] = np.max(np.abs(W.ef - fef)) / np.max(np.abs(fef))
        errs.append(err)
    keys = ("rms", "rho", "ef", "phi", "ef_vs_gs", "gs_ef", "pos", "drift_rho", "drift_ef")
    worst = {k: max(e_.get(k, 0.0) for e_ in errs) for k in keys}
    print("worst over 100 steps:", worst)
    assert all(e_["n"] == (0, 0) for e_ in errs), [e_ for e_ in errs if e_["n"] != (0, 0)]
    assert worst["rms"] <= 1e-4  # the same Poisson rule as the reference
    assert worst["rho"] <= 1e-6
    assert worst["ef"] <= 1e-6
    assert worst["phi"] <= 4e-6
    assert worst["ef_vs_gs"] <= 2e-6  # both within their truncation of the exact answer
    assert worst["pos"] <= 1e-5
    # free-running: E stays close; rho in the max norm is not bounded this way, since a single
    # wall absorption that one loop makes a step earlier than the other moves one macroparticle,
    # about 8 % of max |rho| on this grid (printed above)
    assert worst["drift_ef"] <= 1e-5


def test_den_avg_and_cell_counts_match_oracle(pic, port):
    """updateAverages after every push for 45 steps (two restarts of the 20-sample moving
    average, Field.h:245-261) against the oracle's restatement, fed each step with the oracle's
    density of the same push from the device's pre-step particles; then the per-cell
    macroparticle counts (Species.cpp:813-819) of the device's particles."""
    nn, x0, xm = (17, 13, 21), (0.0, 0.0, 0.0), (0.016, 0.012, 0.02)
    g = port.grid(nn, x0, xm)
    nv = int(np.prod(nn))
    rng = np.random.default_rng(31)
    n = 60_000
    p = np.zeros(n, O.PARTICLE)
    p["pos"] = rng.uniform(0.0, 1.0, (n, 3)) * np.array(xm) * 0.999999
    p["vel"] = rng.normal(size=(n, 3)) * 3e5
    p["w"] = rng.lognormal(np.log(50.0) - 0.125, 0.5, n).astype(np.float32)
    ef = np.zeros((nv, 3))
    ef[:, 2] = 2e4  # a uniform field: densities change from step to step
    dt = 2e-11
    W = pic.World(*nn, x0, xm)
    W.dirichletBoundries(0.0)
    W.setTime(dt, 1000)
    W.ef = ef
    S = pic.Species("e-", pic.ME, -pic.QE, W, 50.0, capacity=n + 64)
    ids = np.arange(n, dtype=np.uint64)
    S.addParticles(p["pos"], p["vel"], p["w"], ids=ids, rewind=False)
    avg = np.zeros(nv)
    samples = 0
    for step in range(45):
        po, ido = gpu_parts(S)
        S.advance(dt, deposit=True)
        W.computeChargeDensity()
        S.updateAverages()
        m = port.push(g, po, ef, dt, -O.QE, O.ME, ids=ido)
        den = port.number_density(g, po[:m])
        assert np.max(np.abs(S.den - den)) <= 1e-6 * np.max(den), step
        samples = O.moving_average_update(avg, samples, den)
        assert np.max(np.abs(S.den_avg - avg)) <= 1e-6 * np.max(avg), step
    assert samples == 5  # 45 samples: restarted at 21 and 41
    counts = S.computeMacroParticlesCount()
    pg, _ = gpu_parts(S)
    ref = O.macro_particle_count(g, pg)
    assert counts.sum() == len(pg)
    # positions come back as x0 + (cell + FP32 offset) dx in FP64: a particle within rounding of a
    # cell face may land on the other side
    assert np.sum(np.abs(counts - ref)) <= 2 + len(pg) // 20000


# ------------------------------------------------------------------------------------------
# merge against the reference's own algorithm (or_merge_ref)
# ------------------------------------------------------------------------------------------
def cells_of(pos, x0, dx, nn):
    ijk = np.floor((pos - np.asarray(x0)) / np.asarray(dx)).astype(np.int64)
    ijk = np.minimum(np.maximum(ijk, 0), np.asarray(nn) - 2)
    return (ijk[:, 2] * (nn[1] - 1) + ijk[:, 1]) * (nn[0] - 1) + ijk[:, 0]


def cell_moments(pos, vel, w, x0, dx, nn):
    """Per cell: sum w, sum w v (3), sum w v^2 (3)."""
    c = cells_of(pos, x0, dx, nn)
    nc = int(np.prod(np.asarray(nn) - 1))
    out = np.zeros((nc, 7))
    out[:, 0] = np.bincount(c, w, nc)
    for d in range(3):
        out[:, 1 + d] = np.bincount(c, w * vel[:, d], nc)
        out[:, 4 + d] = np.bincount(c, w * vel[:, d] ** 2, nc)
    return out


def range_quirk_inactive(pos, vel, x0, dx, nn, min_count):
    """The reference starts each cell's velocity range from particle 0 of the species
    (Species.cpp:985).  That start changes nothing when particle 0's velocity lies inside every
    merged cell's own range, which this checks."""
    c = cells_of(pos, x0, dx, nn)
    v0 = vel[0]
    for cell in np.unique(c):
        sel = c == cell
        if sel.sum() < min_count:
            continue
        if np.any(vel[sel].min(0) > v0) or np.any(vel[sel].max(0) < v0):
            return False
    return True


def bin_flips(pos, vel32, x0, dx, nn, min_count):
    """Particles whose velocity bin differs between the reference's FP64 arithmetic
    (Species.cpp:985-1030) and the device's FP32 arithmetic (round-to-nearest subtract, multiply
    and divide, emulated exactly with numpy float32), for cells that are merged."""
    c = cells_of(pos, x0, dx, nn)
    bad = np.zeros(len(vel32), bool)
    for cell in np.unique(c):
        sel = np.nonzero(c == cell)[0]
        if len(sel) < min_count:
            continue
        v64 = vel32[sel]
        lo64, hi64 = v64.min(0), v64.max(0)
        hi64 = np.where(hi64 > 0, hi64 * 1.001, hi64 * 0.999)
        b64 = ((v64 - lo64) / ((hi64 - lo64) / 15.0)).astype(np.int64)
        v32 = v64.astype(np.float32)
        lo32, hi32 = v32.min(0), v32.max(0)
        hi32 = np.where(hi32 > 0, hi32 * np.float32(1.001), hi32 * np.float32(0.999)).astype(np.float32)
        dv32 = ((hi32 - lo32) / np.float32(15.0)).astype(np.float32)
        b32 = np.clip(((v32 - lo32) / dv32).astype(np.int64), 0, 14)
        bad[sel] = np.any(np.clip(b64, 0, 14) != b32, axis=1)
    return bad


def run_both(pic, port, nn, x0, xm, pos, vel, w, ef, dt, min_count=10):
    """GPU merge and the oracle's reference merge on the same particles (FP32-rounded)."""
    n = len(w)
    vel32 = vel.astype(np.float32).astype(np.float64)
    w32 = w.astype(np.float32).astype(np.float64)
    W = pic.World(*nn, x0, xm)
    W.setTime(dt, 10)
    W.ef = ef
    W.advanceTime()
    e = pic.Species("e-", pic.ME, -pic.QE, W, float(np.mean(w)), capacity=2 * n + 1024)
    ids = np.arange(n, dtype=np.uint64)
    e.addParticles(pos, vel32, w32, ids=ids, rewind=False)
    e.merge(min_count=min_count)
    st = e.merge_stats()
    gp = e.getPartRef()
    g = port.grid(nn, x0, xm)
    p = np.zeros(2 * n + 1024, O.PARTICLE)
    p["pos"][:n], p["vel"][:n], p["w"][:n] = pos, vel32, w32
    n_ref = port.merge_ref(g, port.mt(17), p, n, ef, -O.QE, O.ME, dt, min_count)
    return st, gp, ids, p[:n_ref].copy()


def test_merge_matches_reference_on_its_golden_input(pic, port):
    """merge.npz holds the reference's own merge of 1 200 electrons in 2 cells under a random
    node field.  Same cells and bins merged, same particle count after the merge; per-cell
    weight exactly, momentum and energy within the spread of the half-step rewind (addParticle
    gathers E at the randomly chosen member position, Species.cpp:431)."""
    d = golden("merge")
    nn, x0, xm = tuple(int(v) for v in d["nn"]), d["x0"], d["xm"]
    dt = float(d["dt"])
    dx = (np.asarray(xm) - np.asarray(x0)) / (np.asarray(nn) - 1)
    assert range_quirk_inactive(d["in_pos"], d["in_vel"], x0, dx, nn, 10)
    assert not bin_flips(d["in_pos"], d["in_vel"], x0, dx, nn, 10).any()
    st, gp, ids, _ = run_both(pic, port, nn, x0, xm, d["in_pos"], d["in_vel"], d["in_w"], d["ef"], dt)
    n_in, n_out = len(d["in_w"]), len(d["out_w"])
    # the reference's output (golden) against the GPU
    assert len(gp) == n_out
    assert st["removed"] - 2 * st["bins"] == n_in - n_out
    mg = cell_moments(gp["pos"], gp["vel"], gp["w"], x0, dx, nn)
    mr = cell_moments(d["out_pos"], d["out_vel"], d["out_w"], x0, dx, nn)
    assert np.allclose(mg[:, 0], mr[:, 0], rtol=1e-6)
    # the rewind moves each product's velocity by q/m E(x) dt / 2 at its (random) position
    qm = O.QE / O.ME
    span = qm * 0.5 * dt * (np.abs(d["ef"]).max(0) * 2)
    wprod = gp["w"][~np.isin(gp["id"], ids)].sum()
    for ax in range(3):
        assert np.all(np.abs(mg[:, 1 + ax] - mr[:, 1 + ax]) <= wprod * span[ax] + 1e-6 * np.abs(mr[:, 1 + ax]).max())


def test_merge_matches_reference_on_lognormal_cells(pic, port):
    """A lognormal-weight (sigma 0.5) electron population, 2 eV Maxwellian, ~800 per cell in
    27 cells (about 2 000 bins merged), under a uniform field (the rewind is then the same for every product).  The
    binning rule is the reference's with the cell's own velocity range, the 15^3 grid, the
    1.001 / 0.999 upper-bound widening and merging of bins with more than two particles; the
    merge threshold is the reference's 10 particles per cell.  Exclusions: the range start from
    particle 0 (checked inactive on this input) and the per-species cell cap of 1 024
    particles (not reached).  Compared: bins merged, particles removed, per-cell sum w, sum w v
    and sum w v^2, and the sorted product weights and velocities per cell; product positions are
    member positions chosen by different generators (MT19937 / Philox), so only their cells and
    membership are compared."""
    nn, x0, xm = (4, 4, 4), (0.0, 0.0, 0.0), (0.003, 0.003, 0.003)
    dx = (np.asarray(xm) - np.asarray(x0)) / (np.asarray(nn) - 1)
    rng = np.random.default_rng(8)
    n = 27 * 800
    pos = rng.uniform(0.0, 1.0, (n, 3)) * np.array(xm) * 0.999999
    vth = np.sqrt(O.KB * 2.0 * EV / O.ME)
    vel = rng.normal(size=(n, 3)) * vth
    vel[0] = 0.0  # particle 0 at the centre of every cell's velocity range
    w = rng.lognormal(np.log(64.0) - 0.125, 0.5, n)
    # keep every particle off the bin faces where FP32 and FP64 could disagree (a rounding-level
    # nudge of the few that sit on one), so that both sides merge the same bins
    for _ in range(10):
        bad = bin_flips(pos, vel.astype(np.float32).astype(np.float64), x0, dx, nn, 10)
        if not bad.any():
            break
        vel[bad] *= 1.0 + 1e-4
    assert not bin_flips(pos, vel.astype(np.float32).astype(np.float64), x0, dx, nn, 10).any()
    assert range_quirk_inactive(pos, vel, x0, dx, nn, 10)
    nv = int(np.prod(nn))
    ef = np.tile([3e3, -2e3, 1e3], (nv, 1)).astype(np.float64)
    dt = 1e-12
    st, gp, ids, rp = run_both(pic, port, nn, x0, xm, pos, vel, w, ef, dt)
    # the reference output: survivors keep their exact input (pos, vel); products are new
    in_keys = {tuple(v) for v in vel.astype(np.float32).astype(np.float64)}
    is_prod_ref = np.array([tuple(v) not in in_keys for v in rp["vel"]])
    bins_ref = int(is_prod_ref.sum()) // 2
    removed_ref = n - (len(rp) - 2 * bins_ref)
    assert st["bins"] == bins_ref
    assert st["removed"] == removed_ref
    assert len(gp) == len(rp)
    mg = cell_moments(gp["pos"], gp["vel"], gp["w"], x0, dx, nn)
    mr = cell_moments(rp["pos"], rp["vel"], rp["w"], x0, dx, nn)
    assert np.allclose(mg[:, 0], mr[:, 0], rtol=1e-6)
    assert np.all(np.abs(mg[:, 1:4] - mr[:, 1:4]) <= 1e-5 * np.abs(mr[:, 1:4]).max())
    assert np.allclose(mg[:, 4:7], mr[:, 4:7], rtol=1e-5)
    # products per cell: the same multiset of (w, v)
    is_prod_gpu = ~np.isin(gp["id"], ids)
    assert is_prod_gpu.sum() == 2 * bins_ref
    cg = cells_of(gp["pos"][is_prod_gpu], x0, dx, nn)
    cr = cells_of(rp["pos"][is_prod_ref], x0, dx, nn)
    assert np.array_equal(np.bincount(cg, minlength=27), np.bincount(cr, minlength=27))
    for cell in range(27):
        a = np.column_stack([gp["w"][is_prod_gpu][cg == cell], gp["vel"][is_prod_gpu][cg == cell]])
        b = np.column_stack([rp["w"][is_prod_ref][cr == cell], rp["vel"][is_prod_ref][cr == cell]])
        a = a[np.lexsort(a.T[::-1])]
        b = b[np.lexsort(b.T[::-1])]
        assert np.allclose(a, b, rtol=1e-5, atol=1e-5 * vth), cell
    # every product sits at the position of an input particle of its cell (to the FP32 offset)
    cin = cells_of(pos, x0, dx, nn)
    for q, cell in zip(gp["pos"][is_prod_gpu], cg):
        dmin = np.min(np.abs(pos[cin == cell] - q).max(1))
        assert dmin <= 1e-6 * dx.max()
