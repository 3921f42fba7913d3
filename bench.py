"""Benchmark of the GB300 PIC + DSMC step loop: particle-steps per second on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload large|discharge|plain]
    python bench.py --impl reference ...   (the reference algorithm on the host cores)

A step is one iteration of the ch4/v3 time loop on the workload's synthetic discharge:
electron-impact collisions against the O2 background (fused into the electron push), leapfrog
push with trilinear gather and fixed-point deposition for both species, charge density,
FP64-refined Poisson solve to a 1e-6 relative residual, E = -grad(phi), and a counting sort
by cell every 20 steps.  value = particles pushed per step / device step time (CUDA events on
the library's stream).  Inputs (particles, fields) are resident in HBM and larger than L2.
e2e runs the same K steps through the C ABI from pinned host buffers: the particle upload and
a per-step read of the conservation diagnostics (Outputs.cpp:143-182) are inside its clock.
One JSON line on stdout (rank 0).
"""
import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
PKG = "engineering-degree-in-plasma-simulations_gb300"

QE, AMU, ME, KB = 1.602176565e-19, 1.660538921e-27, 9.10938215e-31, 1.380648e-23
EV_K = QE / KB

# Lotz-form ionisation of O2 (threshold 12.06 eV, peak ~2.7e-20 m^2 near 100 eV):
#   sigma = A ln(E/I) / (E I) (1 - b exp(-c (E/I - 1)))
LOTZ = dict(A=2.107e-17, b=1.0, c=0.18, I=12.06)


def sigma_tables():
    """Synthetic O2 collision table: elastic 6e-20/sqrt(1+E/10eV) m^2 plus Lotz ionisation."""
    E = np.geomspace(0.01, 1e5, 400)
    el = 6e-20 / np.sqrt(1 + E / 10.0)
    x = E / LOTZ["I"]
    ion = np.where(E > LOTZ["I"], LOTZ["A"] * np.log(np.maximum(x, 1)) / (E * LOTZ["I"]) *
                   (1 - LOTZ["b"] * np.exp(-LOTZ["c"] * (x - 1))), 0.0)
    return E, el + ion


WORKLOADS = {
    # 256 x 256 x 512 nodes over 0.04 x 0.04 x 0.08 m, 1000 V anode, O2 2e21 m^-3, 100 M + 100 M
    "large": dict(nn=(256, 256, 512), L=(0.04, 0.04, 0.08), V=1000.0, n_gas=2e21, n_each=100_000_000,
                  w_mean=5.12, dt=1e-12, name="large discharge 256x256x512, 100M e- + 100M O2+"),
    # 64 x 64 x 256 nodes over 0.02 x 0.02 x 0.08 m, 500 V, O2 1e21 m^-3, 2 M + 2 M, mean weight 64
    "discharge": dict(nn=(64, 64, 256), L=(0.02, 0.02, 0.08), V=500.0, n_gas=1e21, n_each=2_000_000,
                      w_mean=64.0, dt=2e-12, name="electrode discharge 64x64x256, 2M e- + 2M O2+"),
    # the large discharge at one eighth of the nodes and particles: particle arrays (0.5 GB per
    # species) still exceed L2, small enough for a full profiler capture
    "mid": dict(nn=(128, 128, 256), L=(0.04, 0.04, 0.08), V=1000.0, n_gas=2e21, n_each=12_500_000,
                w_mean=40.96, dt=1e-12, name="mid discharge 128x128x256, 12.5M e- + 12.5M O2+"),
}
# BASELINE config 4: 64 independent discharges on 32 x 32 x 128 nodes (C2 physics), anodes spaced
# uniformly over 200-800 V, background densities over 5e20-2e21 m^-3, particles per species per
# instance log-uniform over 10k-2M; the instances are stacked along z in one world (instance slabs),
# so every kernel launch advances all of them
ENSEMBLE = dict(kind="ensemble", instances=64, nn=(32, 32, 128), L=(0.02, 0.02, 0.08), V=(200.0, 800.0),
                n_gas=(5e20, 2e21), n_range=(10_000, 2_000_000), density=1e13, dt=2e-12,
                name="ensemble of 64 discharges, 32x32x128 nodes each, stacked in one world")
WORKLOADS["ensemble"] = ENSEMBLE
MERGE_EVERY = 20  # merge pass cadence in the timed loop (the reference merges every 50 steps)
MERGE_MIN = 64    # a cell is merged when it holds more than this many particles of a species


SORT_EVERY = [20]  # steps between the loop's sort checks (a species re-sorts when 2 % of it moved)


def setup_world(pic, wl, seed=1):
    nn, L = wl["nn"], wl["L"]
    W = pic.World(*nn, (0.0, 0.0, 0.0), L)
    W.set_boundaries((1, 1, 0), (1,) * 6, (0, 0, 0, 0, 0.0, wl["V"]))
    W.setTime(wl["dt"], 1 << 30)
    n = wl["n_each"]
    cap = int(n * 1.25) + 4096
    bound = cap * wl["w_mean"] * 400.0
    e = pic.Species("e-", ME, -QE, W, wl["w_mean"], capacity=cap, weight_bound=bound)
    i = pic.Species("O2+", 32 * AMU, QE, W, wl["w_mean"], capacity=cap, weight_bound=bound)
    lo, hi = (0.0, 0.0, 0.3 * L[2]), (L[0], L[1], 0.7 * L[2])
    e.loadUniform(lo, hi, n, 2.0 * EV_K, wl["w_mean"], 0.5, seed=seed)
    i.loadUniform(lo, hi, n, 0.03 * EV_K, wl["w_mean"], 0.5, seed=seed + 1)
    E, S = sigma_tables()
    M = pic.MC_MEX_Ionization(e, i, W, wl["n_gas"], 300.0, 32 * AMU, LOTZ["I"], E, S, sigma_ion_kind=1,
                              sigma_ion_params=(LOTZ["A"], LOTZ["b"], LOTZ["c"], 0.0), seed=seed)
    S_ = pic.PotentialSolver(W, 20000, 1e-6, pic.SOLVER_LEARNED)
    W.configure_loop(solve_each_step=True, sort_every=SORT_EVERY[0], merge_every=MERGE_EVERY, merge_after=0,
                     merge_min=MERGE_MIN)
    return W, e, i, M, S_


def setup_ensemble(pic, wl, seed=1):
    nI = wl["instances"]
    ni, nj, nks = wl["nn"]
    L = wl["L"]
    dz = L[2] / (nks - 1)
    nk = nI * nks
    W = pic.World(ni, nj, nk, (0.0, 0.0, 0.0), (L[0], L[1], (nk - 1) * dz))
    W.set_boundaries((1, 1, 0), (1,) * 6, (0.0,) * 6)
    volts = np.linspace(wl["V"][0], wl["V"][1], nI)
    W.set_slabs(np.zeros(nI), volts)
    W.setTime(wl["dt"], 1 << 30)
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(np.log(wl["n_range"][0]), np.log(wl["n_range"][1]), nI)).astype(np.int64)
    band = L[0] * L[1] * 0.4 * L[2]
    w_means = wl["density"] * band / counts
    cap = int(counts.sum() * 1.25) + 4096
    bound = float((counts * w_means).sum()) * 400.0
    e = pic.Species("e-", ME, -QE, W, float(np.median(w_means)), capacity=cap, weight_bound=bound)
    i = pic.Species("O2+", 32 * AMU, QE, W, float(np.median(w_means)), capacity=cap, weight_bound=bound)
    for s_ in range(nI):
        z0 = s_ * nks * dz
        lo, hi = (0.0, 0.0, z0 + 0.3 * L[2]), (L[0], L[1], z0 + 0.7 * L[2])
        e.loadUniform(lo, hi, int(counts[s_]), 2.0 * EV_K, w_means[s_], 0.5, seed=seed + 2 * s_)
        i.loadUniform(lo, hi, int(counts[s_]), 0.03 * EV_K, w_means[s_], 0.5, seed=seed + 2 * s_ + 1)
    E, S = sigma_tables()
    dens = np.geomspace(wl["n_gas"][0], wl["n_gas"][1], nI)
    M = pic.MC_MEX_Ionization(e, i, W, float(dens[0]), 300.0, 32 * AMU, LOTZ["I"], E, S, sigma_ion_kind=1,
                              sigma_ion_params=(LOTZ["A"], LOTZ["b"], LOTZ["c"], 0.0), seed=seed)
    M.set_slab_density(dens)
    S_ = pic.PotentialSolver(W, 20000, 1e-6, pic.SOLVER_LEARNED)
    W.configure_loop(solve_each_step=True, sort_every=SORT_EVERY[0], merge_every=MERGE_EVERY, merge_after=0,
                     merge_min=MERGE_MIN)
    return W, e, i, M, S_


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.proc:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (getattr(self, "out", "") or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def roofline_traffic():
    """DRAM bytes per particle-step of the push kernel from the committed ncu capture, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return 0, 1, 0
    import torch
    import torch.distributed as dist

    rank, local = int(os.environ["RANK"]), int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist.init_process_group("nccl")
    return rank, ws, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def _reduce(x, ws, op):
    """Reduction over replicas: tensors live on the GPU under NCCL, on the CPU under gloo."""
    if ws <= 1:
        return x
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(x, ws):
    import torch.distributed as dist

    return _reduce(x, ws, dist.ReduceOp.MAX) if ws > 1 else x


def sum_over_ranks(x, ws):
    import torch.distributed as dist

    return _reduce(x, ws, dist.ReduceOp.SUM) if ws > 1 else x


def aggregate(parts_per_rank, seconds_per_rank, ws):
    """Whole-job throughput of independent replicas: all ranks' particle-steps over the slowest
    rank's time."""
    return sum_over_ranks(parts_per_rank, ws) / max_over_ranks(seconds_per_rank, ws)


# ------------------------------------------------------------------------------------------
# CPU side: the reference algorithm (oracle port of ch4/v3) on the host cores
# ------------------------------------------------------------------------------------------
def cpu_reference(wl, gpu_inner_per_step, seed=3, sample=1_000_000, steps=2):
    """Times the FP64 restatement of the reference loop on a bounded sample.

    Particle work (collisions, push, deposit) runs on `sample` electrons + `sample` ions for
    `steps` steps and is scaled linearly to the full particle count; the field work (charge
    density, Poisson iterations at the GPU's average count per step, E field) runs on the full
    grid.  The electron push uses host_cores-1 threads like the reference's ThreadPool; the ion
    push, deposit and collisions are serial as in the reference."""
    import oracle as O

    port = O.Port()
    nn, L = wl["nn"], wl["L"]
    g = port.grid(nn, (0, 0, 0), L, periodic=(1, 1, 0))
    kind = port.node_kinds(g, 1)
    nv = int(np.prod(nn))
    threads = max(1, (os.cpu_count() or 2) - 1)
    rng = np.random.default_rng(seed)
    n = min(sample, wl["n_each"])

    def make(T, mass):
        p = np.zeros(int(n * 1.2) + 1024, O.PARTICLE)
        p["pos"][:n] = rng.uniform((0, 0, 0.3 * L[2]), (L[0], L[1], 0.7 * L[2]), (n, 3))
        p["vel"][:n] = rng.normal(size=(n, 3)) * np.sqrt(KB * T / mass)
        p["w"][:n] = rng.lognormal(np.log(wl["w_mean"]) - 0.125, 0.5, n)
        return p

    ele, ion = make(2.0 * EV_K, ME), make(0.03 * EV_K, 32 * AMU)
    eid = np.arange(len(ele), dtype=np.uint64)
    iid = np.arange(len(ion), dtype=np.uint64) + (1 << 40)
    E, S = sigma_tables()
    cp = port.coll_params(E, S, 32 * AMU, LOTZ["I"], 1, (0.0, LOTZ["b"], LOTZ["c"]), sig_A=LOTZ["A"],
                          n_neutral=wl["n_gas"], T_neutral=300.0)
    ef = np.zeros((nv, 3))
    ne_, ni_ = n, n
    t_part = 0.0
    t_push_mt = 0.0
    for s in range(steps):
        t0 = time.perf_counter()
        _, _, ne_, ni_ = port.mcc_background(g, cp, ele, eid, ne_, ion, iid, ni_, wl["dt"], seed, s)
        t1 = time.perf_counter()
        ne_ = port.push(g, ele[:ne_], ef, wl["dt"], -QE, ME, ids=eid[:ne_], threads=threads)
        t_push_mt += time.perf_counter() - t1
        ni_ = port.push(g, ion[:ni_], ef, wl["dt"], QE, 32 * AMU, ids=iid[:ni_], threads=1)
        de = port.number_density(g, ele[:ne_])
        di = port.number_density(g, ion[:ni_])
        t_part += time.perf_counter() - t0
    t_part_per_particle = t_part / steps / (ne_ + ni_)
    # the same electron push on one thread, for the single-core figure
    t0 = time.perf_counter()
    port.push(g, ele[:ne_].copy(), ef, wl["dt"], -QE, ME, ids=eid[:ne_].copy(), threads=1)
    t_push_1 = time.perf_counter() - t0
    t_part_1 = (t_part - t_push_mt + steps * t_push_1) / steps / (ne_ + ni_)
    # field work on the full grid
    t0 = time.perf_counter()
    rho = QE * (di - de)
    t_rho = time.perf_counter() - t0
    phi = np.zeros(nv)
    phi[kind == O.FIXED] = np.where(np.arange(nv)[kind == O.FIXED] // (nn[0] * nn[1]) == nn[2] - 1, wl["V"], 0.0)
    probe = 3
    t0 = time.perf_counter()
    port.solve_fpcg(g, kind, phi, rho, 1e-30, probe)
    t_iter = (time.perf_counter() - t0) / probe
    t0 = time.perf_counter()
    port.compute_ef(g, phi)
    t_ef = time.perf_counter() - t0
    n_full = 2 * wl["n_each"]
    t_step = n_full * t_part_per_particle + t_rho + gpu_inner_per_step * t_iter + t_ef
    t_step_1 = n_full * t_part_1 + t_rho + gpu_inner_per_step * t_iter + t_ef
    return {
        "value": n_full / t_step,
        "single_thread_value": n_full / t_step_1,
        "unit": "particle-steps/s",
        "cores": threads,
        "kind": "port",
        "sample": (f"{n} e- + {n} O2+ for {steps} steps on the full {nn[0]}x{nn[1]}x{nn[2]} grid "
                   f"(collisions, push, deposit: {t_part_per_particle * 1e9:.1f} ns/particle-step, scaled to "
                   f"{n_full} particles); charge density, {gpu_inner_per_step:.1f} PCG iterations "
                   f"({t_iter:.3f} s each, timed on {probe}) and E field on the full grid"),
        "seconds_per_step": t_step,
    }


def run_reference(args, wl, rank, ws):
    if rank != 0:
        return
    # the Poisson iteration count per step follows the plain PCG on this grid; 60 is the
    # warm-started count measured on the GPU for this workload and is re-read when available
    inner = float(os.environ.get("PIC_BENCH_INNER_ITERS", "60"))
    samples = []
    for _ in range(max(1, args.steps // 10)):
        samples.append(cpu_reference(wl, inner, sample=args.cpu_sample, steps=1))
    best = max(samples, key=lambda s: s["value"])
    line = {
        "metric": "particle-steps/s", "value": best["value"], "unit": "particle-steps/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": best["seconds_per_step"] * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": wl["name"]},
        "cpu_baseline": {k: best[k] for k in ("value", "unit", "cores", "kind", "sample", "single_thread_value")},
        "e2e": {"value": best["value"], "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------
def run_gpu(args, wl, rank, ws, local):
    import torch

    pic = importlib.import_module(PKG)
    ensemble = wl.get("kind") == "ensemble"
    W, e, i, M, S = (setup_ensemble if ensemble else setup_world)(pic, wl, seed=1 + rank)
    assert S.solve(raise_on_fail=True)  # initial vacuum + space-charge field (main.cpp:172-173)
    S.computeEF()
    tuned = W.autotune()  # launch shapes measured on this world's data (outside the timed region)
    for _ in range(args.warmup):
        W.step()
    W.synchronize()
    W.timing(True)
    W.timing_reset()
    st0 = S.stats()
    n0 = e.getNumParticles() + i.getNumParticles()
    launches0 = W.launches()
    coll0 = M.stats()
    barrier(ws)
    W.synchronize()
    with ClockSampler(local) as clk:
        # the timed steps are the profiler range (cudaProfilerStart/Stop; no effect without a profiler)
        torch.cuda.profiler.start()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            W.step()
        W.synchronize()
        wall = time.perf_counter() - t0
        torch.cuda.profiler.stop()
    n1 = e.getNumParticles() + i.getNumParticles()
    launches = W.launches() - launches0
    step_ms, _ = W.timer("step")
    st1 = S.stats()
    coll1 = M.stats()
    groups = {}
    for name in ("push_deposit", "mcc", "compact", "rho", "poisson", "efield", "sort"):
        ms, nl = W.timer(name)
        groups[name] = dict(ms=ms, launches=nl)
    parts_per_step = 0.5 * (n0 + n1)
    value = aggregate(parts_per_step * args.steps, step_ms / 1e3, ws)
    # roofline of the dominant kernel group
    peak, peak_kind = measured_peak()
    nv = int(W.nv)
    inner = st1["inner"] - st0["inner"]
    refine = st1["refinements"] - st0["refinements"]
    n_e_avg = 0.5 * parts_per_step  # electrons ~ half
    algo = {
        # 60 B per particle-step + 20 B per node per species push
        "push_deposit": (60.0 * parts_per_step + 2 * 20.0 * nv) * args.steps,
        # collision candidates: the 8 B id of every electron (the collisions themselves are rare)
        "mcc": 8.0 * n_e_avg * args.steps,
        # 40 B per node per inner PCG iteration, 24 B per node per FP64 refinement
        "poisson": 40.0 * nv * inner + 24.0 * nv * refine,
        "efield": 24.0 * nv * args.steps,
        "rho": (2 * 20.0 + 4.0) * nv * args.steps,
    }
    kernels = {}
    for name, b in algo.items():
        ms = groups[name]["ms"]
        if ms > 0:
            kernels[name] = dict(share=ms / step_ms, achieved_gbs=b / (ms / 1e3) / 1e9,
                                 ms_per_step=ms / args.steps)
    dom = max(kernels, key=lambda k: kernels[k]["share"])
    launches_dom = max(1, groups[dom]["launches"])
    achieved = algo[dom] / (groups[dom]["ms"] / 1e3) / 1e9
    traffic = roofline_traffic().get(dom)
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind,
            "traffic": traffic * algo[dom] / launches_dom if traffic else None,
            "algorithmic_bytes_per_launch": algo[dom] / launches_dom}
    push_ms = groups["push_deposit"]["ms"]
    push_gbs = algo["push_deposit"] / (push_ms / 1e3) / 1e9 if push_ms > 0 else None
    clocks = clk.summary()
    W.close()
    # e2e: same loop through the C ABI from pinned host buffers (upload + per-step diagnostics)
    e2e = None if ensemble else run_e2e(pic, wl, args, rank)
    poisson = None
    if rank == 0 and args.poisson > 0:
        poisson = poisson_bench(pic, args.poisson, methods=args.poisson_methods.split(","))
    dsmc = None
    if rank == 0 and args.dsmc > 0:
        dsmc = dsmc_bench(pic, args.dsmc, cpu=not args.no_cpu)
    cpu = None
    if rank == 0 and not args.no_cpu and not ensemble:
        cpu = cpu_reference(wl, inner / max(1, args.steps), sample=args.cpu_sample, steps=1)
        cpu = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample", "single_thread_value")}
    coll = {k: coll1[k] - coll0[k] for k in coll1}
    line = {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": wl["name"],
                   "grid": list(wl["nn"]) + ([wl["instances"]] if ensemble else []),
                   "particles_per_step": parts_per_step,
                   "poisson": "flexible CG with the learned multilevel preconditioner, FP32 iterations in "
                                      "float-float refinement to 1e-6 relative, warm-started",
                   "collisions_per_step": coll["collisions"] / args.steps,
                   "ionizations_per_step": coll["ionizations"] / args.steps,
                   "poisson_inner_per_step": inner / args.steps, "sort_every": SORT_EVERY[0],
                   "l2": "inputs larger than L2 (particles %.1f GB)" % (parts_per_step * 36 / 1e9),
                   "merging": "every %d steps, cells above %d particles" % (MERGE_EVERY, MERGE_MIN),
                   "parallelism": "replicas" if ws > 1 else "1 GPU",
                   "autotuned": tuned},
        "wall_s": wall,
        "gpu_launches": launches,
        "roofline": roof,
        "push_deposit_gbs": push_gbs,
        "kernels": kernels,
        "groups_ms_per_step": {k: v["ms"] / args.steps for k, v in groups.items()},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "poisson_time_to_1e-6": poisson,
        "dsmc": dsmc,
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def blob_rho(nn, seed):
    """Seeded sum of 8-64 Gaussian blobs, amplitude +-1e-3 C/m^3, widths 2-20 cells (node field)."""
    rng = np.random.default_rng(seed)
    rho = np.zeros(nn[::-1])  # [k][j][i]
    for _ in range(int(rng.integers(8, 65))):
        c = rng.uniform(0, 1, 3) * (np.array(nn) - 1)
        wdt = rng.uniform(2, 20)
        amp = rng.uniform(-1e-3, 1e-3)
        lo = np.maximum(0, np.floor(c - 3 * wdt)).astype(int)
        hi = np.minimum(np.array(nn), np.ceil(c + 3 * wdt + 1)).astype(int)
        ax = [np.arange(lo[d], hi[d]) for d in range(3)]
        gx, gy, gz = [np.exp(-0.5 * ((a - c[d]) / wdt) ** 2) for d, a in enumerate(ax)]
        rho[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]] += amp * gz[:, None, None] * gy[None, :, None] * gx[None, None, :]
    return rho.ravel()


def poisson_bench(pic, n, seed=5, train_steps=300, methods=("rbsor", "pcg", "learned_start", "learned")):
    """Time to a 1e-6 FP64 relative residual from the Dirichlet-only start, n^3 nodes over a
    0.04 m cube, z faces at 0 V / 1000 V, periodic x, y; blob charge density.  Plain red-black
    SOR and Jacobi-PCG against the learned multilevel preconditioner, first at its starting
    (BPX) weights, then after online training on the pairs of four solves of other blob densities
    plus white-noise pairs.  Training time is reported separately (it is amortised over a run)."""
    nn = (n, n, n)
    W = pic.World(n, n, n, (0.0, 0.0, 0.0), (0.04, 0.04, 0.04))
    W.set_boundaries((1, 1, 0), (1,) * 6, (0, 0, 0, 0, 0.0, 1000.0))
    rho_test = blob_rho(nn, seed)
    W.rho = rho_test
    phi0 = W.phi
    omega = 2.0 / (1.0 + np.sin(np.pi / (n - 1)))  # optimal SOR weight of the model problem
    out = {"grid": [n, n, n], "tol": 1e-6}

    def timed(method, w=1.4):
        W.phi = phi0
        S = pic.PotentialSolver(W, 200000, 1e-6, method, omega=w)
        W.timing(True)
        W.timing_reset()
        W.synchronize()
        t0 = time.perf_counter()
        ok = S.solve()
        W.synchronize()
        wall = time.perf_counter() - t0
        dev_ms, launches = W.timer("poisson")
        W.timing(False)
        return {"seconds": wall, "iterations": S.iters, "rel": S.rel, "converged": ok,
                "device_seconds": dev_ms / 1e3, "launches": launches}

    if "rbsor" in methods:
        out["rbsor"] = timed(pic.SOLVER_RBSOR, omega)
        out["rbsor"]["omega"] = omega
    if "pcg" in methods:
        out["pcg"] = timed(pic.SOLVER_PCG)
    lp = pic.LearnedPreconditioner(W)
    lp.reset()
    if "learned_start" in methods:
        out["learned_start"] = timed(pic.SOLVER_LEARNED)
    if "learned" not in methods:
        W.close()
        return out
    # online training on (rho, phi) pairs of the run's other solves
    W.synchronize()
    t0 = time.perf_counter()
    lp.collect(True)
    S = pic.PotentialSolver(W, 200000, 1e-6, pic.SOLVER_LEARNED)
    for k in range(4):
        W.rho = blob_rho(nn, seed + 101 + k)
        W.phi = phi0
        S.solve()
    lp.collect(False)
    cal_before, cal_after = lp.calibrate()  # level gains, judged by validation solves
    rounds = [{"calibration": True, "val_iters_before": cal_before, "val_iters_after": cal_after, "kept": True}]
    for k in range(max(1, train_steps // 100)):
        loss, before, after, kept = lp.train(100, lr=1e-3 / (1 + k), pair_every=0)
        rounds.append({"loss": loss, "val_iters_before": before, "val_iters_after": after, "kept": kept})
    W.synchronize()
    train_s = time.perf_counter() - t0
    W.rho = rho_test
    out["learned"] = timed(pic.SOLVER_LEARNED)
    out["learned"]["training"] = {"pair_solves": 4, "steps": train_steps, "seconds": train_s, "rounds": rounds}
    for m in ("pcg", "rbsor"):
        if m in out:
            out["speedup_vs_" + m] = out[m]["seconds"] / out["learned"]["seconds"]
    W.close()
    return out


def dsmc_bench(pic, ncell, ppc=16, calls=10, cpu=True):
    """DSMC_MEX (VHS O-O collisions, Interactions.cpp:143-284) on ncell^3 cells of 1 mm^3 with ppc
    particles per cell (n = 1e21 m^-3, 300 K, dt = 1 us): time per call (sort + collisions) after
    three calls, candidate pairs and collisions per call, the collision kernel's roofline at 32 B per
    particle (its velocities read and written once; pairs re-read them from L1/L2), and the
    reference's serial algorithm (the oracle's port) on a 32^3-cell sample of the same density."""
    L = ncell * 1e-3
    W = pic.World(ncell + 1, ncell + 1, ncell + 1, (0.0, 0.0, 0.0), (L, L, L))
    W.set_boundaries((1, 1, 1), (1,) * 6, (0.0,) * 6)
    W.setTime(1e-6, 1 << 20)
    mpw0 = 1e21 * 1e-9 / ppc
    n = ncell ** 3 * ppc
    a = pic.Species("O", 16 * AMU, 0.0, W, mpw0, capacity=n + 4096)
    a.loadUniform((0, 0, 0), (L, L, L), n, 300.0, mpw0, 0.0, seed=1)
    D = pic.DSMC_MEX(a, W, seed=3)
    for _ in range(3):
        D.apply(1e-6)
    W.synchronize()
    W.timing(True)
    W.timing_reset()
    s0 = D.stats()
    t0 = time.perf_counter()
    for _ in range(calls):
        D.apply(1e-6)
    W.synchronize()
    wall = time.perf_counter() - t0
    s1 = D.stats()
    coll_ms, coll_l = W.timer("dsmc")
    sort_ms, _ = W.timer("sort")
    W.timing(False)
    W.close()
    pairs = (s1["pairs"] - s0["pairs"]) / calls
    peak, peak_kind = measured_peak()
    kernel_s = coll_ms / 1e3 / calls
    achieved = 32.0 * n / kernel_s / 1e9
    out = {"cells": ncell ** 3, "particles": n, "calls": calls, "ms_per_call": wall * 1e3 / calls,
           "device_ms_per_call": (coll_ms + sort_ms) / calls, "collide_ms_per_call": coll_ms / calls,
           "sort_ms_per_call": sort_ms / calls, "pairs_per_call": pairs,
           "collisions_per_call": (s1["collisions"] - s0["collisions"]) / calls,
           "pairs_per_s": pairs / (wall / calls), "sigma_v_rel_max": s1["sigma_v_rel_max"],
           "roofline": {"bound": "hbm", "kernel": "k_dsmc", "achieved": achieved, "peak": peak, "unit": "GB/s",
                        "frac": achieved / peak, "peak_source": peak_kind,
                        "algorithmic_bytes_per_launch": 32.0 * n}}
    if cpu:
        import oracle as O

        port = O.Port()
        nc = 32
        g = port.grid((nc + 1,) * 3, (0, 0, 0), (nc * 1e-3,) * 3)
        q = port.dsmc_params(g, 16 * AMU, 16 * AMU, mpw0)
        rng = np.random.default_rng(2)
        m = nc ** 3 * ppc
        p = np.zeros(m, O.PARTICLE)
        p["pos"] = rng.uniform(0, nc * 1e-3, (m, 3)) * 0.999999
        p["vel"] = rng.normal(size=(m, 3)) * np.sqrt(KB * 300.0 / (16 * AMU))
        p["w"] = mpw0
        mt = port.mt(5)
        sv = 1e-14
        for _ in range(2):  # the majorant settles
            _, _, sv = port.dsmc_ref(g, q, mt, p, None, 1e-6, sv)
        t0 = time.perf_counter()
        tot, k = 0, 0
        while time.perf_counter() - t0 < 3.0:
            _, pr, sv = port.dsmc_ref(g, q, mt, p, None, 1e-6, sv)
            tot += pr
            k += 1
        dt_cpu = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": tot / dt_cpu, "unit": "candidate pairs/s", "cores": 1, "kind": "port",
                               "sample": "%d^3 cells, %d particles, %d calls (sort included)" % (nc, m, k)}
    return out


def run_e2e(pic, wl, args, rank):
    """Host-facing run: particles uploaded from pinned FP64 host buffers through the C ABI,
    K steps, and the conservation diagnostics read back every step."""
    import torch

    n = wl["n_each"]
    rng = np.random.default_rng(7 + rank)
    L = wl["L"]

    def host_arrays(T, mass):
        pos = torch.empty((n, 3), dtype=torch.float64, pin_memory=True)
        vel = torch.empty((n, 3), dtype=torch.float64, pin_memory=True)
        w = torch.empty((n,), dtype=torch.float64, pin_memory=True)
        chunk = 10_000_000
        for a in range(0, n, chunk):
            b = min(n, a + chunk)
            pos[a:b] = torch.from_numpy(rng.uniform((0, 0, 0.3 * L[2]), (L[0], L[1], 0.7 * L[2]), (b - a, 3)))
            vel[a:b] = torch.from_numpy(rng.normal(size=(b - a, 3)) * np.sqrt(KB * T / mass))
            w[a:b] = torch.from_numpy(rng.lognormal(np.log(wl["w_mean"]) - 0.125, 0.5, b - a))
        return pos, vel, w

    he = host_arrays(2.0 * EV_K, ME)
    hi = host_arrays(0.03 * EV_K, 32 * AMU)
    nn = wl["nn"]
    W = pic.World(*nn, (0.0, 0.0, 0.0), L)
    W.set_boundaries((1, 1, 0), (1,) * 6, (0, 0, 0, 0, 0.0, wl["V"]))
    W.setTime(wl["dt"], 1 << 30)
    cap = int(n * 1.25) + 4096
    bound = cap * wl["w_mean"] * 400.0
    e = pic.Species("e-", ME, -QE, W, wl["w_mean"], capacity=cap, weight_bound=bound)
    i = pic.Species("O2+", 32 * AMU, QE, W, wl["w_mean"], capacity=cap, weight_bound=bound)
    E, S = sigma_tables()
    pic.MC_MEX_Ionization(e, i, W, wl["n_gas"], 300.0, 32 * AMU, LOTZ["I"], E, S, sigma_ion_kind=1,
                          sigma_ion_params=(LOTZ["A"], LOTZ["b"], LOTZ["c"], 0.0), seed=1)
    Sv = pic.PotentialSolver(W, 20000, 1e-6, pic.SOLVER_LEARNED)
    W.configure_loop(solve_each_step=True, sort_every=SORT_EVERY[0])
    import ctypes as C

    L_ = W._L
    W.synchronize()
    t0 = time.perf_counter()
    marks = {}
    for sp, (pos, vel, w) in ((e, he), (i, hi)):
        rc = L_.pic_species_add_particles(W.handle, sp.id, C.c_void_p(pos.data_ptr()), C.c_void_p(vel.data_ptr()),
                                          C.c_void_p(w.data_ptr()), None, n, 1)
        if rc:
            raise RuntimeError("upload failed %d" % rc)
        sp.sortIndexes()  # cell order, as after a sort step of the loop
    W.synchronize()
    marks["upload_and_sort"] = time.perf_counter() - t0
    Sv.solve(raise_on_fail=True)
    Sv.computeEF()
    W.synchronize()
    marks["initial_solve"] = time.perf_counter() - t0 - marks["upload_and_sort"]
    diag = np.zeros(5)
    for _ in range(args.steps):
        W.step()
        for sp in (e, i):
            L_.pic_species_sums(W.handle, sp.id, diag.ctypes.data_as(C.c_void_p))
    W.synchronize()
    t = time.perf_counter() - t0
    marks["steps"] = t - marks["upload_and_sort"] - marks["initial_solve"]
    parts = e.getNumParticles() + i.getNumParticles()
    W.close()
    h2d = 2 * n * (7 * 8)  # pos, vel, w in FP64
    return {"value": parts * args.steps / t, "unit": "particle-steps/s",
            "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": 2 * 5 * 8 * 512,
            "seconds": t, "seconds_by_part": marks}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="large", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-sample", type=int, default=1_000_000)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--poisson", type=int, default=256, help="n of the n^3 Poisson time-to-1e-6 case (0: skip)")
    ap.add_argument("--poisson-methods", default="rbsor,pcg,learned_start,learned",
                    help="comma list of the Poisson solves to time (rbsor, pcg, learned_start, learned)")
    ap.add_argument("--sort-every", type=int, default=20, help="steps between the loop's sort checks")
    ap.add_argument("--dsmc", type=int, default=128, help="n of the n^3-cell DSMC_MEX case (0: skip)")
    ap.add_argument("--dsmc-only", action="store_true", help="run only the DSMC_MEX case and print it")
    ap.add_argument("--poisson-only", action="store_true",
                    help="run only the Poisson time-to-1e-6 comparison (the second metric) and print it")
    args = ap.parse_args()
    SORT_EVERY[0] = args.sort_every
    if args.warmup < 3:
        args.warmup = 3
    wl = WORKLOADS[args.workload]
    rank, ws, local = dist_init()
    if args.poisson_only:
        if rank == 0 and args.impl != "reference":
            pic = importlib.import_module(PKG)
            print(json.dumps({"metric": "Poisson time-to-1e-6 FP64 residual", "unit": "s",
                              "poisson_time_to_1e-6": poisson_bench(pic, args.poisson or 256,
                                                                    methods=args.poisson_methods.split(","))}),
                  flush=True)
        return
    if args.dsmc_only:
        if rank == 0 and args.impl != "reference":
            pic = importlib.import_module(PKG)
            print(json.dumps({"metric": "DSMC_MEX candidate pairs/s", "unit": "pairs/s",
                              "dsmc": dsmc_bench(pic, args.dsmc or 128, cpu=not args.no_cpu)}), flush=True)
        return
    if args.impl == "reference":
        run_reference(args, wl, rank, ws)
    else:
        run_gpu(args, wl, rank, ws, local)
    if ws > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
