"""Benchmark of the GB300 PIC + DSMC step loop: particle-steps per second on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload large|discharge|mid|ensemble]
    python bench.py --impl reference ...   (the reference algorithm on the host cores)

A step is one iteration of the ch4/v3 time loop on the workload's synthetic discharge:
electron-impact collisions against the O2 background, leapfrog push with trilinear gather and
fixed-point deposition for both species, charge density, Poisson solve warm-started from the
last potential to ||b - L phi|| <= 1e-6 min(||b||, ||rho/eps0||) in float-float refinement (the
residual relative to the space-charge part of b as well, so that the electrode term cannot hide
an unresolved space-charge potential), E = -grad(phi), a counting sort by cell when 2 % of a
species moved (checked every 20 steps) and a merge pass every 20 steps.  value = particles pushed
per step / device step time (CUDA events on the library's stream).  Inputs (particles, fields)
are resident in HBM and larger than L2.  e2e runs the same K steps through the C ABI from pinned
host buffers: the particle upload and a per-step read of the conservation diagnostics
(Outputs.cpp:143-182) are inside its clock.  Beside the headline (the large discharge) the line
carries the electrode discharge (64x64x256), the 64-instance ensemble, and the Poisson
time-to-tolerance comparisons at 256^3 (blob charge) and 128^3 (a charge-density snapshot of the
discharge), each with a CPU baseline.  One JSON line on stdout (rank 0).
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
STOP = ["charge"]  # Poisson stopping rule of the loop and of the time-to-tolerance cases
WARM = ["extrapolate"]  # start of the loop's warm solves: "previous" phi or "extrapolate"d in time
WARM_JACOBI = [0]  # Jacobi-PCG iterations a warm learned solve runs first (measured best with training)
STOP_TEXT = {"charge": "||b - L phi|| <= 1e-6 min(||b||, ||rho/eps0||)", "rhs": "||b - L phi|| <= 1e-6 ||b||"}


def stop_rule(pic):
    return pic.STOP_REL_CHARGE if STOP[0] == "charge" else pic.STOP_REL_RHS


def loop_solver(pic, W):
    """The loop's Poisson solver: learned-preconditioned flexible CG, the stopping rule and warm start."""
    S = pic.PotentialSolver(W, 20000, 1e-6, pic.SOLVER_LEARNED, stop=stop_rule(pic))
    S.setWarmStart(pic.WARM_EXTRAPOLATE if WARM[0] == "extrapolate" else pic.WARM_PREVIOUS)
    S.setWarmJacobi(WARM_JACOBI[0])
    return S


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
    S_ = loop_solver(pic, W)
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
    S_ = loop_solver(pic, W)
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
        if self.index < 0:  # not sampled
            return self
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
LOOP_POISSON = os.path.join(ROOT, "profiles", "loop_poisson_iterations.json")


def measured_loop_poisson(key):
    """Poisson work per step of the GPU loop on a workload (inner FP32 iterations and FP64
    residual passes), measured by this benchmark's GPU arm and recorded in
    profiles/loop_poisson_iterations.json; the reference arm charges the same work."""
    with open(LOOP_POISSON) as f:
        rec = json.load(f)[key]
    return rec


class CpuLoop:
    """The FP64 port of the reference loop (oracle/pic_oracle.c, a restatement of ch4/v3) on the
    host cores, one step at a time on a bounded sample of a workload.

    Particle work (collisions, push, deposit) runs on `sample` electrons + `sample` ions and is
    scaled linearly to the workload's particle count; the electron push uses host_cores-1
    threads like the reference's ThreadPool, the ion push, deposit and collisions are serial as
    in the reference.  Field work runs on the full grid (one instance grid, times the instance
    count, for the ensemble): charge density, Poisson work at a given count of Jacobi-PCG
    iterations and FP64 residual passes (one of each timed per step and scaled), and E."""

    def __init__(self, wl, sample=1_000_000, seed=3):
        import oracle as O

        self.O = O
        self.port = O.Port()
        self.wl = wl
        ens = wl.get("kind") == "ensemble"
        self.instances = wl["instances"] if ens else 1
        nn, L = wl["nn"], wl["L"]
        self.nn = nn
        self.g = self.port.grid(nn, (0, 0, 0), L, periodic=(1, 1, 0))
        self.kind = self.port.node_kinds(self.g, 1)
        self.nv = int(np.prod(nn))
        self.threads = max(1, (os.cpu_count() or 2) - 1)
        rng = np.random.default_rng(seed)
        if ens:
            nI = wl["instances"]
            counts = np.exp(np.random.default_rng(1).uniform(np.log(wl["n_range"][0]), np.log(wl["n_range"][1]),
                                                             nI)).astype(np.int64)
            self.n_full = 2 * int(counts.sum())
            w_mean = wl["density"] * L[0] * L[1] * 0.4 * L[2] / float(np.median(counts))
            V, n_gas = wl["V"][1], wl["n_gas"][1]
        else:
            self.n_full = 2 * wl["n_each"]
            w_mean, V, n_gas = wl["w_mean"], wl["V"], wl["n_gas"]
        self.V = V
        n = min(sample, self.n_full // 2)
        self.n = n

        def make(T, mass):
            p = np.zeros(int(n * 1.2) + 1024, O.PARTICLE)
            p["pos"][:n] = rng.uniform((0, 0, 0.3 * L[2]), (L[0], L[1], 0.7 * L[2]), (n, 3))
            p["vel"][:n] = rng.normal(size=(n, 3)) * np.sqrt(KB * T / mass)
            p["w"][:n] = rng.lognormal(np.log(w_mean) - 0.125, 0.5, n)
            return p

        self.ele, self.ion = make(2.0 * EV_K, ME), make(0.03 * EV_K, 32 * AMU)
        self.eid = np.arange(len(self.ele), dtype=np.uint64)
        self.iid = np.arange(len(self.ion), dtype=np.uint64) + (1 << 40)
        E, S = sigma_tables()
        self.cp = self.port.coll_params(E, S, 32 * AMU, LOTZ["I"], 1, (0.0, LOTZ["b"], LOTZ["c"]), sig_A=LOTZ["A"],
                                        n_neutral=n_gas, T_neutral=300.0)
        self.ef = np.zeros((self.nv, 3))
        self.ne, self.ni = n, n
        self.s = 0
        self.phi = np.zeros(self.nv)
        fixed = np.nonzero(self.kind == O.FIXED)[0]
        self.phi[fixed] = np.where(fixed // (nn[0] * nn[1]) == nn[2] - 1, V, 0.0)

    def particle_step(self, electron_threads=None):
        """Collisions, pushes and deposits of the sample; seconds, and of that the electron push."""
        O, port, wl = self.O, self.port, self.wl
        th = self.threads if electron_threads is None else electron_threads
        t0 = time.perf_counter()
        _, _, self.ne, self.ni = port.mcc_background(self.g, self.cp, self.ele, self.eid, self.ne, self.ion, self.iid,
                                                      self.ni, wl["dt"], 1, self.s)
        t1 = time.perf_counter()
        self.ne = port.push(self.g, self.ele[:self.ne], self.ef, wl["dt"], -QE, ME, ids=self.eid[:self.ne],
                            threads=th)
        t2 = time.perf_counter()
        self.ni = port.push(self.g, self.ion[:self.ni], self.ef, wl["dt"], QE, 32 * AMU, ids=self.iid[:self.ni])
        self.de = port.number_density(self.g, self.ele[:self.ne])
        self.di = port.number_density(self.g, self.ion[:self.ni])
        t3 = time.perf_counter()
        self.s += 1
        return t3 - t0, t2 - t1

    def iteration_seconds(self, rho):
        """Seconds of one Jacobi-PCG iteration of the port on the full grid: the difference of a
        3-iteration and a 1-iteration solve from the same start (the set-up cancels), timed once."""
        if getattr(self, "t_iter", None) is None:
            ts = []
            for its in (1, 3):
                phi = self.phi.copy()
                t0 = time.perf_counter()
                self.port.solve_fpcg(self.g, self.kind, phi, rho, 1e-30, its)
                ts.append(time.perf_counter() - t0)
            self.t_iter = max((ts[1] - ts[0]) / 2, 1e-9)
        return self.t_iter

    def step(self, inner, refine):
        """One sampled step; the estimated seconds of the full workload's step."""
        O, port = self.O, self.port
        t_part, _ = self.particle_step()
        per_particle = t_part / (self.ne + self.ni)
        t0 = time.perf_counter()
        rho = QE * (self.di - self.de)
        t_rho = time.perf_counter() - t0
        t_iter = self.iteration_seconds(rho)
        t0 = time.perf_counter()
        port.residual(self.g, self.kind, self.phi, rho)  # one FP64 residual pass
        t_res = time.perf_counter() - t0
        t0 = time.perf_counter()
        self.ef = port.compute_ef(self.g, self.phi)
        t_ef = time.perf_counter() - t0
        field = (t_rho + inner * t_iter + refine * t_res + t_ef) * self.instances
        return {"seconds": self.n_full * per_particle + field, "ns_per_particle": per_particle * 1e9,
                "t_iter": t_iter, "t_res": t_res, "field": field}

    def describe(self, inner, refine, steps, rec):
        nn = self.nn
        grid = f"{nn[0]}x{nn[1]}x{nn[2]}" + (f" (x{self.instances} instances)" if self.instances > 1 else "")
        return (f"per step: {self.n} e- + {self.n} O2+ (collisions, push with {self.threads} threads, deposit: "
                f"{rec['ns_per_particle']:.1f} ns/particle-step, scaled to {self.n_full} particles); charge density, "
                f"{inner:.2f} Jacobi-PCG iterations ({rec['t_iter']:.3f} s each, timed once as the difference of 3- and "
                f"1-iteration solves) and {refine:.2f} FP64 residual passes ({rec['t_res']:.3f} s each, timed every "
                f"step) -- the GPU loop's measured Poisson work per step -- and E on the full {grid} grid; "
                f"{steps} steps timed")


def cpu_baseline(wl, inner, refine, sample=1_000_000, steps=1):
    """The CPU port on `steps` sampled steps of the workload, and on one thread for the electron push."""
    loop = CpuLoop(wl, sample=sample)
    loop.particle_step()  # warm-up
    recs = [loop.step(inner, refine) for _ in range(steps)]
    t = sum(r["seconds"] for r in recs)
    value = loop.n_full * steps / t
    # the single-core figure: the electron push on one thread (the rest is serial already)
    t_mt = loop.particle_step()[1]
    t1 = loop.particle_step(electron_threads=1)[1]
    extra = (t1 - t_mt) / (loop.ne + loop.ni) * loop.n_full
    single = loop.n_full / (t / steps + extra)
    return {"value": value, "unit": "particle-steps/s", "cores": loop.threads, "kind": "port",
            "sample": loop.describe(inner, refine, steps, recs[-1]), "single_thread_value": single,
            "seconds_per_step": t / steps}


def run_reference(args, wl, rank, ws):
    if rank != 0:
        return
    rec = measured_loop_poisson(args.workload)
    inner, refine = rec["inner_per_step"], rec["refinements_per_step"]
    loop = CpuLoop(wl, sample=args.cpu_sample)
    for _ in range(args.warmup):
        loop.particle_step()  # untimed warm-up steps (particle work only)
    recs = [loop.step(inner, refine) for _ in range(args.steps)]
    t = sum(r["seconds"] for r in recs)
    value = loop.n_full * args.steps / t
    cpu = {"value": value, "unit": "particle-steps/s", "cores": loop.threads, "kind": "port",
           "sample": loop.describe(inner, refine, args.steps, recs[-1])}
    line = {
        "metric": "particle-steps/s", "value": value, "unit": "particle-steps/s", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": wl["name"], "poisson_inner_per_step": inner, "poisson_refinements_per_step": refine,
                   "poisson_work_source": rec.get("source", "")},
        "cpu_baseline": cpu,
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------
def measure_loop(pic, args, wl, rank, ws, local, clocks=True):
    """K timed steps of the loop on a workload (after the initial solve, the autotuner and W
    warm-up steps): throughput, the roofline of the dominant kernel group, the Poisson work per
    step and the final solve's norms.  Returns (result dict, world, species) with the world open."""
    import torch

    ensemble = wl.get("kind") == "ensemble"
    W, e, i, M, S = (setup_ensemble if ensemble else setup_world)(pic, wl, seed=1 + rank)
    assert S.solve(raise_on_fail=True)  # initial vacuum + space-charge field (main.cpp:172-173)
    S.computeEF()
    tuned = W.autotune()  # launch shapes measured on this world's data (outside the timed region)
    lp = pic.LearnedPreconditioner(W)
    training = None
    if args.train:
        # online training on the run's own (residual, correction) pairs: the warm-up steps' solves
        # are collected, then the level gains are calibrated and gradient rounds run on those
        # pairs, each round kept only if the validation solve (the latest pair's residual) needs
        # fewer iterations; outside the timed region, its time reported
        lp.collect(True)
    for _ in range(args.warmup):
        W.step()
    if args.train:
        lp.collect(False)
        W.synchronize()
        t0 = time.perf_counter()
        cal_before, cal_after = lp.calibrate()
        rounds = [{"calibration": True, "val_iters_before": cal_before, "val_iters_after": cal_after, "kept": True}]
        for k in range(args.train_rounds):
            loss, before, after, kept = lp.train(100, lr=args.train_lr / (1 + k), pair_every=1)
            rounds.append({"loss": loss, "val_iters_before": before, "val_iters_after": after, "kept": kept})
        W.synchronize()
        training = {"pairs_from_steps": args.warmup, "lr": args.train_lr, "seconds": time.perf_counter() - t0, "rounds": rounds}
        for _ in range(2):  # the loop's warm start settles on the trained preconditioner
            W.step()
    trained_weights = lp.weights() if args.train else None
    W.synchronize()
    W.timing(True)
    W.timing_reset()
    st0 = S.stats()
    n0 = e.getNumParticles() + i.getNumParticles()
    launches0 = W.launches()
    coll0 = M.stats()
    barrier(ws)
    W.synchronize()
    with ClockSampler(local if clocks else -1) as clk:
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
    norms = S.norms()
    groups = {}
    for name in ("push_deposit", "mcc", "compact", "rho", "poisson", "efield", "sort", "merge"):
        ms, nl = W.timer(name)
        groups[name] = dict(ms=ms, launches=nl)
    parts_per_step = 0.5 * (n0 + n1)
    value = aggregate(parts_per_step * args.steps, step_ms / 1e3, ws)
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
        # per inner iteration 56 B per node for the learned-preconditioned CG (CG 40, fine level 14,
        # coarse levels 2) -- the loop's warm solves run no Jacobi iterations first unless asked,
        # which count 40 B -- and 24 B per node per FP64 refinement
        "poisson": (56.0 if WARM_JACOBI[0] == 0 else 40.0) * nv * inner + 24.0 * nv * refine,
        "efield": 24.0 * nv * args.steps,
        "rho": (2 * 20.0 + 4.0) * nv * args.steps,
    }
    kernels = {}
    for name, b_ in algo.items():
        ms = groups[name]["ms"]
        if ms > 0:
            kernels[name] = dict(share=ms / step_ms, achieved_gbs=b_ / (ms / 1e3) / 1e9, ms_per_step=ms / args.steps)
    dom = max(kernels, key=lambda k: kernels[k]["share"])
    launches_dom = max(1, groups[dom]["launches"])
    achieved = algo[dom] / (groups[dom]["ms"] / 1e3) / 1e9
    traffic = roofline_traffic().get(dom)
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind,
            "traffic": traffic * algo[dom] / launches_dom if traffic else None,
            "algorithmic_bytes_per_launch": algo[dom] / launches_dom}
    coll = {k: coll1[k] - coll0[k] for k in coll1}
    res = {
        "value": value, "ms_per_step": step_ms / args.steps, "wall_s": wall, "gpu_launches": launches,
        "parts_per_step": parts_per_step, "roofline": roof, "kernels": kernels,
        "groups_ms_per_step": {k: v["ms"] / args.steps for k, v in groups.items()},
        "inner_per_step": inner / args.steps, "refinements_per_step": refine / args.steps,
        "collisions_per_step": coll["collisions"] / args.steps, "ionizations_per_step": coll["ionizations"] / args.steps,
        # how much of b the space charge carries, and the final residual against both scales
        "poisson_norms": {"rho_over_b": norms["charge"] / norms["b"] if norms["b"] > 0 else None,
                          "residual_rel_b": norms["r"] / norms["b"] if norms["b"] > 0 else None,
                          "residual_rel_charge": norms["r"] / norms["charge"] if norms["charge"] > 0 else None},
        "autotuned": tuned, "clocks": clk.summary() if clocks else None, "training": training,
        "trained_weights": trained_weights,
    }
    return res, W, (e, i)


def run_gpu(args, wl, rank, ws, local):
    pic = importlib.import_module(PKG)
    ensemble = wl.get("kind") == "ensemble"
    res, W, _ = measure_loop(pic, args, wl, rank, ws, local)
    W.close()
    # e2e: same loop through the C ABI from pinned host buffers (upload + per-step diagnostics)
    e2e = None if ensemble else run_e2e(pic, wl, args, rank, weights=res.pop("trained_weights"),
                                        shapes=res["autotuned"])
    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline(wl, res["inner_per_step"], res["refinements_per_step"], sample=args.cpu_sample)
        cpu.pop("seconds_per_step", None)
    extra = {}
    poisson = None
    poisson128 = None
    dsmc = None
    if rank == 0 and args.extra and args.workload == "large":
        extra, snap = extra_workloads(pic, args, rank, ws, local)
        if args.poisson > 0 and snap is not None:
            poisson128 = poisson_bench(pic, (128, 128, 128), WORKLOADS["discharge"]["L"],
                                       WORKLOADS["discharge"]["V"], rho=snap, cpu=not args.no_cpu,
                                       methods=args.poisson_methods.split(","),
                                       rho_name="charge-density snapshot of the electrode discharge after its "
                                                "timed steps, trilinearly resampled onto 128^3 nodes")
    if rank == 0 and args.poisson > 0:
        n = args.poisson
        poisson = poisson_bench(pic, (n, n, n), (0.04, 0.04, 0.04), 1000.0, cpu=not args.no_cpu,
                                methods=args.poisson_methods.split(","))
    if rank == 0 and args.dsmc > 0:
        dsmc = dsmc_bench(pic, args.dsmc, cpu=not args.no_cpu)
    line = {
        "metric": "particle-steps/s", "value": res["value"], "unit": "particle-steps/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": wl["name"],
                   "grid": list(wl["nn"]) + ([wl["instances"]] if ensemble else []),
                   "particles_per_step": res["parts_per_step"],
                   "poisson": "flexible CG with the learned multilevel preconditioner, FP32 iterations in "
                              "float-float refinement, warm start: " + WARM[0] + "; stop: " + STOP_TEXT[STOP[0]],
                   "collisions_per_step": res["collisions_per_step"],
                   "ionizations_per_step": res["ionizations_per_step"],
                   "poisson_inner_per_step": res["inner_per_step"],
                   "poisson_refinements_per_step": res["refinements_per_step"],
                   "poisson_norms": res["poisson_norms"],
                   "poisson_training": res["training"],
                   "sort_every": SORT_EVERY[0],
                   "l2": "inputs larger than L2 (particles %.1f GB)" % (res["parts_per_step"] * 36 / 1e9),
                   "merging": "every %d steps, cells above %d particles" % (MERGE_EVERY, MERGE_MIN),
                   "parallelism": "replicas" if ws > 1 else "1 GPU",
                   "autotuned": res["autotuned"]},
        "wall_s": res["wall_s"],
        "gpu_launches": res["gpu_launches"],
        "roofline": res["roofline"],
        "push_deposit_gbs": res["kernels"].get("push_deposit", {}).get("achieved_gbs"),
        "kernels": res["kernels"],
        "groups_ms_per_step": res["groups_ms_per_step"],
        "cpu_baseline": cpu,
        "e2e": e2e,
        "workloads": extra or None,
        "poisson_time_to_1e-6": poisson,
        "poisson_128_discharge_rho": poisson128,
        "dsmc": dsmc,
        "clocks": res["clocks"],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def extra_workloads(pic, args, rank, ws, local):
    """The electrode discharge and the 64-instance ensemble, each K steps after W warm-up steps
    with its roofline and CPU baseline; returns them and the discharge's final charge density."""
    out = {}
    snap = None
    for key in ("discharge", "ensemble"):
        wl = WORKLOADS[key]
        res, W, _ = measure_loop(pic, args, wl, rank, 1, local, clocks=False)
        if key == "discharge":
            snap = (W.rho.reshape(wl["nn"][2], wl["nn"][1], wl["nn"][0]), wl["nn"])
        W.close()
        cpu = None
        if not args.no_cpu:
            cpu = cpu_baseline(wl, res["inner_per_step"], res["refinements_per_step"], sample=args.cpu_sample)
            cpu.pop("seconds_per_step", None)
        out[key] = {"workload": wl["name"], "metric": "particle-steps/s", "value": res["value"],
                    "unit": "particle-steps/s", "ms_per_step": res["ms_per_step"], "steps": args.steps,
                    "particles_per_step": res["parts_per_step"], "roofline": res["roofline"],
                    "groups_ms_per_step": res["groups_ms_per_step"],
                    "poisson_inner_per_step": res["inner_per_step"],
                    "poisson_refinements_per_step": res["refinements_per_step"],
                    "poisson_norms": res["poisson_norms"], "poisson_training": res["training"],
                    "gpu_launches": res["gpu_launches"],
                    "cpu_baseline": cpu}
    return out, snap


def resample(field, nn_src, nn_dst):
    """Trilinear resampling of a node field ([k][j][i], nn_src nodes) onto nn_dst nodes spanning
    the same box."""
    from scipy.ndimage import map_coordinates

    axes = [np.linspace(0, nn_src[d] - 1, nn_dst[d]) for d in range(3)]
    kk, jj, ii = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    return map_coordinates(field, [kk, jj, ii], order=1, mode="nearest").ravel()


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


def poisson_bench(pic, nn, L, V, rho=None, seed=5, train_steps=300, cpu=True,
                  methods=("rbsor", "pcg", "learned_start", "learned"), rho_name=None):
    """Time to tolerance (the loop's stopping rule at 1e-6) from the Dirichlet-only start on nn
    nodes over the box L, z faces at 0 V / V, periodic x, y; the charge density is a seeded sum of
    Gaussian blobs, or a given snapshot (field [k][j][i], its node counts) resampled onto nn.
    Plain red-black SOR and Jacobi-PCG against the learned multilevel preconditioner, first at its
    starting (BPX) weights, then after online training on the pairs of four solves of other blob
    densities plus white-noise pairs (training time reported separately: it is amortised over a
    run).  The learned solve's roofline counts 56 B per node and iteration (CG 40, fine-level apply
    14, coarse levels 2) and 24 B per node and FP64 residual pass; the CPU baseline is the port's
    FP64 Jacobi-PCG (the reference's method) timed on a few iterations of the same system and
    charged the GPU Jacobi-PCG's iteration count."""
    nn = tuple(int(v) for v in nn)
    W = pic.World(*nn, (0.0, 0.0, 0.0), L)
    W.set_boundaries((1, 1, 0), (1,) * 6, (0, 0, 0, 0, 0.0, V))
    if rho is None:
        rho_test = blob_rho(nn, seed)
        rho_name = "seeded sum of 8-64 Gaussian blobs (amplitude +-1e-3 C/m^3, widths 2-20 cells)"
    else:
        rho_test = resample(rho[0], rho[1], nn)
    W.rho = rho_test
    phi0 = W.phi
    omega = 2.0 / (1.0 + np.sin(np.pi / (max(nn) - 1)))  # optimal SOR weight of the model problem
    out = {"grid": list(nn), "box": list(L), "anode_V": V, "rho": rho_name, "tol": 1e-6, "stop": STOP_TEXT[STOP[0]]}
    nv = int(np.prod(nn))

    def timed(method, w=1.4):
        W.phi = phi0
        S = pic.PotentialSolver(W, 200000, 1e-6, method, omega=w, stop=stop_rule(pic))
        st0 = S.stats()
        W.timing(True)
        W.timing_reset()
        W.synchronize()
        t0 = time.perf_counter()
        ok = S.solve()
        W.synchronize()
        wall = time.perf_counter() - t0
        dev_ms, launches = W.timer("poisson")
        W.timing(False)
        st1 = S.stats()
        nr = S.norms()
        return {"seconds": wall, "iterations": S.iters, "rel": S.rel, "converged": ok,
                "device_seconds": dev_ms / 1e3, "launches": launches,
                "refinements": st1["refinements"] - st0["refinements"],
                "rho_over_b": nr["charge"] / nr["b"] if nr["b"] > 0 else None}

    if "rbsor" in methods:
        out["rbsor"] = timed(pic.SOLVER_RBSOR, omega)
        out["rbsor"]["omega"] = omega
    if "pcg" in methods:
        out["pcg"] = timed(pic.SOLVER_PCG)
    lp = pic.LearnedPreconditioner(W)
    lp.reset()
    if "learned_start" in methods:
        out["learned_start"] = timed(pic.SOLVER_LEARNED)
    if "learned" in methods:
        # online training on (rho, phi) pairs of the run's other solves
        W.synchronize()
        t0 = time.perf_counter()
        lp.collect(True)
        S = pic.PotentialSolver(W, 200000, 1e-6, pic.SOLVER_LEARNED, stop=stop_rule(pic))
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
        r = out["learned"]
        peak, peak_kind = measured_peak()
        achieved = (56.0 * nv * r["iterations"] + 24.0 * nv * r["refinements"]) / r["device_seconds"] / 1e9
        out["learned"]["roofline"] = {"bound": "hbm", "kernel": "learned CG iteration", "achieved": achieved,
                                      "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind}
        for m in ("pcg", "rbsor"):
            if m in out:
                out["speedup_vs_" + m] = out[m]["seconds"] / out["learned"]["seconds"]
    if cpu and "pcg" in out:
        import oracle as O

        port = O.Port()
        g = port.grid(nn, (0, 0, 0), L, periodic=(1, 1, 0))
        kind = port.node_kinds(g, 1)
        phi = np.zeros(nv)
        fixed = np.nonzero(kind == O.FIXED)[0]
        phi[fixed] = np.where(fixed // (nn[0] * nn[1]) == nn[2] - 1, V, 0.0)
        probe = 3
        t0 = time.perf_counter()
        port.solve_fpcg(g, kind, phi, rho_test, 1e-30, probe)
        t_iter = (time.perf_counter() - t0) / probe
        its = out["pcg"]["iterations"]
        out["cpu_baseline"] = {"value": its * t_iter, "unit": "s", "cores": 1, "kind": "port",
                               "sample": "FP64 Jacobi-PCG of the port, %d iterations timed on the same system "
                                         "(%.3f s each), charged the GPU Jacobi-PCG's %d iterations" % (probe, t_iter, its)}
        if "learned" in out:
            out["speedup_vs_cpu_pcg"] = out["cpu_baseline"]["value"] / out["learned"]["seconds"]
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


def run_e2e(pic, wl, args, rank, weights=None, shapes=None):
    """Host-facing run: particles uploaded from pinned FP64 host buffers through the C ABI,
    K steps, and the conservation diagnostics read back every step.  The preconditioner starts
    from `weights` and the launch shapes are `shapes` when given: the ones the device arm trained
    and tuned on this workload, loaded before the clock as a user loads a previous run's trained
    weights and tuned shapes (the training and tuning themselves are reported with the device arm)."""
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
    import ctypes as C

    def one_pass(steps):
        """A fresh world (outside the clock), then: upload of both species from the pinned host
        arrays, sort, initial solve and `steps` loop steps with the diagnostics read every step."""
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
        Sv = loop_solver(pic, W)
        W.configure_loop(solve_each_step=True, sort_every=SORT_EVERY[0], merge_every=MERGE_EVERY, merge_after=0,
                         merge_min=MERGE_MIN)
        if weights is not None:
            pic.LearnedPreconditioner(W).set_weights(weights)
        if shapes is not None:
            W.set_launch_shapes(**shapes)
        L_ = W._L
        W.synchronize()
        t0 = time.perf_counter()
        marks = {}
        # both species through the batch upload: read in place from the pinned arrays, each sorted
        # into cell order (as after a sort step of the loop) while the next one uploads
        W.add_particles_batch([e, i], [he[0], hi[0]], [he[1], hi[1]], [he[2], hi[2]], rewind=True, sort=True)
        W.synchronize()
        marks["upload_and_sort"] = time.perf_counter() - t0
        Sv.solve(raise_on_fail=True)
        Sv.computeEF()
        W.synchronize()
        marks["initial_solve"] = time.perf_counter() - t0 - marks["upload_and_sort"]
        W.timing(True)
        W.timing_reset()
        st0 = Sv.stats()
        diag = np.zeros(5)
        for _ in range(steps):
            W.step()
            for sp in (e, i):
                L_.pic_species_sums(W.handle, sp.id, diag.ctypes.data_as(C.c_void_p))
        W.synchronize()
        t = time.perf_counter() - t0
        marks["steps"] = t - marks["upload_and_sort"] - marks["initial_solve"]
        parts = e.getNumParticles() + i.getNumParticles()
        groups = {name: W.timer(name)[0] / max(steps, 1)
                  for name in ("step", "push_deposit", "poisson", "sums", "sort", "merge")}
        inner = (Sv.stats()["inner"] - st0["inner"]) / max(steps, 1)
        shapes_used = W.launch_shapes()
        W.close()
        return t, parts, marks, groups, inner, shapes_used

    # warm-up pass over the same pinned arrays (the first device reads of freshly pinned pages are
    # slow), then the timed pass
    one_pass(args.warmup)
    t, parts, marks, groups, inner, shapes_used = one_pass(args.steps)
    h2d = 2 * n * (7 * 8)  # pos, vel, w in FP64
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    d2h = 2 * min(8 * sms, 1638) * 5 * 8  # per species the block partials of the five sums
    return {"value": parts * args.steps / t, "unit": "particle-steps/s",
            "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h,
            "seconds": t, "seconds_by_part": marks, "groups_ms_per_step": groups, "poisson_inner_per_step": inner,
            "warmup": "one untimed pass (upload, sort, solve, %d steps) over the same pinned arrays" % args.warmup,
            "preconditioner": "trained weights of the device arm" if weights is not None else "starting weights",
            "launch_shapes": shapes_used}


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
    ap.add_argument("--stop", default="charge", choices=sorted(STOP_TEXT),
                    help="Poisson stopping rule: charge (relative to min(||b||, ||rho/eps0||)) or rhs (to ||b||)")
    ap.add_argument("--warm", default="extrapolate", choices=["extrapolate", "previous"],
                    help="start of the loop's warm Poisson solves: the last phi, or extrapolated in time")
    ap.add_argument("--warm-jacobi", type=int, default=0,
                    help="Jacobi-PCG iterations a warm learned solve runs before the learned preconditioner")
    ap.add_argument("--no-train", dest="train", action="store_false",
                    help="run the loop with the learned preconditioner's starting (BPX) weights")
    ap.add_argument("--train-rounds", type=int, default=3, help="gradient rounds after the level-gain calibration")
    ap.add_argument("--train-lr", type=float, default=1e-4, help="Adam step of the first gradient round")
    ap.add_argument("--no-extra", dest="extra", action="store_false",
                    help="skip the discharge, ensemble and 128^3 snapshot cases beside the headline")
    ap.add_argument("--dsmc", type=int, default=128, help="n of the n^3-cell DSMC_MEX case (0: skip)")
    ap.add_argument("--dsmc-only", action="store_true", help="run only the DSMC_MEX case and print it")
    ap.add_argument("--poisson-only", action="store_true",
                    help="run only the Poisson time-to-1e-6 comparison (the second metric) and print it")
    args = ap.parse_args()
    SORT_EVERY[0] = args.sort_every
    STOP[0] = args.stop
    WARM[0] = args.warm
    WARM_JACOBI[0] = args.warm_jacobi
    if args.warmup < 3:
        args.warmup = 3
    wl = WORKLOADS[args.workload]
    rank, ws, local = dist_init()
    if args.poisson_only:
        if rank == 0 and args.impl != "reference":
            pic = importlib.import_module(PKG)
            n = args.poisson or 256
            print(json.dumps({"metric": "Poisson time-to-1e-6 FP64 residual", "unit": "s",
                              "poisson_time_to_1e-6": poisson_bench(pic, (n, n, n), (0.04, 0.04, 0.04), 1000.0,
                                                                    cpu=not args.no_cpu,
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
