"""Benchmark of the solver hot path: compartment-steps/s on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl ours|reference]

A "step" is one loop iteration of the reference driver (src/neurite.cpp:224-236:
update + calculate) applied to every tree of the workload.  `value` is whole-job
throughput with the trees resident in HBM (CUDA events on the library's stream around K
steps); `e2e` is the same metric through the public C ABI from host buffers (create =
H2D of every tree, K steps, snapshot of every tree = D2H).  Inputs are larger than L2.

Workloads (synthetic, seeded; see model.py):
  batch-implicit-mixed  4096 random trees, 1e3-1e5 elements log-uniform, implicit backward
                        Euler, FP32 GMRES(20) inner + FP64 refinement to 1e-10 (relative),
                        dt 0.025 ms, stimulus U(0.5, 3) nA, strain U(0, 0.15)
  batch-explicit-mixed  the same tree population, explicit, mixed precision, dt 0.8 dT_crit
  batch-explicit-fp64   as above in plain FP64
  axon-explicit-fp64    the 1 cm squid axon (1002 elements), plain FP64 (single tree)

--impl reference times the oracle port of the reference's CPU solver (no GPU) on the box's
host cores over a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import importlib
import json
import multiprocessing as mp
import os
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "compartment-steps/s"

# DRAM bytes (read + write) per compartment-step of the dominant kernel, from ncu captures
# above L2 (profiles/ gives the commands): the explicit step on 1024 trees (21.9M elements)
# moved 1.394 GB per launch; the implicit launch on 608 trees of 10k elements (6.08M)
# moved 3.720 GB over 3 steps.  The traffic of a full-size step is scaled from these by the
# compartments it processes.
TRAFFIC_PER_ELEMENT_STEP = {"batch-explicit-mixed": 1.394e9 / 21910344,
                            "batch-implicit-mixed": 3.720006e9 / (3 * 6081291)}
WORKLOADS = ("batch-implicit-mixed", "batch-explicit-mixed", "batch-explicit-fp64",
             "axon-explicit-fp64", "myelin-explicit-mixed", "serve")
DEFAULT_WORKLOAD = "batch-implicit-mixed"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=0)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--workload", choices=WORKLOADS, default=DEFAULT_WORKLOAD)
    ap.add_argument("--trees", type=int, default=0, help="override the tree count (probes only)")
    ap.add_argument("--uniform-size", type=int, default=0,
                    help="every tree of about this many elements instead of the log-uniform "
                         "sizes (probes only: a population whose CTAs finish together)")
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--no-cpu-baseline", action="store_true",
                    help="skip the CPU baseline leg (profiling runs)")
    ap.add_argument("--precond", default="tree", choices=("tree", "segment", "jacobi"),
                    help="implicit workloads: GMRES preconditioner")
    ap.add_argument("--no-plain", action="store_true",
                    help="skip the plain-FP64 single-tree comparison run")
    ap.add_argument("--sub-results", choices=("auto", "on", "off"), default="auto",
                    help="also measure the other workloads and attach them in compact form "
                         "(auto: with the default workload on one GPU)")
    ap.add_argument("--autotune", action="store_true",
                    help="run on the launch shape the autotuner picks "
                         "(tuned before the timed regions; default: the automatic shapes)")
    return ap.parse_args()


# ------------------------------------------------------------------ workloads

UNIFORM_SIZE = 0  # --uniform-size (probes only)


def tree_population(count: int, seed: int):
    model = importlib.import_module("168861_gb300.model")
    sizes = model.log_uniform_sizes(count, 1e3, 1e5, seed)
    if UNIFORM_SIZE:
        sizes = [UNIFORM_SIZE] * count
    return [(seed * 7919 + i, int(sizes[i])) for i in range(count)]


def shard(population, rank: int, world: int):
    """Round-robin split of the tree population over ranks: trees are independent, so a
    rank steps its own share with no data exchange (replicas only, weak scaling)."""
    return population[rank::world]


def combine_ranks(dist, device, ms: float, e2e_s: float, n_elem: int, alg_bytes: float):
    """Job-wide figures from the per-rank ones: the slowest rank's device time and
    end-to-end time, the element count and algorithmic bytes summed over ranks.  With
    `dist` None (one process) the inputs come back unchanged."""
    if dist is None:
        return ms, e2e_s, float(n_elem), float(alg_bytes)
    import torch
    t = torch.tensor([ms, e2e_s], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    s = torch.tensor([float(n_elem), float(alg_bytes)], device=device, dtype=torch.float64)
    dist.all_reduce(s)
    return float(t[0]), float(t[1]), float(s[0]), float(s[1])


_POPULATION = {}  # (count, seed, rank, world) -> [(spec, derived)]: built once per process


def build_batch_problems(workload: str, count: int, seed: int, rank: int, world: int):
    pkg = importlib.import_module("168861_gb300")
    model = pkg.model
    key = (count, seed, rank, world)
    if key not in _POPULATION:
        _POPULATION[key] = [(s, pkg.derive(s)) for s in
                            (model.random_tree(seed=tseed, n_target=size)
                             for tseed, size in shard(tree_population(count, seed), rank, world))]
    probs, runs = [], []
    n_elem = 0
    for spec, d in _POPULATION[key]:
        if workload.startswith("batch-explicit"):
            dT = 0.8 * d.dT_crit
        else:
            dT = spec.dt_abs
        p = pkg.ProblemArrays.from_spec(spec, d, dT)
        probs.append(p)
        runs.append((1, spec.num_steps(dT) - 1, spec.init_time, spec.end_input))
        n_elem += spec.n
    return probs, runs, n_elem


def myelin_workload(pkg):
    """The myelinated axon: 200 nodes of Ranvier (1 um, HH at 10x density) between 1 mm
    passive internodes (myelin Cm 0.005 uF/cm^2, Rm x1000), dx 1 um, with a strain ramp
    0 -> 20% over 5 ms on the 5 mm segment in the middle.  Returns (spec, problem, segment),
    dT = 0.8 of the smaller critical step of the unstrained and the fully strained axon."""
    import copy
    spec = pkg.model.myelinated_axon()
    mid = spec.n // 2
    seg = np.arange(mid - 2500, mid + 2500)
    s2 = copy.deepcopy(spec)
    s2.epsilon[seg] = 0.2
    d = pkg.derive(spec)
    dT = 0.8 * min(d.dT_crit, pkg.derive(s2).dT_crit)
    return spec, pkg.ProblemArrays.from_spec(spec, d, dT), seg


def workload_config(workload: str, count: int, precond: str = "tree"):
    if workload == "axon-explicit-fp64":
        return {"workload": "axon-explicit-fp64", "trees": 1, "elements_per_tree": 1002,
                "mode": "explicit", "precision": "fp64", "dt": "0.8 dT_crit = 8e-4 ms"}
    if workload == "myelin-explicit-mixed":
        return {"workload": "myelin-explicit-mixed", "trees": 1,
                "geometry": "200 nodes (1 um, HH x10) + 1 mm internodes, dx 1 um",
                "mode": "explicit", "precision": "FP32 state + FP64 accumulator",
                "strain": "ramp 0 -> 20% over 5 ms on the middle 5 mm",
                "dt": "0.8 of the smaller critical step (unstrained, 20% strained)"}
    cfg = {"workload": workload, "trees": count, "elements_per_tree": "log-uniform 1e3-1e5",
           "depth": "4-12", "branching_prob": "0.6-0.9", "stimulus_nA": "U(0.5,3)",
           "strain": "U(0,0.15)"}
    if workload == "batch-implicit-mixed":
        cfg.update(mode="implicit backward Euler", precision="FP32 GMRES(20) + FP64 refinement",
                   tol="1e-10 relative", dt_ms=0.025,
                   preconditioner={"tree": "exact tree (Hines) factorisation in FP32",
                                   "segment": "segment tridiagonal", "jacobi": "Jacobi"}[precond])
    else:
        cfg.update(mode="explicit", precision=workload.rsplit("-", 1)[1], dt="0.8 dT_crit")
    cfg["l2"] = "inputs larger than L2 (129 MB)"
    return cfg


# ------------------------------------------------------------------ measurement helpers

class ClockSampler:
    """nvidia-smi clocks during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        if not self.proc or not self.path:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9 and f[1].replace(".", "").isdigit():
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(rows[0][2]),
                "samples": len(rows), "reasons": sorted(reasons)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _varies(a) -> bool:
    return len(a) > 1 and bool(np.any(a != a[0]))


def algorithmic_bytes_explicit(probs, precision: str) -> float:
    """Compulsory bytes per explicit step: per compartment the potential (FP64) read and
    written, the gates read and written (FP64, or FP32 in mixed precision), the parent
    index, the coefficients dT/(c_m dX) and 1/(r_a dX) only where the geometry varies
    within a tree, and a channel parameter only where it varies within a tree (uniform
    ones live in a per-tree table).  Passive compartments: potential, index, the
    coefficients where they vary, and W dX, K dX where they vary."""
    fb = 8 if precision == "fp64" else 4
    total = 0.0
    for p in probs:
        n, n_hh = p.num_elem, int(p.struct.num_hh)
        ph, pp = _param_bytes(p, fb)
        total += n_hh * (16 + 6 * fb + 4 + ph) + (n - n_hh) * (16 + 4 + pp)
    return total


def _param_bytes(p, fb: int):
    """Per-compartment parameter bytes the rule counts (where they vary within the tree):
    (HH compartments, passive compartments).  Variation is judged over the compartments a
    step computes: the terminals (the fictitious root and the sealed ends) are copies of
    their neighbours and stream no coefficients."""
    a = p.arrays
    core = np.ones(p.num_elem, bool)
    core[np.asarray(a["terminals"], np.int64)] = False
    geo = 2 * fb if (_varies((a["c_m"] * a["dx"])[core]) or
                     _varies((a["r_a"] * a["dx"])[core])) else 0
    chan = sum(fb for k in ("g_Na", "g_K", "G_L", "E_Na", "E_K", "E_L", "ls_Na", "ls_K")
               if _varies(a[k]))
    passive = core.copy()
    passive[a["hh_elem"]] = False
    wk = 2 * fb if (_varies(a["W"][passive]) or _varies(a["K"][passive])) else 0
    return geo + chan, geo + wk


def algorithmic_bytes_implicit(probs, steps: int, iters, counts):
    """Bytes per implicit step (mixed precision), two ways, from the kernel's own counts of
    its passes over the rows (`Batch.pass_counts`; per instance over `steps` steps).

    rule: the compulsory-traffic rule for an implicit step, per compartment: assembly = HH
      state (FP32 gates r/w 24) + V r 8 + b w 8 + diagonal w 8 + the parameters that vary
      within the tree; plus, per Krylov iteration j, a CSR SpMV (36 B with FP32 values and
      int32 indices at 3 nonzeros per row) and the orthogonalisation, 4 (2 (j + 1) + 1) B;
      plus, per Richardson refinement step (an iteration without orthogonalisation), the
      FP64 SpMV of the residual that checks it (56 B).  It counts no preconditioner and no
      other refinement residual.

    passes: what this kernel's passes must move per row, counted per pass:
      assembly (HH 85 / passive 77 B: rowf 1, V^n 8, V^n-1 8, c_m dX/dT 8, 1/(r_a dX) 8,
        class index 4, gates r/w 24 or W dX, K dX 16; writes diagonal 8, c 4, b 8, W_0 4),
      tree factorisation 21 (slot row 4, flag 1, conductance 4, c 4; 1/pivot 4, e 4),
      each later FP64 residual 37 (b 8, rowf 1, diagonal 8, conductance 8, x 8; W_0 4),
      each preconditioner application 38 (two passes: slot rows and flags twice 10, e twice
        8, 1/pivot 4, input 4, eliminated side 4 + 4, output 4),
      each Arnoldi step j: SpMV 17 (rowf, c, conductance, Z_j, y) + products and
        update 8 (j + 1) + 8, and its share of the solution update 4,
      each solution update 17 (rowf 1, V r/w 16), plus V^n 8 once per step for x0.
    Neighbour values come from cache; topology records of branch rows and the
    per-instance tables are left out of both.  Returns (rule, passes) in bytes per step."""
    rule = passes = 0.0
    for k, p in enumerate(probs):
        n, n_hh = p.num_elem, int(p.struct.num_hh)
        ph, pp = _param_bytes(p, 4)
        asm_rule = n_hh * (24 + 24 + ph) + (n - n_hh) * (24 + pp)
        I, B = float(iters[k]), float(counts["basis"][k])
        R = float(counts["richardson"][k]) if "richardson" in counts else 0.0
        rule += asm_rule + n * (36 * I + 4 * (2 * B + I) + 56 * R) / steps
        asm = n_hh * 85 + (n - n_hh) * 77
        per_run = (37 * counts["residuals"][k] + 38 * counts["applies"][k]
                   + (17 + 8 + 4) * I + 8 * B + 17 * counts["xupdates"][k])
        passes += asm + n * (21 + 8) + n * per_run / steps
    return rule, passes


def plain_fp64_single(pkg, torch):
    """The plain FP64 single-tree GPU path of the depth-10 random binary tree workload
    (2047 branches, ~2.6e5 elements, Crank-Nicolson as that workload specifies): the drop-in
    solver in FP64 (GMRES(30), tolerance 1e-10 relative), 10 timed steps."""
    spec = pkg.model.random_binary_tree(depth=10, seed=2)
    p = pkg.ProblemArrays.from_spec(spec, pkg.derive(spec))
    s = pkg.SolverIm(p, precision="fp64", restart=30, tol=1e-10, tol_mode="rel", precond="tree",
                     max_iter=2000, scheme="cn")
    s.run(1, 4, spec.init_time, spec.end_input)
    stream = torch.cuda.ExternalStream(s.stream())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    s.run(4, 14, spec.init_time, spec.end_input)
    e1.record(stream)
    e1.synchronize()
    ms = e0.elapsed_time(e1)
    st = s.stats()
    s.close()
    return {"value": spec.n * 10 / (ms / 1e3), "unit": METRIC, "elements": spec.n, "steps": 10,
            "ms_per_step": ms / 10, "config": "random binary tree depth 10 (2047 branches), dx 1 um, "
            "HH everywhere, Crank-Nicolson, FP64 GMRES(30) tree-preconditioned, tol 1e-10 rel, "
            "dt 0.01 ms", "krylov_iters": int(st.krylov_iters)}


# ------------------------------------------------------------------ our arm

def run_ours(args, rank: int, world: int, dist, wl: str, extras: bool = True, steps: int = 0,
             autotune: bool | None = None):
    """One workload on our arm; returns its JSON line (rank 0) or None.  extras: the plain
    FP64 comparison (implicit) and the CPU baseline leg.  autotune: run on the shape the
    autotuner picks (default: --autotune)."""
    import torch
    pkg = importlib.import_module("168861_gb300")
    local = int(os.environ.get("LOCAL_RANK", 0))
    count = args.trees or (4096 if wl.startswith("batch") else 1)
    precision = "fp64" if wl.endswith("fp64") else "mixed"
    implicit = wl.startswith("batch-implicit")
    K = steps or args.steps or (40 if implicit else 2048)
    W = max(3, args.warmup)

    t_build = time.time()
    strained = None
    if wl == "axon-explicit-fp64":
        spec = pkg.model.straight_axon(dtf=0.8)
        d = pkg.derive(spec)
        dT = pkg.step_size(spec, d)
        probs = [pkg.ProblemArrays.from_spec(spec, d, dT)]
        runs = [(1, spec.num_steps(dT) - 1, spec.init_time, spec.end_input)]
        n_elem = spec.n
    elif wl == "myelin-explicit-mixed":
        spec, p, seg = myelin_workload(pkg)
        probs = [p]
        runs = [(1, spec.num_steps(p.dT) - 1, spec.init_time, spec.end_input)]
        n_elem = spec.n
        strained = (spec, seg)
    else:
        probs, runs, n_elem = build_batch_problems(wl, count, args.seed, rank, world)
    t_build = time.time() - t_build
    opts = dict(precision=precision)
    if implicit:
        opts.update(krylov="gmres", restart=20, tol=1e-10, tol_mode="rel", precond=args.precond,
                    max_iter=1000)
    mode = pkg._lib.NRT_IMPLICIT_BE if implicit else pkg._lib.NRT_EXPLICIT
    launch_shape = "automatic"
    if (args.autotune if autotune is None else autotune):  # outside every timed region
        rest = {k: v for k, v in opts.items() if k != "precision"}
        tuned = importlib.import_module(pkg.__name__ + ".autotune").tune(probs, mode, precision,
                                                                         runs=runs, **rest)
        opts.update(tuned["options"])
        launch_shape = {"tuned": tuned["options"], "candidates": tuned["candidates"],
                        "seconds_per_step": tuned["times"]}
    # loop ranges long enough for warm-up + timed steps
    runs = [(a, max(b, a + W + K + 1), c, d_) for a, b, c, d_ in runs]

    # ---- end to end through the public API (host buffers in, host buffers out), after an
    # untimed warm-up of the same calls on the first few trees (module loading, first use
    # of the allocator and the host thread pool), as the device leg has its warm-up steps
    wb = pkg.Batch(probs[:min(len(probs), 16)], mode=mode, **opts)
    wb.set_runs(runs[:min(len(probs), 16)])
    if strained:
        wb.set_strain(0, strained[0], strained[1], 0.0, 0.2, 0.0, 5e-3)
    wb.advance(W)
    wb.snapshot_all()
    wb.close()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    b = pkg.Batch(probs, mode=mode, **opts)
    b.set_runs(runs)
    if strained:
        b.set_strain(0, strained[0], strained[1], 0.0, 0.2, 0.0, 5e-3)
    b.advance(K)
    outs = b.snapshot_all()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    h2d = sum(sum(a.nbytes for a in p.arrays.values()) for p in probs)
    d2h = sum(o.nbytes for o in outs)
    b.close()
    del outs

    # ---- device-resident throughput
    b = pkg.Batch(probs, mode=mode, **opts)
    b.set_runs(runs)
    if strained:
        b.set_strain(0, strained[0], strained[1], 0.0, 0.2, 0.0, 5e-3)
    stream = torch.cuda.ExternalStream(b.stream())
    b.advance(W)
    b.synchronize()
    it0 = b.instance_stats()["iters"] if implicit else None
    pc0 = b.pass_counts() if implicit else None
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        l0 = pkg.kernel_launches()
        ev0.record(stream)
        b.advance(K)
        ev1.record(stream)
        ev1.synchronize()
        launches = pkg.kernel_launches() - l0  # the library's own count of its launches
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1)
    st = b.stats()
    krylov = None
    if implicit:
        ist = b.instance_stats()
        pc1 = b.pass_counts()
        per = (ist["iters"] - it0) / K
        krylov = {"iters_per_tree_step_mean": float(per.mean()), "iters_per_tree_step_max": float(per.max()),
                  "nonconverged_steps": int(ist["nonconverged"].sum()),
                  "max_last_residual": float(ist["last_residual"].max())}
    passes = None
    if implicit:
        counts = {key: pc1[key] - pc0[key] for key in pc1}
        alg, passes = algorithmic_bytes_implicit(probs, K, ist["iters"] - it0, counts)
        krylov.update({key + "_per_tree_step": float(v.mean()) / K for key, v in counts.items()})
    else:
        alg = algorithmic_bytes_explicit(probs, precision)
    ms, e2e_s, n_all, alg_all = combine_ranks(dist, "cuda", ms, e2e_s, n_elem, alg)
    value = n_all * K / (ms / 1e3)
    e2e_value = n_all * K / e2e_s
    peak, peak_kind = measured_peaks()
    # per GPU: the job's algorithmic bytes over the slowest rank's time, divided by N
    achieved = alg_all * K / (ms / 1e3) / 1e9 / world
    per_el = TRAFFIC_PER_ELEMENT_STEP.get(wl)
    traffic = per_el * n_all / world if per_el else None  # per GPU and step, like achieved
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
            "algorithmic_bytes_per_step": alg_all,
            "traffic_note": "DRAM bytes per step from an ncu capture above L2 (1024 trees "
                            "explicit, 608 trees of 10k elements implicit), scaled by compartments"
                            if per_el else None}
    roof_passes = None
    if passes is not None:
        # the same kernel time against the bytes its own passes must move (preconditioner
        # and refinement residuals included), counted from the kernel's pass counters
        _, _, _, passes_all = combine_ranks(dist, "cuda", ms, e2e_s, 0, passes)
        a2 = passes_all * K / (ms / 1e3) / 1e9 / world
        roof_passes = {"bound": "hbm", "achieved": a2, "peak": peak, "unit": "GB/s",
                       "frac": a2 / peak, "bytes_per_step": passes_all}
    line = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world, "steps": K,
        "warmup": W, "ms_per_step": ms / K, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if precision == "fp64" else "f32+f64",
        "data": "synthetic (seeded random trees)",
        "config": {**workload_config(wl, count, args.precond), "launch_shape": launch_shape},
        "elements": n_all,
        "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": h2d / K,
                "d2h_bytes_per_step": d2h / K, "seconds": e2e_s},
        "roofline": roof, "roofline_passes": roof_passes, "gpu_launches": launches,
        "clocks": clk.summary(),
        "build_seconds": t_build,
        "krylov": krylov,
    }
    b.close()
    if rank == 0 and extras:
        if implicit and not args.no_plain:
            try:
                line["plain_fp64_single"] = plain_fp64_single(pkg, torch)
                line["speedup_vs_plain_fp64_single"] = value / line["plain_fp64_single"]["value"]
            except Exception as exc:
                line["plain_fp64_single"] = {"value": None, "error": repr(exc)[:300]}
        if not args.no_cpu_baseline:
            try:
                line["cpu_baseline"] = cpu_baseline(wl, args.seed, count)
            except Exception as exc:  # the GPU line is still reported
                line["cpu_baseline"] = {"value": None, "error": repr(exc)[:300]}
            if implicit:
                # the same CPU with the exact tree solve instead of the reference's
                # unpreconditioned GMRES: splits the GPU's lead into algorithm and hardware
                try:
                    line["cpu_tree_solve"] = cpu_baseline(wl, args.seed, count, linsolve=0)
                    line["speedup_vs_cpu_tree_solve"] = value / line["cpu_tree_solve"]["value"]
                except Exception as exc:
                    line["cpu_tree_solve"] = {"value": None, "error": repr(exc)[:300]}
    return line if rank == 0 else None


# ------------------------------------------------------------------ serving

def serve_requests(count: int, seed: int):
    """Request stream: Poisson arrivals (mean 2000 req/s), drawn in turn from the four
    workload shapes:
      - explicit 1 cm / 1002-element squid axons (dt 0.8 dT_crit), simulated U(10, 100) ms;
      - implicit random trees of the batched population (1e3-1e5 elements, dt 0.025 ms),
        simulated U(10, 100) ms;
      - implicit random binary trees of the Crank-Nicolson workload's shape (depth 6-9,
        dx 1 um, 2 nA at the root, dt 0.01 ms), simulated U(10, 100) ms, stepped with the
        server's implicit settings;
      - explicit myelinated axons of that workload's shape (4-10 nodes of Ranvier, 1 mm
        internodes, dx 1 um), simulated U(0.5, 2) us: their internode step is ~5e-11 s, so
        10 ms would be 2e8 steps.
    Returns (gap to the previous arrival, problem, implicit, run) per request."""
    pkg = importlib.import_module("168861_gb300")
    model = pkg.model
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / 2000.0, size=count)
    out = []
    sizes = model.log_uniform_sizes(count, 1e3, 1e5, seed + 1)
    for q in range(count):
        kind = q % 4
        if kind == 0:
            spec = model.straight_axon(dtf=0.8, tspan=rng.uniform(10.0, 100.0) * 1e-3)
            d = pkg.derive(spec)
            dT, implicit = pkg.step_size(spec, d), False
        elif kind == 1:
            spec = model.random_tree(seed=seed * 31 + q, n_target=int(sizes[q]),
                                     tspan=rng.uniform(10.0, 100.0) * 1e-3)
            d = pkg.derive(spec)
            dT, implicit = spec.dt_abs, True
        elif kind == 2:
            spec = model.random_binary_tree(depth=int(rng.integers(6, 10)), seed=seed * 37 + q,
                                            tspan=rng.uniform(10.0, 100.0) * 1e-3)
            d = pkg.derive(spec)
            dT, implicit = spec.dt_abs, True
        else:
            spec = model.myelinated_axon(n_nodes=int(rng.integers(4, 11)))
            d = pkg.derive(spec)
            dT, implicit = 0.8 * d.dT_crit, False
            spec.tspan = rng.uniform(0.5, 2.0) * 1e-6
        p = pkg.ProblemArrays.from_spec(spec, d, dT)
        out.append((float(gaps[q]), p, implicit,
                    (1, spec.num_steps(dT) - 1, spec.init_time, spec.end_input)))
    return out


SERVE_IMPLICIT = dict(restart=20, tol=1e-10, tol_mode="rel", max_iter=1000)


def serve_plain_fp64(pkg, reqs, precond: str):
    """The plain FP64 per-request path on the same arrival stream: one request at a time in
    arrival order through the drop-in solvers (SolverEx / SolverIm in FP64, the implicit
    ones with the served tolerance), each run as a whole.  Latency = completion - arrival."""
    t0 = time.perf_counter()
    arrive, lat, work = 0.0, [], 0.0
    for gap, p, imp, run in reqs:
        arrive += gap
        now = time.perf_counter() - t0
        if now < arrive:
            time.sleep(arrive - now)
        if imp:
            s = pkg.SolverIm(p, precision="fp64", precond=precond, **SERVE_IMPLICIT)
        else:
            s = pkg.SolverEx(p, precision="fp64")
        s.run(*run)
        s.snapshot()
        s.close()
        lat.append(time.perf_counter() - t0 - arrive)
        work += p.num_elem * max(0, run[1] - run[0])
    wall = time.perf_counter() - t0
    lat = np.array(lat) * 1e3
    return {"value": work / wall, "unit": METRIC, "p50_ms": float(np.percentile(lat, 50)),
            "p99_ms": float(np.percentile(lat, 99)), "max_ms": float(lat.max()),
            "seconds": wall, "path": "one request at a time, FP64 drop-in solvers"}


def run_serve(args, rank: int, world: int, dist, count: int = 0, plain: bool = True):
    """The serving workload; returns its JSON line (rank 0) or None."""
    import torch
    pkg = importlib.import_module("168861_gb300")
    count = count or args.trees or 64
    # each rank serves its own share of the arrival stream (one server per GPU)
    reqs = shard(serve_requests(count, args.seed), rank, world)
    ex = dict(precision="mixed")
    im = dict(precision="mixed", precond=args.precond, **SERVE_IMPLICIT)
    # warm-up: one small request of each kind through a throwaway server
    w = pkg.Server(budget_bytes=8 << 30, explicit_opts=ex, implicit_opts=im)
    for gap, p, imp, run in reqs[:4]:
        w.submit(p, imp, run[0], min(run[1], run[0] + 16), run[2], run[3])
    w.drain()
    w.close()
    srv = pkg.Server(budget_bytes=64 << 30, chunk_steps=64, max_wait_us=200,
                     explicit_opts=ex, implicit_opts=im)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", 0))) as clk:
        l0 = pkg.kernel_launches()
        t0 = time.perf_counter()
        nxt = t0
        for gap, p, imp, run in reqs:
            nxt += gap
            dt = nxt - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            srv.submit(p, imp, *run)
        srv.drain()
        wall = time.perf_counter() - t0
        launches = pkg.kernel_launches() - l0
    st = srv.stats()
    srv.close()
    work = float(st.compartment_steps)
    p50, p99, pmax = st.p50_ms, st.p99_ms, st.max_ms
    h2d = sum(sum(a.nbytes for a in r[1].arrays.values()) for r in reqs)
    d2h = sum(r[1].num_elem * 8 for r in reqs)
    if dist:
        t = torch.tensor([wall, p50, p99, pmax], device="cuda", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        s_ = torch.tensor([work, float(h2d), float(d2h)], device="cuda", dtype=torch.float64)
        dist.all_reduce(s_)
        wall, p50, p99, pmax = (float(x) for x in t)
        work, h2d, d2h = (float(x) for x in s_)
    if rank != 0:
        return None
    line = {"metric": "serve compartment-steps/s", "value": work / wall,
            "unit": "compartment-steps/s", "n_gpus": world, "steps": count, "warmup": 4,
            "ms_per_step": wall * 1e3 / count, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded requests)",
            "config": {"workload": "serve", "requests": count, "arrivals": "Poisson 2000/s",
                       "mix": "in turn: explicit 1 cm axon; implicit random tree 1e3-1e5; "
                              "implicit random binary tree depth 6-9; explicit myelinated axon "
                              "4-10 nodes (mixed precision; implicit GMRES(20) + FP64 "
                              "refinement to 1e-10)",
                       "sim_time": "U(10,100) ms (myelinated axons U(0.5,2) us)"},
            "p50_ms": p50, "p99_ms": p99, "max_ms": pmax,
            "batches": int(st.batches_created), "completed": int(st.completed),
            "gpu_launches": launches, "clocks": clk.summary(),
            "e2e": {"value": work / wall, "unit": "compartment-steps/s",
                    "h2d_bytes_per_step": h2d / count, "d2h_bytes_per_step": d2h / count}}
    if plain and world == 1:
        try:
            line["plain_fp64_per_request"] = serve_plain_fp64(pkg, reqs, args.precond)
            line["speedup_vs_plain_fp64_per_request"] = line["value"] / line["plain_fp64_per_request"]["value"]
        except Exception as exc:
            line["plain_fp64_per_request"] = {"value": None, "error": repr(exc)[:300]}
    return line


# ------------------------------------------------------------------ CPU (reference) arm

def _oracle_job(job):
    """One oracle run in a worker process (spawned; no CUDA here).  Implicit: linsolve 2 is
    the reference's method (unpreconditioned GMRES(150) to 1e-14), 0 the exact tree solve."""
    wl, tseed, size, steps, linsolve = job
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    model = importlib.import_module("168861_gb300.model")
    if wl == "axon-explicit-fp64":
        spec = model.straight_axon(dtf=0.8)
    elif wl == "myelin-explicit-mixed":  # a scaled axon (20 nodes), as the oracle can cover
        spec = model.myelinated_axon(n_nodes=20)
    else:
        spec = model.random_tree(seed=tseed, n_target=size)
    orc = O.Oracle()
    d = orc.derive(spec)
    t0 = time.perf_counter()
    if wl.startswith("batch-implicit"):
        orc.implicit_run(spec, d, spec.dt_abs, 1, 1 + steps, linsolve=linsolve)
    else:
        dT = O.spec_dT(spec, d.dT_crit) if wl == "axon-explicit-fp64" else 0.8 * d.dT_crit
        orc.explicit_run(spec, d, dT, 1, 1 + steps)
    return spec.n * steps, time.perf_counter() - t0


def _sample_jobs(wl: str, seed: int, count: int, cores: int, linsolve: int = 2):
    """About 10-20 s of CPU work spread over `cores` processes."""
    if wl == "axon-explicit-fp64":
        return [(wl, 0, 1002, 12000, 2)] * cores, "1002-element axon, 12000 steps per process"
    if wl == "myelin-explicit-mixed":
        return ([(wl, 0, 0, 200000, 2)] * cores,
                "20-node myelinated axon (~2e4 elements, no strain ramp), 2e5 steps per process")
    pop = tree_population(count, seed)
    if wl.startswith("batch-implicit") and linsolve == 0:
        # the exact tree (Hines) solve: the first trees of the population, as drawn
        pick = pop[: 2 * cores]
        jobs = [(wl, s, n, 200, 0) for s, n in pick]
        return jobs, (f"first {len(jobs)} trees of the workload, 200 steps each, exact tree "
                      "(Hines) solve in FP64")
    if wl.startswith("batch-implicit"):
        # unpreconditioned GMRES(150) to 1e-14 (the reference's solve) on the smallest trees,
        # which converge fastest per compartment: a conservative (CPU-favouring) sample
        per = 10
        pick = sorted(pop, key=lambda t: t[1])[: 2 * cores]
        what = "smallest"
    else:
        per = 600
        pick = pop[: 2 * cores]
        what = "first"
    jobs = [(wl, s, n, per, 2) for s, n in pick]
    return jobs, f"{what} {len(jobs)} trees of the workload, {per} steps each"


def _warm(_):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.Oracle()
    importlib.import_module("168861_gb300.model")
    return os.getpid()


def cpu_baseline(wl: str, seed: int, count: int, linsolve: int = 2):
    """The oracle port timed on the host cores (one process per core, spawned, warmed).
    Implicit workloads: linsolve 2 runs the reference's method, 0 the exact tree solve."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    jobs, sample = _sample_jobs(wl, seed, count, cores, linsolve)
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        pool.map(_warm, range(cores))
        t0 = time.perf_counter()
        res = pool.map(_oracle_job, jobs, chunksize=1)
        wall = time.perf_counter() - t0
    work = sum(r[0] for r in res)
    return {"value": work / wall, "unit": METRIC, "cores": cores, "kind": "port",
            "sample": sample, "seconds": wall}


def run_reference(args, rank: int, world: int):
    if rank != 0:
        return
    wl = args.workload
    count = args.trees or (4096 if wl.startswith("batch") else 1)
    K = args.steps or 3
    W = max(3, args.warmup)
    vals = []
    cb = None
    for it in range(W + K):
        cb = cpu_baseline(wl, args.seed, count)
        if it >= W:
            vals.append(cb["value"])
    v = float(np.mean(vals))
    cb["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": METRIC, "n_gpus": world,
            "steps": K, "warmup": W, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded random trees)",
            "config": workload_config(wl, count), "cpu_baseline": cb,
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def compact(line: dict) -> dict:
    """The figures of a workload's line that a sub-result keeps."""
    keep = ("value", "unit", "ms_per_step", "steps", "elements", "p50_ms", "p99_ms", "max_ms",
            "completed", "plain_fp64_per_request", "speedup_vs_plain_fp64_per_request")
    out = {k: line[k] for k in keep if k in line}
    out["workload"] = line["config"]["workload"]
    if line.get("roofline"):
        r = line["roofline"]
        out["roofline"] = {k: r[k] for k in ("achieved", "peak", "unit", "frac") if k in r}
    if isinstance(line.get("e2e"), dict):
        out["e2e"] = line["e2e"]["value"]
    out["clocks"] = line.get("clocks")
    return out


SUB_WORKLOADS = ("batch-implicit-mixed-tuned", "batch-explicit-mixed", "axon-explicit-fp64",
                 "myelin-explicit-mixed", "serve")


def main():
    global UNIFORM_SIZE
    args = parse()
    UNIFORM_SIZE = args.uniform_size
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", args.gpus))
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0))))
    if args.workload == "serve":
        line = run_serve(args, rank, world, dist)
    else:
        line = run_ours(args, rank, world, dist, args.workload)
        subs = args.sub_results == "on" or (
            args.sub_results == "auto" and args.workload == DEFAULT_WORKLOAD and world == 1
            and not args.trees and not args.steps and not args.uniform_size)
        if subs:
            # the other workloads the results quote, each measured as its own line would be
            # (without a CPU leg), kept in compact form
            sub = {}
            for wl in SUB_WORKLOADS:
                try:
                    if wl == "serve":
                        l2 = run_serve(args, rank, world, dist)
                    elif wl.endswith("-tuned"):  # the headline on the autotuner's launch shape
                        l2 = run_ours(args, rank, world, dist, wl[: -len("-tuned")],
                                      extras=False, autotune=True)
                    else:
                        l2 = run_ours(args, rank, world, dist, wl, extras=False)
                    sub[wl] = compact(l2) if l2 else None
                    if l2 and isinstance(l2["config"].get("launch_shape"), dict):
                        sub[wl]["launch_shape"] = l2["config"]["launch_shape"]
                except Exception as exc:  # the headline line is still reported
                    sub[wl] = {"error": repr(exc)[:300]}
            if line is not None:
                line["sub_results"] = sub
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
