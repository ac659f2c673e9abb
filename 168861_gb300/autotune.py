"""Launch-shape autotuner for batches of trees (`Batch(..., autotune=True)`).

The explicit steps have launch shapes that do not change their results (each element's
arithmetic is the same whatever the grid):
- the mixed step: staged tiles (`tiled`) with 1 .. 4 persistent CTAs per SM
  (`tile_ctas_per_sm`), or one thread per element (`tiled=0`) with 64 .. 256 threads per
  block (`step_threads`);
- the FP64 step: 32 .. 256 threads per block.

Which one is fastest depends on the tree sizes, the share of HH compartments and the
device, so `tune` times every candidate on the workload itself, in a batch of its own, so
the caller's state is never touched. The explicit steps tile the elements, and a sample
stands for the workload: every k-th tree (the workload's mix of sizes), about
`sample_elements` compartments. The implicit kernel gives each tree to one CTA, and its best
CTA count depends on the whole population: on a quarter of the 4096-tree batch, 2 CTAs per
SM ran fastest (the largest trees, which set a sample's time, share their SMs less), while on
the whole batch 4 per SM beat 2 by a third (throughput over all trees). So the implicit
kernel is timed on the whole workload, over fewer steps. It keeps the fastest. Results are cached in a JSON file
per device, mode, precision and workload size, so a workload is tuned once per machine.

The implicit block-per-instance kernel (batches) has one shape-only knob: how many of its
persistent CTAs run per SM (`tile_ctas_per_sm`, 1 .. 4; its register budget allows 4). Each
instance is one CTA's from start to end, so the trees come out bit for bit the same. Its other
tunable, the GMRES restart length, changes the iteration count but leaves the answer within
the solve tolerance; it is searched (with every CTA count) only when `restarts` is given.
"""
from __future__ import annotations

import json
import math
import os
import time

from . import _lib

CACHE_ENV = "NRT_AUTOTUNE_CACHE"
DEFAULT_CACHE = os.path.join(os.path.expanduser("~"), ".cache", "neurite_gb300_autotune.json")


def candidates(mode: int, precision: str, restarts=None) -> list[dict]:
    """The launch shapes searched for a workload, as option overrides."""
    if mode == _lib.NRT_EXPLICIT:
        if precision == "mixed":
            return ([{"tiled": True, "tile_ctas_per_sm": c} for c in (1, 2, 3, 4)] +
                    [{"tiled": False, "step_threads": t} for t in (64, 128, 256)])
        return [{"step_threads": t} for t in (32, 64, 128, 256)]
    shapes = [{"tile_ctas_per_sm": c} for c in (2, 3, 4)]
    if restarts:
        return [{"restart": int(r), **s} for r in restarts for s in shapes]
    return shapes


def choose(times: list[float]) -> int:
    """Index of the fastest candidate (the first one on a tie); non-finite times lose."""
    best = None
    for i, t in enumerate(times):
        if t is None or not math.isfinite(t) or t <= 0:
            continue
        if best is None or t < times[best]:
            best = i
    if best is None:
        raise ValueError("no candidate could be timed")
    return best


def sample_indices(problems, sample_elements: float, min_trees: int = 1) -> list:
    """Every k-th tree's index from the first: about sample_elements compartments, and at
    least min_trees trees (all of them when there are no more)."""
    n = len(problems)
    total = sum(p.num_elem for p in problems)
    k = max(1, math.ceil(total / max(sample_elements, 1)))
    k = min(k, max(1, n // max(min_trees, 1)))
    return list(range(0, n, k))


def sample(problems, sample_elements: float, min_trees: int = 1) -> list:
    """The trees of sample_indices."""
    return [problems[i] for i in sample_indices(problems, sample_elements, min_trees)]


def workload_key(device: str, mode: int, precision: str, problems, restarts=None) -> str:
    """Cache key: the device, the stepper, and the workload's tree count and total size
    (each rounded to a power of two)."""
    n = sum(p.num_elem for p in problems)
    b = lambda x: int(round(math.log2(max(x, 1))))  # noqa: E731
    mode_s = "explicit" if mode == _lib.NRT_EXPLICIT else "implicit"
    tail = "" if not restarts else "|restart" + ",".join(str(int(r)) for r in restarts)
    return f"{device}|{mode_s}|{precision}|trees2^{b(len(problems))}|elements2^{b(n)}{tail}"


def device_name(device: int = -1) -> str:
    try:
        import torch
        d = torch.cuda.current_device() if device < 0 else device
        return torch.cuda.get_device_name(d)
    except Exception:  # no torch or no device: one shared key
        return "cuda"


def time_candidate(problems, mode: int, precision: str, overrides: dict, steps: int,
                   warmup: int, repeats: int = 2, runs=None, **opts) -> float:
    """Seconds per step of a batch of `problems` built with `overrides`: the best of
    `repeats` timings of `steps` steps after `warmup` steps, with the device idle on both
    sides of each timing.  runs: each tree's (i_begin, i_end, init_time, end_input), whose
    stimulus windows the timed steps use (the loop ranges are lengthened to cover them);
    None: no stimulus."""
    from .solver import Batch
    b = Batch(problems, mode, precision=precision, **{**opts, **overrides})
    try:
        total = warmup + repeats * steps
        if runs is None:
            b.set_runs([(1, 1 + total, 0.0, -1.0)] * len(problems))
        else:
            b.set_runs([(a, max(e, a + total), t0, t1) for a, e, t0, t1 in runs])
        b.advance(warmup)
        b.synchronize()
        best = math.inf
        for _ in range(repeats):
            t0 = time.perf_counter()
            b.advance(steps)
            b.synchronize()
            best = min(best, time.perf_counter() - t0)
        return best / steps
    finally:
        b.close()


def _load(path: str) -> dict:
    try:
        with open(path) as f:
            d = json.load(f)
        return d if isinstance(d, dict) else {}
    except (OSError, ValueError):
        return {}


def _store(path: str, cache: dict) -> None:
    try:
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        tmp = path + f".{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(cache, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass  # a read-only home: tune again next time


def tune(problems, mode: int = _lib.NRT_EXPLICIT, precision: str = "fp64", *,
         steps: int = 0, warmup: int = 3, sample_elements: float = 0, min_trees: int = 1,
         restarts=None, cache: str | None = None, timer=None, device_key: str | None = None,
         runs=None, **opts) -> dict:
    """The fastest launch shape for `problems`: {"options": overrides, "key": cache key,
    "times": seconds per step of each candidate (None when served from the cache),
    "candidates": the shapes searched}.

    timer(problems, mode, precision, overrides) -> seconds per step replaces the device
    timing (tests use it); device_key replaces the device's name in the cache key.
    steps: timed steps per repeat (0: 64 explicit, 16 implicit); sample_elements: the sample's
    size (0: 4e6 compartments explicit, the whole workload implicit); min_trees: the sample's
    fewest trees.  runs: the trees' loop ranges and stimulus windows (as Batch.set_runs), so
    the timed steps see the workload's stimulus (None: none).  `opts` are the caller's other
    options (make_options keywords), kept fixed."""
    cands = candidates(mode, precision, restarts)
    dev = device_key if device_key is not None else device_name(int(opts.get("device", -1)))
    key = workload_key(dev, mode, precision, problems, restarts)
    path = cache if cache is not None else os.environ.get(CACHE_ENV, DEFAULT_CACHE)
    stored = _load(path) if path else {}
    hit = stored.get(key)
    if isinstance(hit, dict) and hit.get("options") in cands:
        return {"options": dict(hit["options"]), "key": key, "times": None, "candidates": cands}
    if len(cands) == 1:
        return {"options": dict(cands[0]), "key": key, "times": [None], "candidates": cands}
    explicit = mode == _lib.NRT_EXPLICIT
    steps = steps or (64 if explicit else 16)
    sample_elements = sample_elements or (4e6 if explicit else math.inf)
    idx = sample_indices(problems, sample_elements, min_trees)
    part = [problems[i] for i in idx]
    part_runs = [runs[i] for i in idx] if runs is not None else None
    if timer is None:
        def timer(ps, m, prec, ov):
            return time_candidate(ps, m, prec, ov, steps, warmup, runs=part_runs, **opts)
    times = []
    for ov in cands:
        try:
            times.append(float(timer(part, mode, precision, ov)))
        except _lib.NeuriteError:
            times.append(None)  # a shape this device cannot launch
    best = cands[choose(times)]
    if path:
        stored = _load(path)  # another process may have written meanwhile
        stored[key] = {"options": best, "seconds_per_step": dict(
            (json.dumps(c, sort_keys=True), t) for c, t in zip(cands, times))}
        _store(path, stored)
    return {"options": dict(best), "key": key, "times": times, "candidates": cands}
