"""Autotuner for the kernel's tunable knobs (cwgpu_tuning).

The knobs are the bin thresholds of the Myers-Miller stage: frames with at
most `tiny_m` rows and `tiny_n` columns are solved one frame per lane, the rest
by warp-wide sweeps. The best split depends on the length distribution of the
workload (short families produce mostly tiny frames, long ones mostly large),
so the tuner times a length-stratified sample of the workload's pairs under
each candidate and keeps the fastest. Results never depend on the knobs, only
the time does. Choices are cached per GPU and length profile in
$XDG_CACHE_HOME/clustalw_gb300/tuning.json.
"""
import json
import os
import time

import numpy as np

CANDIDATES = [(0, 0), (16, 8), (16, 16), (32, 12), (32, 16), (64, 16)]


def _cache_path():
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "clustalw_gb300", "tuning.json")


def length_profile(lens):
    """Signature of a workload: log2-binned length histogram (8 bins)."""
    lens = np.asarray(lens, dtype=np.float64)
    if len(lens) == 0:
        return "empty"
    b = np.clip(np.floor(np.log2(np.maximum(lens, 1))), 0, 15).astype(int)
    h = np.bincount(b, minlength=16)
    top = np.argsort(-h)[:3]
    return "-".join(f"{int(k)}:{int(round(100 * h[k] / len(lens)))}" for k in sorted(top))


def stratified_sample(lens, pairs, target_cells, seed=0):
    """Pairs drawn evenly across the work (n*m) quantiles, up to target_cells of n*m."""
    lens = np.asarray(lens, dtype=np.int64)
    pairs = np.asarray(pairs).reshape(-1, 2)
    work = lens[pairs[:, 0]] * lens[pairs[:, 1]]
    order = np.argsort(work)
    rng = np.random.default_rng(seed)
    nq = 16
    chunks = np.array_split(order, nq)
    mean = max(1.0, float(work.mean()))
    per = max(1, int(target_cells / mean / nq))
    pick = [rng.choice(c, size=min(per, len(c)), replace=False) for c in chunks if len(c)]
    return pairs[np.sort(np.concatenate(pick))]


def tune(ctx, lens, pairs, gpu_name="gpu", target_cells=2e10, candidates=CANDIDATES, use_cache=True, repeats=2):
    """Pick (tiny_m, tiny_n) for this workload on `ctx` (a native.Context with
    matrix, params and sequences set), apply it and return
    (choice, {candidate: seconds})."""
    key = f"{gpu_name}|{length_profile(lens)}"
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            with open(path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
    if use_cache and key in cache:
        choice = tuple(cache[key]["choice"])
        ctx.set_tuning(*choice)
        return choice, {}
    sample = stratified_sample(lens, pairs, target_cells)
    timings = {}
    for cand in candidates:
        ctx.set_tuning(*cand)
        plan = ctx.plan(sample)
        plan.launch()
        plan.results()
        best = float("inf")
        for _ in range(repeats):
            t = time.perf_counter()
            plan.launch()
            plan.results()
            best = min(best, time.perf_counter() - t)
        plan.close()
        timings[cand] = best
    choice = min(timings, key=timings.get)
    ctx.set_tuning(*choice)
    if use_cache:
        cache[key] = {"choice": list(choice), "seconds": {f"{m},{n}": s for (m, n), s in timings.items()}}
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            with open(path, "w") as f:
                json.dump(cache, f, indent=1)
        except OSError:
            pass
    return choice, timings
