"""Autotuner for the kernel's tunable knobs (cwgpu_tuning).

The knobs are bin thresholds. In the Myers-Miller stage, frames with at most
`tiny_m` rows and `tiny_n` columns are solved one frame per lane, the rest by
warp-wide sweeps. Across pairs, those whose first sequence has at most
`short_rows` residues run in the short-pair kernel (4 rows per lane), the rest
in the long-pair kernel (8 rows per lane). The best splits depend on the length
distribution of the workload (short families produce mostly tiny frames, long
ones mostly large), so the tuner times a length-stratified sample of the
workload's pairs: first each tiny-frame candidate, then each short-pair
threshold with the chosen tiny-frame pair, and keeps the fastest. Results never
depend on the knobs, only the time does. Choices are cached per GPU and length
profile in $XDG_CACHE_HOME/clustalw_gb300/tuning.json. $CLUSTALW_GB300_TUNING
("tiny_m,tiny_n,short_rows") overrides both the cache and the search, and is
applied to every new native.Context.

tune_cta() picks the one-CTA-per-pair knobs (cwgpu_cta_tuning) for a launch
with few long pairs: it times the whole launch one warp per pair and one CTA
per pair with 4, 8 and 16 warps, and sets the threshold so that a launch of
this size takes the faster form.
"""
import json
import os
import time

import numpy as np

CANDIDATES = [(0, 0), (16, 8), (16, 16), (32, 12), (32, 16), (64, 16)]
SHORT_ROWS = [0, 64, 128, 192, 256]
ENV_VAR = "CLUSTALW_GB300_TUNING"


def env_override():
    """(tiny_m, tiny_n, short_rows) from $CLUSTALW_GB300_TUNING, e.g. "32,16,128";
    None when it is unset or empty. A malformed value raises ValueError (the
    library itself rejects values outside its ranges)."""
    text = os.environ.get(ENV_VAR, "").strip()
    if not text:
        return None
    parts = [p.strip() for p in text.split(",")]
    if len(parts) != 3:
        raise ValueError(f"{ENV_VAR} must be 'tiny_m,tiny_n,short_rows', got {text!r}")
    return tuple(int(p) for p in parts)


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


def _time_sample(ctx, sample, repeats):
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
    return best


def tune(ctx, lens, pairs, gpu_name="gpu", target_cells=2e10, candidates=CANDIDATES, short_rows=SHORT_ROWS,
         use_cache=True, repeats=2):
    """Pick (tiny_m, tiny_n, short_rows) for this workload on `ctx` (a
    native.Context with matrix, params and sequences set), apply it and return
    (choice, {candidate: seconds})."""
    forced = env_override()
    if forced is not None:
        ctx.set_tuning(*forced)
        return forced, {}
    key = f"{gpu_name}|{length_profile(lens)}"
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            with open(path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
    if use_cache and key in cache and len(cache[key].get("choice", [])) == 3:
        choice = tuple(cache[key]["choice"])
        ctx.set_tuning(*choice)
        return choice, {}
    sample = stratified_sample(lens, pairs, target_cells)
    lens = np.asarray(lens)
    first = lens[np.asarray(sample).reshape(-1, 2)[:, 0]] if len(sample) else lens[:0]
    rows0 = ctx.get_tuning()[2]
    timings = {}
    for cand in candidates:
        ctx.set_tuning(cand[0], cand[1], rows0)
        timings[(cand[0], cand[1], rows0)] = _time_sample(ctx, sample, repeats)
    tiny = min(timings, key=timings.get)[:2]
    # A threshold only matters if it splits the sample differently from the others.
    seen = set()
    for r in short_rows:
        split = int((first <= r).sum())
        if split in seen and r != rows0:
            continue
        seen.add(split)
        cand = (tiny[0], tiny[1], r)
        if cand not in timings:
            ctx.set_tuning(*cand)
            timings[cand] = _time_sample(ctx, sample, repeats)
    choice = min(timings, key=timings.get)
    ctx.set_tuning(*choice)
    if use_cache:
        cache[key] = {"choice": list(choice), "seconds": {",".join(map(str, c)): s for c, s in timings.items()}}
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            with open(path, "w") as f:
                json.dump(cache, f, indent=1)
        except OSError:
            pass
    return choice, timings


CTA_WARPS = [4, 8, 16]
CTA_MAX_TIMED_PAIRS = 4096  # above this one warp per pair fills the GPU; nothing is timed


def tune_cta(ctx, lens, pairs, warps=CTA_WARPS, repeats=2):
    """Pick cwgpu_cta_tuning (max_pairs, warps, large_rows) for launches of
    `pairs` on `ctx` (matrix, params and sequences set), apply it and return
    (choice, {(max_pairs, warps): seconds}). Only the long pairs (first
    sequence longer than short_rows) can take the CTA form; a launch with more
    than CTA_MAX_TIMED_PAIRS of them keeps the current knobs untimed."""
    lens = np.asarray(lens)
    pairs = np.asarray(pairs).reshape(-1, 2)
    short_rows = ctx.get_tuning()[2]
    nlong = int((lens[pairs[:, 0]] > short_rows).sum()) if len(pairs) else 0
    cur = ctx.get_cta_tuning()
    if nlong == 0 or nlong > CTA_MAX_TIMED_PAIRS:
        return cur, {}
    large = cur[2]
    timings = {(0, cur[1]): None}
    ctx.set_cta_tuning(0, cur[1], large)
    timings[(0, cur[1])] = _time_sample(ctx, pairs, repeats)
    for w in warps:
        ctx.set_cta_tuning(nlong, w, large)
        timings[(nlong, w)] = _time_sample(ctx, pairs, repeats)
    best = min(timings, key=timings.get)
    choice = (nlong if best[0] else nlong - 1, best[1], large)
    ctx.set_cta_tuning(*choice)
    return choice, timings
