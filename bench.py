#!/usr/bin/env python
"""Benchmark of the GB300 full-pairwise distance stage (ClustalW 2.0.11
FullPairwiseAlign::pairwiseAlign, all N(N-1)/2 pairs of a sequence set).

One step = one pass of the stage over one synthetic sequence family
(default: 1000 protein sequences from a root of length 1523, 499,500 pairs,
Gonnet, gap open 10.0, extension 0.1). Metric: GCUPS = sum over pairs of n*m
divided by the time of the step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl ours (default) prints one JSON line with
  value      device-resident form: inputs uploaded and the pair plan built
             before timing; K graph launches timed with CUDA events on the
             launching stream, L2 flushed between steps
  e2e        the same through the C ABI with host buffers: cwgpu_upload_seqs +
             cwgpu_align_pairs (pair list in, distances out) per step
  roofline   INT32-issue roofline of the one kernel (k_pairwise)
  cpu_baseline  the oracle restatement on the host cores, bounded sample
  plain      the one-launch-per-pair GPU form on a sample of the same pairs
  serve      served stream of independent jobs (continuous batching), p50/p99
  guide_tree NJTree::generateTree on the step's own distance matrix: GPU
             kernel (device-resident and through the C ABI) beside the oracle
  quick      FastPairwiseAlign (k-tuple distances) on the same sequences:
             GPU kernel beside the oracle on all host threads
  few_pairs  launches with few long pairs (the reference's 100_1523 set whole
             and as a one-column call, 20 and 6 sequences of ~3000 residues):
             the default dispatch (one CTA per pair below a threshold) beside
             one warp per pair
  reference_shaped  the reference fork's launch shape (128 pairs per launch,
             4 streams) with these kernels, beside the batched form
--impl reference times the reference CPU algorithm (the oracle port; the
reference's own build is not available on the GPU host) on all host threads.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (REPO, os.path.join(REPO, "cuda-clustalw_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

FP64_NOMINAL_TFLOPS = 1.25  # GB300 nominal dense fp64 (an FMA counts 2; the join's criterion has none)
OPS_PER_CELL = 8  # E, F via __viaddmax (2), H-gap term (1), diag add + 3-way max (2), max tracking (2), score (1)
INT32_LANES_PER_SM = 128
ALU_PIPE_LANES_PER_SM = 64  # integer ALU pipe (IMNMX, IADD3, DPX): half the INT32 lane rate

WORKLOADS = {
    # name: (kind, generator args)
    "protein-1000x1523": ("protein", dict(nseqs=1000, root_len=1523)),
    "protein-100x97": ("protein", dict(nseqs=100, root_len=97)),
    "dna-2000x1000": ("dna", dict(nseqs=2000, root_len=1000)),
    "protein-uneven-8x125": ("protein", dict(uneven=True)),
}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="protein-1000x1523", choices=sorted(WORKLOADS))
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="CPU-baseline sample budget")
    ap.add_argument("--plain-pairs", type=int, default=64, help="pairs timed in the plain per-pair form")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--nseqs", type=int, default=0, help="smaller case of the same family model (profiling)")
    ap.add_argument("--device-only", action="store_true", help="time only the device-resident form (profiling)")
    ap.add_argument("--serve-seconds", type=float, default=12.0, help="length of the served arrival process")
    ap.add_argument("--serve-rate", type=float, default=6.0, help="served job arrival rate (jobs/s)")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--serve-only", action="store_true",
                    help="only the served stream, for --serve-seconds (use 600 for the stated configuration)")
    ap.add_argument("--no-tree", action="store_true", help="skip the guide-tree leg")
    ap.add_argument("--no-quick", action="store_true", help="skip the quick k-tuple distance leg")
    ap.add_argument("--no-few", action="store_true",
                    help="skip the few-pair launches and the reference-shaped comparator")
    ap.add_argument("--autotune", action="store_true", help="pick the tiny-frame thresholds for this workload first")
    return ap.parse_args()


def make_workload(name, seed, nseqs=0):
    from clustalw_gb300 import load_matrix, synth

    kind, a = WORKLOADS[name]
    if a.get("uneven"):
        seqs = synth.uneven_protein(8, 125, 30, 2000, seed)
    elif kind == "dna":
        seqs = synth.dna_family(nseqs or a["nseqs"], a["root_len"], seed)
    else:
        seqs = synth.protein_family(nseqs or a["nseqs"], a["root_len"], seed)
    matrix, params = load_matrix(kind)
    return seqs, matrix, params


def nm_cells(seqs, pairs):
    lens = np.array([len(s) for s in seqs], dtype=np.int64)
    return int((lens[pairs[:, 0]] * lens[pairs[:, 1]]).sum())


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


# ---------------------------------------------------------------- clocks


class ClockSampler:
    """nvidia-smi samples (200 ms) of SM clock and throttle reasons while running."""

    FIELDS = (
        "uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
        "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, uuid):
        self.uuid = uuid
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.out,
                stderr=subprocess.DEVNULL,
            )
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.out.close()

    def summary(self):
        if self.proc is None or not self.path:
            return None
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9 or (self.uuid and parts[0] != self.uuid):
                    continue
                try:
                    sms.append(float(parts[1]))
                    maxs.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.path)
        if not sms:
            return None
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": max(maxs), "reasons": sorted(reasons), "samples": len(sms)}


# ---------------------------------------------------------------- CPU legs


def run_cpu(seqs, matrix, params, pairs, threads):
    from oracle import oracle

    t = time.perf_counter()
    res = oracle.align_pairs(seqs, matrix, params, pairs, nthreads=threads)
    return time.perf_counter() - t, res


def cpu_baseline(seqs, matrix, params, pairs, seconds, seed=0):
    """GCUPS of the oracle restatement (port of the reference CPU algorithm) on a
    bounded uniform sample of the workload's pairs, all host threads."""
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(seed)
    lens = np.array([len(s) for s in seqs], dtype=np.int64)
    mean_nm = float((lens[pairs[:, 0]] * lens[pairs[:, 1]]).mean())
    perm = rng.permutation(len(pairs))
    used, total_t, total_c, chunk = 0, 0.0, 0, 4 * threads
    while total_t < 0.9 * seconds and used < len(pairs):
        sample = pairs[np.sort(perm[used : used + chunk])]
        dt, _ = run_cpu(seqs, matrix, params, sample, threads)
        used += len(sample)
        total_t += dt
        total_c += nm_cells(seqs, sample)
        rate = total_c / max(total_t, 1e-9)
        chunk = int(max(threads, min(len(pairs), rate * max(0.5, seconds - total_t) / mean_nm)))
    return {
        "value": total_c / total_t / 1e9,
        "unit": "GCUPS",
        "cores": threads,
        "kind": "port",
        "sample": f"{used} of {len(pairs)} pairs (seeded uniform), {total_t:.1f} s on {threads} threads",
    }


def reference_arm(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    seqs, matrix, params = make_workload(args.workload, args.seed, args.nseqs)
    from clustalw_gb300 import synth

    pairs = synth.all_pairs(len(seqs))
    threads = os.cpu_count() or 1
    rng = np.random.default_rng(12345)
    lens = np.array([len(s) for s in seqs], dtype=np.int64)
    # Calibrate the per-step sample so that all W+K steps take about 2 minutes.
    calib = pairs[rng.choice(len(pairs), size=min(len(pairs), 8 * threads), replace=False)]
    dt, _ = run_cpu(seqs, matrix, params, calib, threads)
    rate = nm_cells(seqs, calib) / max(dt, 1e-6)
    per_step = 120.0 / max(1, args.steps + args.warmup)
    mean_nm = float((lens[pairs[:, 0]] * lens[pairs[:, 1]]).mean())
    k = int(min(len(pairs), max(threads, rate * per_step / mean_nm)))
    times, cells = [], []
    for step in range(args.warmup + args.steps):
        sample = pairs[np.sort(rng.choice(len(pairs), size=k, replace=False))]
        dt, _ = run_cpu(seqs, matrix, params, sample, threads)
        if step >= args.warmup:
            times.append(dt)
            cells.append(nm_cells(seqs, sample))
    value = sum(cells) / sum(times) / 1e9
    line = {
        "impl": "reference",
        "metric": "GCUPS",
        "value": value,
        "unit": "GCUPS",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int32",
        "data": "synthetic (seeded tree-evolved family)",
        "config": {"workload": args.workload, "pairs": int(len(pairs)), "sample_pairs_per_step": k},
        "cpu_baseline": {
            "value": value,
            "unit": "GCUPS",
            "cores": threads,
            "kind": "port",
            "sample": f"{k} seeded uniform pairs per step of {len(pairs)}; oracle/oracle.c restatement of "
            "FullPairwiseAlign (the reference build needs its source tree, absent on the GPU host)",
        },
        "e2e": {"value": value, "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- launches with few pairs


def _time_plan(plan, stream, steps):
    import torch

    plan.launch(stream.cuda_stream)
    torch.cuda.synchronize()
    ts = []
    for _ in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan.launch(stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1))
    return statistics.median(ts)


def few_pairs_leg(args, device):
    """Launches with fewer long pairs than the long-pair kernel has warps, each
    timed (CUDA events, median of the steps) as dispatched by default and with
    one warp per pair forced (cwgpu_cta_tuning max_pairs 0); both give the same
    distances. Cases: the reference's own 100-sequence DNA set
    (test_data/correct/100_1523.fa, stored in tests/golden/fixture_100_1523.npz)
    whole and as the one-column call sequencesAlignToProfile makes
    (Clustal.cpp:404-416: pairs (i, 99)), and synthetic protein families of
    20 and 6 sequences of about 3000 residues."""
    import torch

    from clustalw_gb300 import load_matrix, native, synth

    z = np.load(os.path.join(REPO, "tests", "golden", "fixture_100_1523.npz"))
    offs = np.concatenate([[0], np.cumsum(z["lens"])[:-1]])
    ref_seqs = [z["codes"][o : o + L].astype(np.int8) for o, L in zip(offs, z["lens"])]
    dna_m, dna_p = load_matrix("dna")
    prot_m, prot_p = load_matrix("protein")
    n = len(ref_seqs)
    cases = [
        ("reference-100x1523-dna-one-column", ref_seqs, dna_m, dna_p,
         np.stack([np.arange(n - 1), np.full(n - 1, n - 1)], axis=1).astype(np.int32)),
        ("reference-100x1523-dna-all", ref_seqs, dna_m, dna_p, synth.all_pairs(n)),
        ("protein-20x3000", synth.protein_family(20, 3000, args.seed), prot_m, prot_p, synth.all_pairs(20)),
        ("protein-6x3000", synth.protein_family(6, 3000, args.seed), prot_m, prot_p, synth.all_pairs(6)),
    ]
    stream = torch.cuda.Stream()
    out = {}
    with native.Context(device) as ctx:
        for name, seqs, matrix, params, pairs in cases:
            ctx.set_matrix(matrix)
            ctx.set_params(params)
            ctx.upload_seqs(seqs)
            cells = nm_cells(seqs, pairs)
            res = {"pairs": int(len(pairs))}
            dists = []
            for label, max_pairs in (("default", None), ("one_warp_per_pair", 0)):
                old = ctx.get_cta_tuning()
                if max_pairs is not None:
                    ctx.set_cta_tuning(max_pairs=max_pairs)
                plan = ctx.plan(pairs)
                ms = _time_plan(plan, stream, 5)
                dists.append(plan.results())
                res[label] = {"gcups": cells / (ms / 1e3) / 1e9, "ms": ms,
                              "form": "one CTA per pair" if plan.pair_ctas() else "one warp per pair"}
                plan.close()
                ctx.set_cta_tuning(*old)
            if not np.array_equal(dists[0], dists[1]):
                raise RuntimeError(f"{name}: the two forms disagree")
            res["default_over_one_warp"] = res["default"]["gcups"] / res["one_warp_per_pair"]["gcups"]
            out[name] = res
    return out


def ref_shaped_leg(args, seqs, matrix, params, pairs, device, batched_gcups):
    """The reference fork's launch shape with this project's kernels: 128 pairs
    per launch, launches round-robin over 4 streams (G/cuda/cudaFullPairwiseAlign.cu:
    14-20, 977-1036), each stream with its own context (plans of one context
    share its scratch), on a seeded uniform sample of the workload's pairs.
    Timed with one warp per pair and with one CTA per pair, next to the
    batched form's GCUPS on the whole workload."""
    import torch

    from clustalw_gb300 import native

    rng = np.random.default_rng(args.seed + 77)
    nchunks = 4 * 12
    sample = pairs[np.sort(rng.choice(len(pairs), size=min(len(pairs), 128 * nchunks), replace=False))]
    chunks = [sample[k : k + 128] for k in range(0, len(sample), 128)]
    res = {"pairs_per_launch": 128, "streams": 4, "sample_pairs": int(len(sample))}
    for label, max_pairs in (("one_warp_per_pair", 0), ("one_cta_per_pair", 2**31 - 1)):
        ctxs = [native.Context(device) for _ in range(4)]
        streams = [torch.cuda.Stream() for _ in range(4)]
        plans = []
        for c in ctxs:
            c.set_cta_tuning(max_pairs=max_pairs)
            c.set_matrix(matrix)
            c.set_params(params)
            c.upload_seqs(seqs)
        for k, ch in enumerate(chunks):
            plans.append((ctxs[k % 4].plan(ch), streams[k % 4]))
        best = float("inf")
        for rep in range(3):
            torch.cuda.synchronize()
            t = time.perf_counter()
            for pl, st in plans:
                pl.launch(st.cuda_stream)
            torch.cuda.synchronize()
            if rep:
                best = min(best, time.perf_counter() - t)
        gcups = nm_cells(seqs, sample) / best / 1e9
        res[label] = {"gcups": gcups, "batched_over_this": batched_gcups / gcups}
        for pl, _ in plans:
            pl.close()
        for c in ctxs:
            c.close()
    return res


# ---------------------------------------------------------------- served leg


def served_leg(args, matrix, params, device):
    """Served stream: Poisson arrivals of independent protein
    families (sequence count U[10, 500], root length U[50, 1500]) admitted
    under a 40 GB budget and mixed in shared rounds; p50/p99 job latency and
    throughput, next to the plain form that runs the same jobs one at a time."""
    from clustalw_gb300 import native, synth
    from clustalw_gb300.serve import Server, percentile, run_arrivals

    njobs = max(4, int(round(args.serve_rate * args.serve_seconds)))
    spec = synth.serve_jobs(njobs, seed=args.seed)
    jobs, cells = [], []
    for n, L, sd in spec:
        seqs = synth.protein_family(n, L, sd)
        jobs.append(native.pack_sequences(seqs))
        lens = np.array([len(x) for x in seqs], dtype=np.int64)
        cells.append(int((np.sum(lens) ** 2 - np.sum(lens * lens)) // 2))
    # Plain per-job form: each job alone through the C ABI, one after another.
    ctx = native.Context(device)
    ctx.set_matrix(matrix)
    ctx.set_params(params)
    sample = list(range(0, njobs, max(1, njobs // 8)))[:8]
    t_plain, c_plain = 0.0, 0
    for k in sample:
        ctx.upload_seqs(packed=jobs[k])
        pr = synth.all_pairs(len(jobs[k][2]))
        t = time.perf_counter()
        ctx.upload_seqs(packed=jobs[k])
        ctx.align_pairs(pr)
        t_plain += time.perf_counter() - t
        c_plain += cells[k]
    ctx.close()
    # The served line: least remaining work first, jobs older than 500 ms first.
    with Server(matrix, params, device=device, memory_budget=40 << 30, max_seq_len=2048, round_cells=6e9,
                policy="srpt", srpt_age_ms=500) as srv:
        for k in range(2):  # warm-up jobs
            srv.wait(srv.submit(packed=jobs[k]))
        lat, arrivals, wall = run_arrivals(srv, jobs, args.serve_rate, seed=args.seed)
        info = srv.query()
        # Capacity: the same jobs all submitted at once; makespan of the batch.
        t = time.perf_counter()
        ids = [srv.submit(packed=pk) for pk in jobs]
        for jid in ids:
            srv.wait(jid)
            srv.release(jid)
        burst_s = time.perf_counter() - t
    # The batched form on the same job mix: every job's sequences in one
    # context, the pairs within each job in one plan, one launch.
    offs, base, codes_all, lens_all, pairs_all = [], 0, [], [], []
    pos = 0
    for pk in jobs:
        c, o, ln = pk
        codes_all.append(c)
        offs.append(o + pos)
        lens_all.append(ln)
        pairs_all.append(synth.all_pairs(len(ln)) + base)
        pos += len(c)
        base += len(ln)
    mix = (np.concatenate(codes_all), np.concatenate(offs).astype(np.int64), np.concatenate(lens_all))
    pairs_mix = np.concatenate(pairs_all).astype(np.int32)
    with native.Context(device) as cm:
        cm.set_matrix(matrix)
        cm.set_params(params)
        cm.upload_seqs(packed=mix)
        plan = cm.plan(pairs_mix)
        import torch

        ms_mix = _time_plan(plan, torch.cuda.Stream(), 2)
        plan.close()
    # The same arrivals in admission order.
    with Server(matrix, params, device=device, memory_budget=40 << 30, max_seq_len=2048, round_cells=6e9,
                policy="fifo") as srv:
        for k in range(2):
            srv.wait(srv.submit(packed=jobs[k]))
        lat_fifo, _, _ = run_arrivals(srv, jobs, args.serve_rate, seed=args.seed)
    return {
        "rate_jobs_per_s": args.serve_rate,
        "jobs": njobs,
        "arrival_seconds": float(arrivals[-1]),
        "p50_ms": 1e3 * percentile(lat, 50),
        "p99_ms": 1e3 * percentile(lat, 99),
        "mean_ms": 1e3 * float(np.mean(lat)),
        "offered_gcups": sum(cells) / wall / 1e9,
        "capacity_gcups": sum(cells) / burst_s / 1e9,
        "plain_per_job_gcups": c_plain / t_plain / 1e9,
        "capacity_over_plain_per_job": (sum(cells) / burst_s) / (c_plain / t_plain),
        "batched_same_mix_gcups": sum(cells) / (ms_mix / 1e3) / 1e9,
        "capacity_over_batched_same_mix": (sum(cells) / burst_s) / (sum(cells) / (ms_mix / 1e3)),
        "plain_sample_jobs": len(sample),
        "rounds": info["rounds"],
        "policy": "least remaining work first; jobs older than 500 ms first, in admission order",
        "fifo": {"p50_ms": 1e3 * percentile(lat_fifo, 50), "p99_ms": 1e3 * percentile(lat_fifo, 99),
                 "mean_ms": 1e3 * float(np.mean(lat_fifo)), "policy": "admission order"},
        "budget_bytes": 40 << 30,
        "workload": "protein families, N ~ U[10,500], root length ~ U[50,1500], Poisson arrivals",
    }


def _make_job(spec):
    from clustalw_gb300 import native, synth

    n, L, sd = spec
    return native.pack_sequences(synth.protein_family(n, L, sd))


def serve_only(args):
    """The served configuration at its stated length: Poisson arrivals at
    --serve-rate jobs/s for --serve-seconds (default here 600 s), jobs from the
    served generator (protein families, N ~ U[10, 500], root length ~ U[50,
    1500]), 40 GB budget, least remaining work first with a 500 ms age cap.
    Jobs are generated before the run on all host cores (spawned workers, before
    any device call). Prints one JSON line with the latency distribution over
    every job, the arrival rate, the offered GCUPS and the memory peak."""
    import multiprocessing as mp

    from clustalw_gb300 import load_matrix, synth

    njobs = max(4, int(round(args.serve_rate * args.serve_seconds)))
    spec = synth.serve_jobs(njobs, seed=args.seed)
    t = time.perf_counter()
    with mp.get_context("spawn").Pool(os.cpu_count() or 1) as pool:
        jobs = pool.map(_make_job, spec, chunksize=8)
    gen_s = time.perf_counter() - t
    cells = [int((int(ln.sum()) ** 2 - int((ln.astype(np.int64) ** 2).sum())) // 2) for _, _, ln in jobs]

    import torch

    from clustalw_gb300.serve import Server, percentile, run_arrivals

    _, _, local = dist_env()
    torch.cuda.set_device(local)
    matrix, params = load_matrix("protein")
    peaks = {}
    with Server(matrix, params, device=local, memory_budget=40 << 30, max_seq_len=2048, round_cells=6e9,
                policy="srpt", srpt_age_ms=500) as srv:
        for k in range(2):  # warm-up jobs
            srv.wait(srv.submit(packed=jobs[k]))
        uuid = getattr(torch.cuda.get_device_properties(local), "uuid", None)
        uuid = None if uuid is None else (str(uuid) if str(uuid).startswith("GPU-") else "GPU-" + str(uuid))
        with ClockSampler(uuid) as clk:
            lat, arrivals, wall = run_arrivals(srv, jobs, args.serve_rate, seed=args.seed, peaks=peaks)
        info = srv.query()
    lat_ms = 1e3 * lat
    line = {
        "mode": "serve",
        "rate_jobs_per_s": args.serve_rate,
        "seconds": float(arrivals[-1]),
        "jobs": njobs,
        "p50_ms": percentile(lat_ms, 50),
        "p90_ms": percentile(lat_ms, 90),
        "p99_ms": percentile(lat_ms, 99),
        "p999_ms": percentile(lat_ms, 99.9),
        "max_ms": float(np.max(lat_ms)),
        "mean_ms": float(np.mean(lat_ms)),
        "offered_gcups": sum(cells) / wall / 1e9,
        "wall_s": wall,
        "memory_peak_bytes": peaks.get("bytes_in_use"),
        "queued_peak_jobs": peaks.get("queued"),
        "budget_bytes": 40 << 30,
        "rounds": info["rounds"],
        "policy": "least remaining work first; jobs older than 500 ms first, in admission order",
        "workload": "protein families, N ~ U[10,500], root length ~ U[50,1500], Poisson arrivals",
        "job_generation_s": gen_s,
    }
    clocks = clk.summary()
    if clocks:
        line["clocks"] = clocks
    print(json.dumps(line), flush=True)


def packed_distmatrix(n, pairs, dist):
    """The DistMatrix elements FullPairwiseAlign leaves (SymMatrix of size n+1,
    general/SymMatrix.h:166-197): the float distance stored as a double."""
    el = np.zeros((n + 1) * (n + 2) // 2, dtype=np.float64)
    si = pairs[:, 0].astype(np.int64)
    sj = pairs[:, 1].astype(np.int64)
    el[sj * (sj + 1) // 2 + si] = np.asarray(dist, dtype=np.float32).astype(np.float64)
    return el


def guide_tree_leg(args, n, pairs, dist, device, peaks):
    """Guide tree (NJTree::generateTree, tree/NJTree.cpp:161-748) on the distance
    matrix this step produced: the GPU join kernel device-resident (CUDA events
    on its stream) and through the C ABI with host buffers, checked bit for bit
    against the oracle restatement, which is also the timed CPU baseline."""
    import torch

    from clustalw_gb300.tree import NJGpu
    from oracle import oracle

    el = packed_distmatrix(n, pairs, dist)
    nj = NJGpu(device)
    dev = torch.device("cuda", device)
    d_in = torch.from_numpy(el).to(dev)
    d_out = torch.empty_like(d_in)
    d_left = torch.empty(n + 2, dtype=torch.float64, device=dev)
    d_right = torch.empty(n + 2, dtype=torch.float64, device=dev)
    d_desc = torch.empty((n + 1) * (n + 1), dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.synchronize()
    steps, warmup = max(1, args.steps), max(3, args.warmup)
    times = []
    for k in range(warmup + steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        nj.tree_device(n, d_in.data_ptr(), d_out.data_ptr(), d_left.data_ptr(), d_right.data_ptr(),
                       d_desc.data_ptr(), None, stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        if k >= warmup:
            times.append(e0.elapsed_time(e1) / 1e3)
    pairs_eval, kernel_s = nj.last_stats()
    dev_s = statistics.median(times)
    # Through the C ABI with host buffers (copies in and out inside the timing).
    e2e = []
    for k in range(steps + 1):
        w = el.copy()
        t = time.perf_counter()
        left, right, desc, _ = nj.tree(n, w)
        if k:
            e2e.append(time.perf_counter() - t)
    e2e_s = statistics.median(e2e)
    # Oracle: parity and the CPU baseline (one thread, like the reference).
    t = time.perf_counter()
    want = oracle.nj_tree(n, el.copy())
    cpu_s = time.perf_counter() - t
    same = (np.array_equal(left.view(np.int64), want[0].view(np.int64))
            and np.array_equal(right.view(np.int64), want[1].view(np.int64))
            and np.array_equal(desc, want[2]) and np.array_equal(w.view(np.int64), want[3].view(np.int64))
            and np.array_equal(d_out.cpu().numpy().view(np.int64), want[3].view(np.int64)))
    nj.close()
    fp64_ops = 4 * pairs_eval  # fnseqs2*d + 2*sumd - diq - djq per pair (NJTree.cpp:331-376)
    fp64_peak = FP64_NOMINAL_TFLOPS
    return {
        "metric": "ms per tree",
        "value": 1e3 * dev_s,
        "unit": "ms",
        "higher_is_better": False,
        "n": n,
        "cycles": n - 3,
        "pairs_evaluated": int(pairs_eval),
        "e2e": {"value": 1e3 * e2e_s, "unit": "ms", "h2d_bytes_per_step": int(el.nbytes),
                "d2h_bytes_per_step": int(el.nbytes + 16 * (n + 2) + 4 * (n + 1) * (n + 1)),
                "call": "cwgpu_nj_tree (host DistMatrix in; branches, treeDesc, joined matrix out)"},
        "cpu_baseline": {"value": 1e3 * cpu_s, "unit": "ms", "cores": 1, "kind": "port",
                         "sample": f"the full tree on the same {n}-sequence matrix (NJTree is single-threaded)"},
        "speedup_vs_cpu": cpu_s / dev_s,
        "bit_exact_vs_oracle": bool(same),
        "roofline": {"bound": "latency (sequential per-cycle sums and one join per cycle)",
                     "kernel": "k_nj", "fp64_ops_per_launch": int(fp64_ops),
                     "achieved": fp64_ops / kernel_s / 1e12, "peak": fp64_peak, "unit": "TFLOP/s (fp64 add/mul)",
                     "frac": fp64_ops / kernel_s / 1e12 / fp64_peak,
                     "peak_source": "nominal GB300 fp64 (no measured fp64 peak is available)"},
        "gpu_launches": 1,
    }


def quick_leg(args, ctx, seqs, pairs, device):
    """Quick k-tuple distances (FastPairwiseAlign::pairwiseAlign,
    pairwise/FastPairwiseAlign.cpp:20-400) over every pair of the workload with
    the reference's default parameters: device-resident (CUDA events on the
    launching stream), through the C ABI with host buffers, a seeded parity
    sample against the oracle, and the oracle on all host threads."""
    import torch

    from clustalw_gb300 import native
    from oracle import oracle

    n = len(seqs)
    fp = native.FastParams.defaults(0, 2 * max(len(x) for x in seqs))
    lens = np.array([len(x) for x in seqs], dtype=np.int64)
    order = np.argsort(-(lens[pairs[:, 0]] * lens[pairs[:, 1]]), kind="stable").astype(np.int32)
    dev = torch.device("cuda", device)
    d_pairs = torch.from_numpy(np.ascontiguousarray(pairs, dtype=np.int32)).to(dev)
    d_order = torch.from_numpy(order).to(dev)
    d_dist = torch.empty(len(pairs), dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.synchronize()
    steps, warmup = max(1, args.steps), max(3, args.warmup)
    times = []
    for k in range(warmup + steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.fast_align_pairs_device(fp, d_pairs.data_ptr(), d_order.data_ptr(), len(pairs), d_dist.data_ptr(), None,
                                    stream.cuda_stream)
        e1.record(stream)
        torch.cuda.synchronize()
        if k >= warmup:
            times.append(e0.elapsed_time(e1) / 1e3)
    dev_s = statistics.median(times)
    dist_dev = d_dist.cpu().numpy()
    e2e = []
    for k in range(min(steps, 3) + 1):
        t = time.perf_counter()
        ctx.upload_seqs(seqs)
        d = ctx.fast_align_pairs(pairs, fp)
        if k:
            e2e.append(time.perf_counter() - t)
    e2e_s = statistics.median(e2e)
    # Parity sample and CPU baseline: the oracle on all host threads.
    rng = np.random.default_rng(11)
    samp = np.sort(rng.choice(len(pairs), size=min(len(pairs), 4000), replace=False))
    threads = os.cpu_count() or 1
    fpd = {k: int(getattr(fp, k)) for k, _ in native.FastParams._fields_}
    t = time.perf_counter()
    want = oracle.fast_pairs(seqs, fpd, pairs[samp], nthreads=threads)
    cpu_s = time.perf_counter() - t
    same = bool(np.array_equal(want["dist"].view(np.int64), dist_dev[samp].view(np.int64))
                and np.array_equal(d.view(np.int64), dist_dev.view(np.int64)))
    cpu_rate = len(samp) / cpu_s
    return {
        "metric": "pairs per second",
        "value": len(pairs) / dev_s,
        "unit": "pairs/s",
        "ms_per_step": 1e3 * dev_s,
        "pairs": int(len(pairs)),
        "params": fpd,
        "e2e": {"value": len(pairs) / e2e_s, "unit": "pairs/s", "ms_per_step": 1e3 * e2e_s,
                "h2d_bytes_per_step": int(sum(len(x) for x in seqs) + 8 * len(pairs) + 12 * n),
                "d2h_bytes_per_step": int(8 * len(pairs)),
                "call": "cwgpu_upload_seqs + cwgpu_fast_align_pairs (host pair list in, host distances out)"},
        "cpu_baseline": {"value": cpu_rate, "unit": "pairs/s", "cores": threads, "kind": "port",
                         "sample": f"{len(samp)} of {len(pairs)} pairs (seeded uniform), {cpu_s:.1f} s on {threads} threads"},
        "speedup_vs_cpu": (len(pairs) / dev_s) / cpu_rate,
        "bit_exact_vs_oracle_sample": same,
        "roofline": {"bound": "latency (per-pair sequential fragment chaining, one warp per pair)", "kernel": "k_fast"},
        "gpu_launches": steps,
    }


# ---------------------------------------------------------------- GPU arm


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def traffic_per_cell():
    """DRAM bytes per forward cell from the committed ncu summary, if any."""
    path = os.path.join(REPO, "profiles", "k_pairwise_traffic.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["dram_bytes_per_nm_cell"]), d.get("source", path)
    except (OSError, KeyError, ValueError):
        return None, None


def ours_arm(args):
    import torch

    from clustalw_gb300 import native, synth

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    seqs, matrix, params = make_workload(args.workload, args.seed + rank, args.nseqs)
    pairs = synth.all_pairs(len(seqs))
    cells_nm = nm_cells(seqs, pairs)
    packed = native.pack_sequences(seqs)

    ctx = native.Context(local)
    ctx.set_matrix(matrix)
    ctx.set_params(params)
    ctx.upload_seqs(packed=packed)
    tuning = {"tiny_m_tiny_n_short_rows": list(ctx.get_tuning()), "autotuned": False}
    if args.autotune:
        from clustalw_gb300 import autotune

        choice, timings = autotune.tune(ctx, packed[2], pairs, gpu_name=torch.cuda.get_device_name(local))
        cta_choice, cta_timings = autotune.tune_cta(ctx, packed[2], pairs)
        tuning = {"tiny_m_tiny_n_short_rows": list(choice), "autotuned": True,
                  "candidates_s": {",".join(map(str, c)): round(t, 4) for c, t in timings.items()},
                  "cta_max_pairs_warps_large_rows": list(cta_choice),
                  "cta_candidates_s": {",".join(map(str, c)): round(t, 4) for c, t in cta_timings.items()}}
    plan = ctx.plan(pairs)
    # A dedicated stream: the graph is launched on it and the CUDA events are
    # recorded on it (torch's default stream has handle 0, which the C ABI
    # reads as "the context's own stream").
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2

    for _ in range(args.warmup):
        plan.launch(stream.cuda_stream)
    torch.cuda.synchronize()
    fwd, rev, dif = plan.cell_counts()
    ref_dist = plan.results()

    uuid = getattr(torch.cuda.get_device_properties(local), "uuid", None)
    uuid = None if uuid is None else (str(uuid) if str(uuid).startswith("GPU-") else "GPU-" + str(uuid))
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(uuid) as clk:
        for k in range(args.steps):
            flush.zero_()
            starts[k].record(stream)
            plan.launch(stream.cuda_stream)
            ends[k].record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_s = sum(step_ms) / 1e3
    if world > 1:
        t = torch.tensor([total_s], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_s = float(t.item())
    dist_out = plan.results()
    if not np.array_equal(dist_out, ref_dist):
        raise RuntimeError("distances changed between runs")
    ms = 1e3 * total_s / args.steps
    cells_all = cells_nm  # every rank's replica has its own seed: sum the ranks' cells
    if world > 1:
        c = torch.tensor([float(cells_nm)], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(c)
        cells_all = float(c.item())
    value = cells_all * args.steps / total_s / 1e9
    if args.device_only:
        if rank == 0:
            print(json.dumps({"metric": "GCUPS", "value": value, "ms_per_step": ms, "pairs": int(len(pairs)),
                              "cells": [fwd, rev, dif], "device_only": True}), flush=True)
        plan.close()
        ctx.close()
        return

    # End to end through the C ABI with host buffers.
    # At least --e2e-steps calls, more for short steps (about 1 s of calls, at most 100).
    e2e_steps = max(args.e2e_steps, min(100, int(1e3 / max(ms, 1e-3))))
    e2e_times = []
    torch.cuda.set_stream(torch.cuda.default_stream())
    for k in range(e2e_steps + 1):
        torch.cuda.synchronize()
        t = time.perf_counter()
        ctx.upload_seqs(packed=packed)
        d = ctx.align_pairs(pairs)
        e2e_times.append(time.perf_counter() - t)
        if k == 0 and not np.array_equal(d, ref_dist):
            raise RuntimeError("e2e distances differ from the device-resident run")
    e2e_s = statistics.mean(e2e_times[1:])
    if world > 1:  # the slowest rank's call, like the device-resident number
        t = torch.tensor([e2e_s], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
    lmax = int(packed[2].max()) if len(packed[2]) else 0
    codes_padded = int(sum((int(L) + 15) & ~15 for L in packed[2]))
    h2d = codes_padded + 8 * len(seqs) + 4 * len(seqs) + 4 * len(seqs) + 4 * (lmax + 1) + 4 * 1024
    h2d += 8 * len(pairs) + 4 * len(pairs)
    d2h = 4 * len(pairs) + 4  # distances + the kernel status word

    # Plain one-launch-per-pair form on a seeded sample of the same pairs.
    rng = np.random.default_rng(7)
    ps = pairs[np.sort(rng.choice(len(pairs), size=min(args.plain_pairs, len(pairs)), replace=False))]
    ctx.align_pairs(ps[:2], plain=True)
    t = time.perf_counter()
    d_plain = ctx.align_pairs(ps, plain=True)
    plain_s = time.perf_counter() - t
    # Same pairs through the batched form: must agree bit for bit.
    if not np.array_equal(d_plain, ctx.align_pairs(ps)):
        raise RuntimeError("plain and batched forms disagree")
    plain_gcups = nm_cells(seqs, ps) / plain_s / 1e9

    peaks = measured_peaks()
    props = torch.cuda.get_device_properties(local)
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    peak_tops = props.multi_processor_count * INT32_LANES_PER_SM * sm_max * 1e6 / 1e12
    cells_alg = fwd + rev + dif
    achieved = cells_alg * OPS_PER_CELL / (ms / 1e3) / 1e12
    tpc, tsrc = traffic_per_cell()
    roofline = {
        "bound": "int32",
        "achieved": achieved,
        "peak": peak_tops,
        "unit": "Tops/s",
        "frac": achieved / peak_tops,
        "traffic": (tpc * cells_nm) if tpc is not None else None,
        "kernel": "k_pairwise",
        "cells_per_launch": {"forward": fwd, "reverse": rev, "diff": dif, "total": cells_alg},
        "ops_per_cell": OPS_PER_CELL,
        "peak_source": f"{props.multi_processor_count} SMs x {INT32_LANES_PER_SM} INT32 lanes x "
        f"{sm_max:.0f} MHz (sm_max_mhz of MEASURED_PEAKS.json)",
        "hbm_peak_gbs": peaks.get("hbm_gbs"),
        # DRAM bytes per launch over the launch time: how far the kernel is from the HBM roof
        "hbm_achieved_gbs": (tpc * cells_nm / (ms / 1e3) / 1e9) if tpc is not None else None,
        "traffic_source": tsrc,
        # The recurrence's max, add and DPX instructions all issue on the
        # integer ALU pipe, which takes half the INT32 lane rate (64 lanes per
        # SM per clock): the same operation count against that pipe's rate.
        "alu_pipe": {"peak": peak_tops * ALU_PIPE_LANES_PER_SM / INT32_LANES_PER_SM,
                     "frac": achieved / (peak_tops * ALU_PIPE_LANES_PER_SM / INT32_LANES_PER_SM),
                     "lanes_per_sm": ALU_PIPE_LANES_PER_SM},
    }

    line = {
        "metric": "GCUPS",
        "value": value,
        "unit": "GCUPS",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "int32",
        "data": "synthetic (seeded tree-evolved family)",
        "config": {
            "workload": args.workload,
            "nseqs": len(seqs),
            "pairs": int(len(pairs)),
            "mean_len": float(np.mean(packed[2])),
            "matrix": "gonnet" if params["dna"] == 0 else "iub",
            "form": "batched: persistent graph-captured launch, longest pairs first",
            "l2": "flushed between timed steps (256 MiB write, untimed)",
            "pairs_per_s": len(pairs) * world / (ms / 1e3),
            "tuning": tuning,
        },
        "e2e": {
            "value": cells_all / e2e_s / 1e9,
            "unit": "GCUPS",
            "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h,
            "ms_per_step": 1e3 * e2e_s,
            "steps": e2e_steps,
            "call": "cwgpu_upload_seqs + cwgpu_align_pairs (host pair list in, host distances out)",
        },
        "plain": {
            "value": plain_gcups,
            "unit": "GCUPS",
            "sample": f"{len(ps)} pairs, one kernel launch per pair",
            "batched_over_plain": value / world / plain_gcups,
        },
        "roofline": roofline,
        "gpu_launches": args.steps * plan.kernel_count(),
    }
    if rank == 0:
        clocks = clk.summary()
        if clocks:
            line["clocks"] = clocks
        if world == 1:
            line["cpu_baseline"] = cpu_baseline(seqs, matrix, params, pairs, args.cpu_seconds)
            if not args.no_serve:
                line["serve"] = served_leg(args, matrix, params, local)
            if not args.no_tree:
                line["guide_tree"] = guide_tree_leg(args, len(seqs), pairs, dist_out, local, peaks)
            if not args.no_quick:
                line["quick"] = quick_leg(args, ctx, seqs, pairs, local)
            if not args.no_few:
                line["few_pairs"] = few_pairs_leg(args, local)
                line["reference_shaped"] = ref_shaped_leg(args, seqs, matrix, params, pairs, local, value)
        print(json.dumps(line), flush=True)
    plan.close()
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse_args()
    if args.impl == "reference":
        reference_arm(args)
    elif args.serve_only:
        serve_only(args)
    else:
        ours_arm(args)


if __name__ == "__main__":
    main()
