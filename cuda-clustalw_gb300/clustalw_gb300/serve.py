"""Serving: continuous batching of alignment jobs on one GPU (cwgpu_server_*).

A job is one sequence set; its result is the distance array the reference's
FullPairwiseAlign::pairwiseAlign writes for all N(N-1)/2 pairs
(CPU/clustalw-2.0.11/src/pairwise/FullPairwiseAlign.cpp:97-190), in loop order.
The native scheduler admits jobs by device memory, mixes pairs of all admitted
jobs in each persistent launch and keeps two launches in flight; this module
wraps it and runs a timed arrival process for the served benchmark.
"""
import ctypes
import threading
import time

import numpy as np

from . import native
from .native import PAIR_STATS_DTYPE, CwgpuError, Params, ServerOpts, ServerStats

JOB_QUEUED, JOB_RUNNING, JOB_DONE, JOB_FAILED = 0, 1, 2, 3


class Server:
    POLICIES = {"fifo": 0, "srpt": 1}

    def __init__(self, matrix, params, device=0, memory_budget=8 << 30, max_jobs=256, max_seq_len=4096,
                 round_cells=4e9, max_items_per_round=1 << 20, policy="srpt", srpt_age_ms=500):
        """policy: "srpt" (least remaining work first; jobs older than
        srpt_age_ms, if > 0, go first in admission order) or "fifo" (admission
        order)."""
        self._lib = native.load()
        m = np.ascontiguousarray(np.asarray(matrix, dtype=np.int32).reshape(-1))
        p = params if isinstance(params, Params) else Params.from_dict(params)
        opts = ServerOpts(int(memory_budget), int(max_jobs), int(max_seq_len), float(round_cells),
                          int(max_items_per_round), self.POLICIES[policy], int(srpt_age_ms))
        h = ctypes.c_void_p()
        rc = self._lib.cwgpu_server_create(int(device), m.ctypes.data, ctypes.byref(p), ctypes.byref(opts),
                                           ctypes.byref(h))
        if rc:
            raise CwgpuError(rc, "cwgpu_server_create")
        self._h = h
        self._npairs = {}
        self._stats = {}

    def close(self):
        if getattr(self, "_h", None):
            self._lib.cwgpu_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, seqs=None, packed=None, stats=False):
        codes, offsets, lens = packed if packed is not None else native.pack_sequences(seqs)
        codes = np.ascontiguousarray(codes, dtype=np.int8)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        lens = np.ascontiguousarray(lens, dtype=np.int32)
        jid = ctypes.c_int64()
        rc = self._lib.cwgpu_server_submit(self._h, len(lens), codes.ctypes.data, offsets.ctypes.data,
                                           lens.ctypes.data, 1 if stats else 0, ctypes.byref(jid))
        if rc:
            raise CwgpuError(rc, "cwgpu_server_submit")
        n = len(lens)
        self._npairs[jid.value] = n * (n - 1) // 2
        self._stats[jid.value] = bool(stats)
        return jid.value

    def poll(self, job_id):
        st = ctypes.c_int32()
        rc = self._lib.cwgpu_server_poll(self._h, int(job_id), ctypes.byref(st))
        if rc:
            raise CwgpuError(rc, "cwgpu_server_poll")
        return st.value

    def wait(self, job_id, timeout_ms=-1):
        rc = self._lib.cwgpu_server_wait(self._h, int(job_id), int(timeout_ms))
        if rc:
            raise CwgpuError(rc, "cwgpu_server_wait")

    def result(self, job_id):
        """(distances, stats or None, times[submit, admit, first round, done])."""
        n = self._npairs[job_id]
        dist = np.zeros(max(n, 1), dtype=np.float32)
        st = np.zeros(max(n, 1), dtype=PAIR_STATS_DTYPE) if self._stats[job_id] else None
        times = np.zeros(4, dtype=np.float64)
        rc = self._lib.cwgpu_server_result(self._h, int(job_id), dist.ctypes.data,
                                           None if st is None else st.ctypes.data, times.ctypes.data)
        if rc:
            raise CwgpuError(rc, "cwgpu_server_result")
        return dist[:n], (None if st is None else st[:n]), times

    def release(self, job_id):
        rc = self._lib.cwgpu_server_release(self._h, int(job_id))
        if rc:
            raise CwgpuError(rc, "cwgpu_server_release")
        self._npairs.pop(job_id, None)
        self._stats.pop(job_id, None)

    def query(self):
        s = ServerStats()
        rc = self._lib.cwgpu_server_query(self._h, ctypes.byref(s))
        if rc:
            raise CwgpuError(rc, "cwgpu_server_query")
        return dict(queued=s.jobs_queued, running=s.jobs_running, done=s.jobs_done, rounds=s.rounds,
                    pairs=s.pairs, bytes_in_use=s.bytes_in_use, cells=tuple(s.cells))


def percentile(values, q):
    v = np.sort(np.asarray(values, dtype=np.float64))
    if len(v) == 0:
        return float("nan")
    return float(np.percentile(v, q))


def run_arrivals(server, jobs, rate, seed=0, peaks=None):
    """Submit pre-built jobs (list of packed sequence sets) at Poisson times of
    the given rate (jobs/s) while a collector thread waits for, reads and
    releases finished jobs in completion order. Returns the per-job latencies
    (seconds, submission to completion as the server records them), the
    arrival offsets and the session wall time. If `peaks` is a dict, it
    receives the largest device memory the admitted jobs held
    ("bytes_in_use") and the most jobs queued at once ("queued")."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=len(jobs))
    arrivals = np.cumsum(gaps) - gaps[0]
    records = [None] * len(jobs)
    ids = [None] * len(jobs)
    fresh = []  # job indices submitted since the collector last looked
    submitted = threading.Event()
    lock = threading.Lock()
    errors = []
    peak = {"bytes_in_use": 0, "queued": 0}

    def collector():
        pending = set()
        last_query = 0.0
        while True:
            with lock:
                pending.update(fresh)
                fresh.clear()
            if not pending and submitted.is_set():
                break
            done_any = False
            for k in sorted(pending):
                try:
                    if server.poll(ids[k]) not in (JOB_DONE, JOB_FAILED):
                        continue
                    _, _, times = server.result(ids[k])
                    records[k] = times
                    server.release(ids[k])
                except CwgpuError as e:  # surfaced after the run
                    errors.append(e)
                    records[k] = np.array([np.nan] * 4)
                pending.discard(k)
                done_any = True
            now = time.perf_counter()
            if peaks is not None and now - last_query > 0.05:
                q = server.query()
                peak["bytes_in_use"] = max(peak["bytes_in_use"], q["bytes_in_use"])
                peak["queued"] = max(peak["queued"], q["queued"])
                last_query = now
            if not done_any:
                time.sleep(0.001)

    th = threading.Thread(target=collector)
    th.start()
    t0 = time.perf_counter()
    for k, packed in enumerate(jobs):
        delay = arrivals[k] - (time.perf_counter() - t0)
        if delay > 0:
            time.sleep(delay)
        jid = server.submit(packed=packed)
        with lock:
            ids[k] = jid
            fresh.append(k)
    submitted.set()
    th.join()
    wall = time.perf_counter() - t0
    if errors:
        raise errors[0]
    if peaks is not None:
        peaks.update(peak)
    lat = np.array([r[3] - r[0] for r in records])
    return lat, arrivals, wall
