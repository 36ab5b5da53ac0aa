"""Host logic of the served benchmark (clustalw_gb300.serve.run_arrivals and
percentile) against a fake server, on the CPU: jobs arrive at Poisson times,
every finished job is read and released exactly once, latencies come from the
server's own time stamps, and a server error surfaces after the run instead of
stopping the collector."""
import math
import threading
import time

import numpy as np
import pytest


class FakeServer:
    """The four calls run_arrivals makes; job j finishes service_s after its
    submission, and poll raises for the ids in fail_poll."""

    def __init__(self, service_s=0.002, fail_poll=()):
        self.service_s = service_s
        self.fail_poll = set(fail_poll)
        self.submitted = {}
        self.released = []
        self.lock = threading.Lock()

    def submit(self, seqs=None, packed=None, stats=False):
        with self.lock:
            jid = 100 + len(self.submitted)
            self.submitted[jid] = time.perf_counter()
        return jid

    def poll(self, job_id):
        from clustalw_gb300.native import CwgpuError
        from clustalw_gb300.serve import JOB_DONE, JOB_RUNNING

        if job_id in self.fail_poll:
            raise CwgpuError(2, "cwgpu_server_poll")
        return JOB_DONE if time.perf_counter() - self.submitted[job_id] >= self.service_s else JOB_RUNNING

    def result(self, job_id):
        t0 = self.submitted[job_id]
        return np.zeros(0, np.float32), None, np.array([t0, t0, t0, t0 + self.service_s])

    def release(self, job_id):
        with self.lock:
            self.released.append(job_id)

    def query(self):
        with self.lock:  # bytes held: 1 MiB per job submitted and not released
            live = len(self.submitted) - len(self.released)
        return dict(queued=0, bytes_in_use=live << 20)


def test_run_arrivals_reads_and_releases_every_job():
    from clustalw_gb300.serve import run_arrivals

    srv = FakeServer(service_s=0.002)
    lat, arrivals, wall = run_arrivals(srv, [None] * 20, rate=500.0, seed=3)
    assert sorted(srv.released) == list(range(100, 120))  # each job once
    assert np.allclose(lat, 0.002)  # from the server's submit/done stamps
    assert arrivals[0] == 0.0 and np.all(np.diff(arrivals) >= 0)
    assert wall >= arrivals[-1]
    lat2, arrivals2, _ = run_arrivals(FakeServer(), [None] * 20, rate=500.0, seed=3)
    assert np.array_equal(arrivals, arrivals2)  # seeded arrival process


def test_run_arrivals_surfaces_server_errors():
    from clustalw_gb300.native import CwgpuError
    from clustalw_gb300.serve import run_arrivals

    srv = FakeServer(fail_poll={103})
    with pytest.raises(CwgpuError):
        run_arrivals(srv, [None] * 8, rate=1000.0, seed=1)
    assert sorted(srv.released) == [j for j in range(100, 108) if j != 103]


def test_percentile():
    from clustalw_gb300.serve import percentile

    assert math.isnan(percentile([], 50))
    assert percentile([4, 1, 3, 2], 50) == 2.5
    assert percentile(range(101), 99) == 99.0


def test_run_arrivals_records_the_memory_peak():
    from clustalw_gb300.serve import run_arrivals

    srv = FakeServer(service_s=0.12)
    peaks = {}
    lat, _, _ = run_arrivals(srv, [None] * 12, rate=400.0, seed=5, peaks=peaks)
    assert len(lat) == 12 and sorted(srv.released) == sorted(srv.submitted)
    # all 12 jobs arrive within about 30 ms and each is held 120 ms
    assert peaks["bytes_in_use"] >= 8 << 20 and peaks["queued"] == 0
