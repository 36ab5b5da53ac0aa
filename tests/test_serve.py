"""Serving engine (cwgpu_server_*): every job's distances and per-pair
statistics are identical whether the job runs alone (cwgpu_align_pairs on its
own context) or mixed with other jobs in the server's shared rounds; admission
by device-memory budget; jobs arriving while others run; residue codes that
grow the server's alphabet mid-session."""
import threading
import time

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def alone(matrix, params, seqs):
    from clustalw_gb300 import native, synth

    with native.Context(0) as ctx:
        ctx.set_matrix(matrix)
        ctx.set_params(params)
        ctx.upload_seqs(seqs)
        return ctx.align_pairs(synth.all_pairs(len(seqs)), stats=True)


def protein_jobs():
    from clustalw_gb300 import synth

    spec = [(12, 60, 1), (40, 200, 2), (25, 700, 3), (60, 90, 4), (8, 1200, 5), (30, 40, 6), (3, 10, 7), (2, 1, 8)]
    return [synth.protein_family(n, L, s) for n, L, s in spec]


@pytest.mark.parametrize("policy,age", [("fifo", 0), ("srpt", 0), ("srpt", 1)])
def test_mixed_jobs_equal_alone(policy, age):
    from clustalw_gb300 import load_matrix
    from clustalw_gb300.serve import Server

    matrix, params = load_matrix("protein")
    jobs = protein_jobs()
    want = [alone(matrix, params, j) for j in jobs]
    # Small rounds so every round mixes pairs of several jobs.
    with Server(matrix, params, memory_budget=256 << 20, round_cells=2e6, policy=policy, srpt_age_ms=age) as srv:
        ids = [srv.submit(j, stats=True) for j in jobs]
        for jid in ids:
            srv.wait(jid, timeout_ms=120000)
        rounds = srv.query()["rounds"]
        for jid, (wd, ws) in zip(ids, want):
            d, s, times = srv.result(jid)
            assert np.array_equal(d, wd)
            assert np.array_equal(s, ws)
            assert times[0] <= times[1] <= times[3]
            srv.release(jid)
    assert rounds > len(jobs)


def test_admission_waits_for_budget_memory():
    from clustalw_gb300 import load_matrix
    from clustalw_gb300.native import CwgpuError
    from clustalw_gb300.serve import JOB_QUEUED, Server
    from clustalw_gb300 import synth

    matrix, params = load_matrix("protein")
    jobs = [synth.protein_family(80, 300, 20 + k) for k in range(4)]
    want = [alone(matrix, params, j)[0] for j in jobs]
    # Each job needs about 40 KB (24 KB of residues, 13 KB of distances, tables):
    # a 100 KB budget holds two at a time.
    with Server(matrix, params, memory_budget=100 << 10, round_cells=5e7) as srv:
        ids = [srv.submit(j) for j in jobs]
        assert srv.poll(ids[3]) == JOB_QUEUED
        got = {}

        def drain():
            for jid in ids:
                srv.wait(jid, timeout_ms=120000)
                got[jid] = srv.result(jid)[0]
                srv.release(jid)

        th = threading.Thread(target=drain)
        th.start()
        th.join(timeout=180)
        assert not th.is_alive()
        for jid, w in zip(ids, want):
            assert np.array_equal(got[jid], w)
        with pytest.raises(CwgpuError):
            srv.submit(synth.protein_family(300, 400, 99))  # never fits the budget


def test_arrivals_while_running_and_alphabet_growth():
    from clustalw_gb300 import load_matrix, synth
    from clustalw_gb300.serve import Server

    matrix, params = load_matrix("protein")
    big = synth.protein_family(120, 900, 31)
    edge = load_golden("edge_protein")["seqs"]  # gaps, B/Z/X codes: new codes for the server
    small = [synth.protein_family(10, 50, 32), edge, synth.protein_family(6, 300, 33)]
    want_big = alone(matrix, params, big)
    want_small = [alone(matrix, params, j) for j in small]
    with Server(matrix, params, memory_budget=512 << 20, round_cells=3e7) as srv:
        b = srv.submit(big, stats=True)
        time.sleep(0.02)
        ids = [srv.submit(j, stats=True) for j in small]
        for jid, (wd, ws) in zip(ids, want_small):
            srv.wait(jid, timeout_ms=120000)
            d, s, _ = srv.result(jid)
            assert np.array_equal(d, wd) and np.array_equal(s, ws)
        srv.wait(b, timeout_ms=120000)
        d, s, _ = srv.result(b)
        assert np.array_equal(d, want_big[0]) and np.array_equal(s, want_big[1])


def test_dna_server():
    from clustalw_gb300 import load_matrix, synth
    from clustalw_gb300.serve import Server

    matrix, params = load_matrix("dna")
    jobs = [synth.dna_family(20, 400, 41), synth.dna_family(35, 150, 42)]
    want = [alone(matrix, params, j) for j in jobs]
    with Server(matrix, params, memory_budget=64 << 20, round_cells=1e7) as srv:
        ids = [srv.submit(j, stats=True) for j in jobs]
        for jid, (wd, ws) in zip(ids, want):
            srv.wait(jid, timeout_ms=120000)
            d, s, _ = srv.result(jid)
            assert np.array_equal(d, wd) and np.array_equal(s, ws)
