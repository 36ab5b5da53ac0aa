"""Multi-GPU sharding logic on CPU: the static partition covers every pair
once with balanced n*m, and two gloo ranks assemble exactly the distances one
process would produce, with the oracle (the CPU restatement of the full
pairwise stage, and of the quick k-tuple distances) as each rank's aligner,
since this host has no GPU; the GPU path itself is covered by the -m gpu
tests."""
import os

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp


def full_align(seqs, pairs):
    """Full pairwise distances (float32) from the oracle, Gonnet at 10 / 0.1."""
    from clustalw_gb300 import load_matrix
    from oracle import oracle

    matrix, params = load_matrix("protein")
    return oracle.align_pairs(seqs, matrix, params, pairs, nthreads=1)["dist"]


def _seqs_full():
    from clustalw_gb300.synth import protein_family

    return protein_family(18, 70, 4) + protein_family(19, 140, 5)


def test_partition_covers_and_balances():
    from clustalw_gb300.shard import partition_pairs
    from clustalw_gb300.synth import all_pairs

    rng = np.random.default_rng(0)
    lens = rng.integers(30, 2000, size=120)
    pairs = all_pairs(120)
    for nparts in (1, 2, 3, 8):
        shards = partition_pairs(lens, pairs, nparts)
        allidx = np.sort(np.concatenate(shards))
        assert np.array_equal(allidx, np.arange(len(pairs)))
        work = lens[pairs[:, 0]].astype(np.int64) * lens[pairs[:, 1]]
        loads = np.array([work[s].sum() for s in shards])
        assert loads.max() - loads.min() <= work.max()


def _rank_main(rank, world, port, out_path):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    import sys

    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from clustalw_gb300.shard import sharded_pairwise
    from clustalw_gb300.synth import all_pairs

    seqs = _seqs_full()
    res = sharded_pairwise(seqs, all_pairs(37), full_align, group=dist.group.WORLD)
    if rank == 0:
        np.save(out_path, res)
    else:
        assert res is None
    dist.destroy_process_group()


def test_two_gloo_ranks_assemble_the_full_result(tmp_path):
    import socket

    from clustalw_gb300.synth import all_pairs

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "d.npy")
    mp.spawn(_rank_main, args=(2, port, out), nprocs=2, join=True)
    want = full_align(_seqs_full(), all_pairs(37))
    got = np.load(out)
    assert got.dtype == np.float32
    assert np.array_equal(got.view(np.int32), want.view(np.int32))


def quick_align(seqs, pairs):
    """Quick k-tuple distances (float64) from the oracle: the sharded path must
    keep them bit for bit."""
    from oracle import oracle

    fp = dict(dna=0, ktup=1, window=5, window_gap=3, signif=5, percent=1, max_aa=24,
              max_aln_length=2 * max(len(s) for s in seqs))
    return oracle.fast_pairs(seqs, fp, pairs, nthreads=1)["dist"]


def _rank_main_quick(rank, world, port, out_path):
    import sys

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, here)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from clustalw_gb300.shard import sharded_pairwise
    from clustalw_gb300.synth import all_pairs, protein_family

    seqs = protein_family(14, 120, 3)
    res = sharded_pairwise(seqs, all_pairs(len(seqs)), quick_align, group=dist.group.WORLD)
    if rank == 0:
        np.save(out_path, res)
    dist.destroy_process_group()


def test_two_gloo_ranks_keep_quick_distances_exact(tmp_path):
    import socket

    from clustalw_gb300.synth import all_pairs, protein_family

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    out = str(tmp_path / "q.npy")
    mp.spawn(_rank_main_quick, args=(2, port, out), nprocs=2, join=True)
    seqs = protein_family(14, 120, 3)
    want = quick_align(seqs, all_pairs(len(seqs)))
    got = np.load(out)
    assert got.dtype == np.float64
    assert np.array_equal(got.view(np.int64), want.view(np.int64))
