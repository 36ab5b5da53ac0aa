"""Multi-GPU form of the distance stage: the N(N-1)/2 pairs are independent,
so they are split statically across ranks (one process per GPU) with no
collective on the data path; rank 0 assembles the DistMatrix from the shards.

This mirrors the reference fork's multi-GPU split, which hands each GPU's
OpenMP thread a static share of the pair list and lets every thread write its
own distances into the shared SymMatrix (GPU/cuda_clustalw_final/src/cuda/
cudaFullPairwiseAlign.cu:866-878, 977, 1025), but balances the shares by the
work of each pair (n*m) instead of by pair count.
"""
import numpy as np


def partition_pairs(lens, pairs, nparts):
    """Split pair indices into `nparts` shards of near-equal total n*m.

    Pairs are taken longest first and each goes to the currently lightest
    shard (greedy longest-processing-time); within a shard the indices keep
    that longest-first order, which is also the order the kernel's queue wants.
    Returns a list of int64 index arrays into `pairs`."""
    lens = np.asarray(lens, dtype=np.int64)
    pairs = np.asarray(pairs).reshape(-1, 2)
    work = lens[pairs[:, 0]] * lens[pairs[:, 1]]
    order = np.argsort(-work, kind="stable")
    load = np.zeros(nparts, dtype=np.int64)
    shards = [[] for _ in range(nparts)]
    for q in order:
        k = int(np.argmin(load))
        shards[k].append(int(q))
        load[k] += int(work[q])
    return [np.array(s, dtype=np.int64) for s in shards]


def sharded_pairwise(seqs, pairs, align_fn, group=None):
    """Run this rank's shard with `align_fn(seqs, pair_subset) -> distances`
    (float32 for the full stage, float64 for the quick k-tuple distances; the
    dtype is kept) and gather every shard's distances on rank 0 of `group` (a
    torch.distributed process group, or None for one process). Returns the
    full distance array on rank 0 and None elsewhere."""
    pairs = np.asarray(pairs, dtype=np.int32).reshape(-1, 2)
    lens = [len(s) for s in seqs]
    if group is None:
        return np.asarray(align_fn(seqs, pairs))
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    shards = partition_pairs(lens, pairs, world)
    mine = shards[rank]
    d = np.asarray(align_fn(seqs, pairs[mine]))
    gathered = [None] * world if rank == 0 else None
    dist.gather_object((mine, d), gathered, dst=0, group=group)
    if rank != 0:
        return None
    out = np.zeros(len(pairs), dtype=np.result_type(*[vals.dtype for _, vals in gathered]))
    for idx, vals in gathered:
        out[idx] = vals
    return out
