"""Writes whole-set golden fixtures for the four benchmark workloads
(protein 100 x 97, protein 1000 x 1523, uneven protein 8 families x 125,
DNA 2000 x 1000): the seeded synthetic sequences themselves (so the GPU host
does not depend on its numpy producing the same stream), and, over EVERY pair
of the set in the reference's loop order (si < sj, row-major), the SHA-256 of
the distances (little-endian float32) and of the eight per-pair intermediates
(forward max score, end cell, start cell, Myers-Miller score, identities,
aligned pairs; little-endian int32, one row of eight per pair), the totals of
the three sweeps' cell counts and a seeded sample of pairs with their values.

The values come from the oracle (oracle/oracle.c, the CPU restatement of
FullPairwiseAlign.cpp:34-660), which is pinned to the unmodified reference on
every reference fixture, including whole 1000-sequence DistMatrices by hash
(tests/test_oracle_golden.py). It runs on all host cores; the two largest sets
take about an hour of an 8-core host together.

Run from the repository root:
    python tests/golden/make_bench_golden.py [names...]
"""
import hashlib
import os
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
for _p in (REPO, os.path.join(REPO, "cuda-clustalw_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
STAT_FIELDS = ["fwd_score", "se1", "se2", "sb1", "sb2", "mm_score", "n_ident", "n_match"]
# name: (matrix kind, generator); seed 1 is the benchmark's default seed.
WORKLOADS = {
    "protein-100x97": ("protein", lambda synth: synth.protein_family(100, 97, 1)),
    "protein-1000x1523": ("protein", lambda synth: synth.protein_family(1000, 1523, 1)),
    "protein-uneven-8x125": ("protein", lambda synth: synth.uneven_protein(8, 125, 30, 2000, 1)),
    "dna-2000x1000": ("dna", lambda synth: synth.dna_family(2000, 1000, 1)),
}
SAMPLE = 2000


def stats_rows(res):
    return np.stack([res[f].astype("<i4") for f in STAT_FIELDS], axis=1)


def make(name, chunk=100_000):
    from clustalw_gb300 import load_matrix, synth

    kind, gen = WORKLOADS[name]
    seqs = gen(synth)
    matrix, params = load_matrix(kind)
    pairs = synth.all_pairs(len(seqs))
    h_dist, h_stats = hashlib.sha256(), hashlib.sha256()
    cells = np.zeros(3, dtype=np.int64)
    rng = np.random.default_rng(7)
    sample = np.sort(rng.choice(len(pairs), size=min(SAMPLE, len(pairs)), replace=False))
    s_dist = np.zeros(len(sample), dtype="<f4")
    s_stats = np.zeros((len(sample), len(STAT_FIELDS)), dtype="<i4")
    t0 = time.time()
    for a in range(0, len(pairs), chunk):
        b = min(len(pairs), a + chunk)
        res = O.align_pairs(seqs, matrix, params, pairs[a:b])
        h_dist.update(res["dist"].astype("<f4").tobytes())
        st = stats_rows(res)
        h_stats.update(np.ascontiguousarray(st).tobytes())
        cells += [int(res["cells_fwd"].sum()), int(res["cells_rev"].sum()), int(res["cells_diff"].sum())]
        sel = (sample >= a) & (sample < b)
        s_dist[sel] = res["dist"][sample[sel] - a]
        s_stats[sel] = st[sample[sel] - a]
        print(f"{name}: {b}/{len(pairs)} pairs, {time.time() - t0:.0f} s", flush=True)
    lens = np.array([len(s) for s in seqs], dtype=np.int32)
    codes = np.concatenate(seqs).astype(np.int8)
    path = os.path.join(OUT, "bench_" + name.replace("-", "_") + ".npz")
    np.savez_compressed(
        path,
        workload=np.array(name),
        kind=np.array(kind),
        codes=codes,
        lens=lens,
        npairs=np.int64(len(pairs)),
        dist_sha256=np.frombuffer(h_dist.digest(), dtype=np.uint8),
        stats_sha256=np.frombuffer(h_stats.digest(), dtype=np.uint8),
        cells=cells,
        sample_idx=sample.astype(np.int64),
        sample_dist=s_dist,
        sample_stats=s_stats,
    )
    print(f"{name}: wrote {path} ({time.time() - t0:.0f} s)", flush=True)


def main(argv):
    O.lib()
    for name in argv or list(WORKLOADS):
        make(name)


if __name__ == "__main__":
    main(sys.argv[1:])
