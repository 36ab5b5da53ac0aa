"""The four benchmark workloads at full size (protein 100 x 97, protein
1000 x 1523, uneven protein 8 families x 125, DNA 2000 x 1000), every pair on
the GPU through a plan: the SHA-256 of all distances and of all per-pair
intermediates (forward max score, end cell, start cell, Myers-Miller score,
identities, aligned pairs) equals the oracle's over the whole set
(tests/golden/make_bench_golden.py, which stores the sequences themselves),
and so do the totals of the three sweeps' cell counts and a sample of pairs.
A second launch of the same plan gives the same distances."""
import hashlib
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

STAT_FIELDS = ["fwd_score", "se1", "se2", "sb1", "sb2", "mm_score", "n_ident", "n_match"]
NAMES = ["protein-100x97", "protein-1000x1523", "protein-uneven-8x125", "dna-2000x1000"]


def load_bench_golden(name):
    z = np.load(os.path.join(GOLDEN, "bench_" + name.replace("-", "_") + ".npz"))
    lens = z["lens"]
    offs = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int64)
    seqs = [z["codes"][o : o + L].astype(np.int8) for o, L in zip(offs, lens)]
    return dict(seqs=seqs, kind=str(z["kind"]), npairs=int(z["npairs"]), dist_sha256=bytes(z["dist_sha256"]),
                stats_sha256=bytes(z["stats_sha256"]), cells=[int(c) for c in z["cells"]],
                sample_idx=z["sample_idx"], sample_dist=z["sample_dist"], sample_stats=z["sample_stats"])


@pytest.mark.parametrize("name", NAMES)
def test_full_size_workload_whole_set(name):
    from clustalw_gb300 import load_matrix, native, synth

    g = load_bench_golden(name)
    seqs = g["seqs"]
    matrix, params = load_matrix(g["kind"])
    pairs = synth.all_pairs(len(seqs))
    assert len(pairs) == g["npairs"]
    with native.Context(0) as ctx:
        ctx.set_matrix(matrix)
        ctx.set_params(params)
        ctx.upload_seqs(seqs)
        plan = ctx.plan(pairs)
        plan.launch()
        d1, st = plan.results(stats=True)
        cells = list(plan.cell_counts())
        plan.launch()
        d2 = plan.results()
        plan.close()
    assert np.array_equal(d1.view(np.int32), d2.view(np.int32))
    stats = np.stack([st[f].astype("<i4") for f in STAT_FIELDS], axis=1)
    idx = g["sample_idx"]
    assert np.array_equal(d1[idx].view(np.int32), g["sample_dist"].view(np.int32))
    assert np.array_equal(stats[idx], g["sample_stats"])
    assert cells == g["cells"]
    assert hashlib.sha256(d1.astype("<f4").tobytes()).digest() == g["dist_sha256"]
    assert hashlib.sha256(np.ascontiguousarray(stats).tobytes()).digest() == g["stats_sha256"]
