"""Full-size workloads of the benchmark configurations, run in full on the GPU:
a seeded sample of pairs is checked bit-exact against the oracle (distance and
every per-pair intermediate), and size-independent properties are checked on
all pairs: distances in [0, 1], identical results on a second launch, and the
forward-pass cell count equal to the sum of n*m."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = {
    "protein-1000x1523": ("protein", lambda synth: synth.protein_family(1000, 1523, 1)),
    "protein-uneven-8x125": ("protein", lambda synth: synth.uneven_protein(8, 125, 30, 2000, 1)),
    "dna-2000x1000": ("dna", lambda synth: synth.dna_family(2000, 1000, 1)),
}
STAT_FIELDS = ["fwd_score", "se1", "se2", "sb1", "sb2", "mm_score", "n_ident", "n_match"]


@pytest.mark.parametrize("name", sorted(CASES))
def test_full_size_workload(name, oracle_mod):
    from clustalw_gb300 import load_matrix, native, synth

    kind, make = CASES[name]
    matrix, params = load_matrix(kind)
    seqs = make(synth)
    pairs = synth.all_pairs(len(seqs))
    lens = np.array([len(s) for s in seqs], dtype=np.int64)
    with native.Context(0) as ctx:
        ctx.set_matrix(matrix)
        ctx.set_params(params)
        ctx.upload_seqs(seqs)
        plan = ctx.plan(pairs)
        plan.launch()
        d1, st = plan.results(stats=True)
        fwd, rev, dif = plan.cell_counts()
        plan.launch()
        d2 = plan.results()
        plan.close()
    assert np.array_equal(d1, d2)
    assert np.all((d1 >= 0) & (d1 <= 1))
    assert fwd == int((lens[pairs[:, 0]] * lens[pairs[:, 1]]).sum())
    rng = np.random.default_rng(2024)
    sample = np.sort(rng.choice(len(pairs), size=200, replace=False))
    want = oracle_mod.align_pairs(seqs, matrix, params, pairs[sample])
    assert np.array_equal(d1[sample], want["dist"])
    for f in STAT_FIELDS:
        assert np.array_equal(st[f][sample], want[f]), f
