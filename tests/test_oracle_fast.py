"""The quick k-tuple distance restatement (oracle.c cwo_fast_pairs) against the
unmodified reference FastPairwiseAlign::pairwiseAlign
(pairwise/FastPairwiseAlign.cpp:20-400) on the reference's fixtures (protein
and DNA), a partial range, synthetic sets and protein/DNA edge cases
(tests/golden/fast_*.npz). Bit-exact: the reference stores a double."""
import numpy as np
import pytest

from conftest import fast_golden_names, load_fast_golden, quick_limit_names, quick_variant_names, range_pairs, sym_index


@pytest.mark.parametrize("name", fast_golden_names() + quick_limit_names() + quick_variant_names())
def test_fast_oracle_matches_reference(name, oracle_mod):
    g = load_fast_golden(name)
    n = len(g["seqs"])
    pairs = range_pairs(n, *g["range"])
    res = oracle_mod.fast_pairs(g["seqs"], g["fast_params"], pairs)
    want = np.zeros_like(g["elements"])
    if len(pairs):
        want[sym_index(pairs)] = res["dist"]
    assert np.array_equal(want.view(np.int64), g["elements"].view(np.int64)), \
        f"{name}: {np.count_nonzero(want != g['elements'])} entries differ"


def test_fast_fixtures_cover_the_branches(oracle_mod):
    """The fixtures exercise scored pairs, pairs with no fragment (distance 1.0)
    and both the protein (ktup 1) and DNA (ktup 2) parameter sets."""
    kinds, unscored = set(), 0
    for name in fast_golden_names():
        g = load_fast_golden(name)
        kinds.add((g["fast_params"]["dna"], g["fast_params"]["ktup"]))
        n = len(g["seqs"])
        res = oracle_mod.fast_pairs(g["seqs"], g["fast_params"], range_pairs(n, *g["range"]))
        unscored += int(np.count_nonzero(res["score"] == 0))
    assert kinds == {(0, 1), (1, 2)}
    assert unscored > 0
