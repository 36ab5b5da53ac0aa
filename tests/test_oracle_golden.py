"""The oracle restatement (oracle/oracle.c) against distance matrices written by
the unmodified reference on its own fixtures, partial ranges, synthetic sets and
edge cases (tests/golden/). Bit-exact: the reference stores a float in a double."""
import numpy as np
import pytest

from conftest import golden_names, load_golden, range_pairs, sym_index


@pytest.mark.parametrize("name", golden_names())
def test_oracle_matches_reference(name, oracle_mod):
    g = load_golden(name)
    n = len(g["seqs"])
    pairs = range_pairs(n, *g["range"])
    res = oracle_mod.align_pairs(g["seqs"], g["matrix"], g["params"], pairs)
    want = np.zeros_like(g["elements"])
    if len(pairs):
        want[sym_index(pairs)] = res["dist"].astype(np.float64)
    assert np.array_equal(want, g["elements"]), f"{name}: {np.count_nonzero(want != g['elements'])} entries differ"


def test_gap_penalties_match_reference_types(oracle_mod):
    """The float/double expression types of FullPairwiseAlign.cpp:129-148."""
    prot = load_golden("fixture_100_97")["params"]
    dna = load_golden("fixture_100_1002")["params"]
    assert oracle_mod.gap_penalties(dna, 1002, 1000) == (3000, 666)  # 6.66f*100 rounds to 666 in float
    assert oracle_mod.gap_penalties(prot, 97, 96)[1] == 1
    assert oracle_mod.gap_penalties(prot, 97, 97)[0] == 2390
    assert oracle_mod.gap_penalties(prot, 1523, 1600)[0] == 2841
