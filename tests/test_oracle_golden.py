"""The oracle restatement (oracle/oracle.c) against distance matrices written by
the unmodified reference on its own fixtures, partial ranges, synthetic sets and
edge cases (tests/golden/). Bit-exact: the reference stores a float in a double."""
import numpy as np
import pytest

from conftest import golden_names, load_big_golden, load_golden, pw_variant_names, range_pairs, sym_index


@pytest.mark.parametrize("name", golden_names() + pw_variant_names())
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


def test_oracle_matches_reference_on_1000_97(oracle_mod):
    """The oracle on the reference's own 1000 x 97 test set, all 499,500
    pairs: the DistMatrix it fills hashes to what the unmodified reference
    filled (the larger compact fixtures are checked on the GPU only)."""
    import hashlib

    g = load_big_golden("big_1000_97")
    n = len(g["seqs"])
    pairs = range_pairs(n, *g["range"])
    r = oracle_mod.align_pairs(g["seqs"], g["matrix"], g["params"], pairs)
    el = np.zeros(g["n_elements"])
    si, sj = pairs[:, 0].astype(np.int64), pairs[:, 1].astype(np.int64)
    el[(sj * (sj + 1)) // 2 + si] = r["dist"].astype(np.float64)
    assert np.array_equal(el[g["sample_idx"]].view(np.int64), g["sample_val"].view(np.int64))
    assert hashlib.sha256(np.ascontiguousarray(el, dtype="<f8").tobytes()).digest() == g["sha256"]


@pytest.mark.parametrize("name", ["big_1000_498", "big_1000_1002", "big_1000_1523"])
def test_oracle_matches_reference_samples_full_size(oracle_mod, name):
    """The oracle on the 2,000 sampled pairs of the reference's larger
    1000-sequence sets (protein 498, DNA 1002 and 1523): each distance equals
    the entry the unmodified reference wrote."""
    g = load_big_golden(name)
    pairs = _pairs_of(g["sample_idx"])
    assert np.all((pairs[:, 0] >= 0) & (pairs[:, 0] < pairs[:, 1]))
    r = oracle_mod.align_pairs(g["seqs"], g["matrix"], g["params"], pairs)
    assert np.array_equal(r["dist"].astype(np.float64).view(np.int64), g["sample_val"].view(np.int64))


def _pairs_of(idx):
    """0-based (si, sj), si < sj, of packed DistMatrix entries (sj*(sj+1))/2 + si."""
    idx = np.asarray(idx, dtype=np.int64)
    sj = ((np.sqrt(8 * idx.astype(np.float64) + 1) - 1) // 2).astype(np.int64)
    sj += (sj + 1) * (sj + 2) // 2 <= idx  # guard the float square root at exact boundaries
    si = idx - sj * (sj + 1) // 2
    return np.stack([si, sj], axis=1).astype(np.int32)


@pytest.mark.parametrize("name", ["big_1000_97", "big_1000_498", "big_1000_1002", "big_1000_1523"])
def test_oracle_quick_matches_reference_samples_full_size(oracle_mod, name):
    """The oracle's quick k-tuple distances on the 2,000 sampled pairs of each
    of the reference's 1000-sequence sets equal what FastPairwiseAlign wrote."""
    from conftest import load_big_extra

    g = load_big_golden(name)
    x = load_big_extra(name)
    pairs = _pairs_of(x["fast_sample_idx"])
    r = oracle_mod.fast_pairs(g["seqs"], x["fast_params"], pairs)
    assert np.array_equal(np.asarray(r["dist"], np.float64).view(np.int64), x["fast_sample_val"].view(np.int64))


def test_oracle_tree_matches_reference_on_1000_97(oracle_mod):
    """The oracle's guide tree on the reference's 1000 x 97 DistMatrix (itself
    checked by hash above) hashes to what the unmodified NJTree leaves."""
    import hashlib

    from conftest import load_big_extra

    g = load_big_golden("big_1000_97")
    x = load_big_extra("big_1000_97")
    n = len(g["seqs"])
    pairs = range_pairs(n, *g["range"])
    r = oracle_mod.align_pairs(g["seqs"], g["matrix"], g["params"], pairs)
    el = np.zeros(g["n_elements"])
    si, sj = pairs[:, 0].astype(np.int64), pairs[:, 1].astype(np.int64)
    el[(sj * (sj + 1)) // 2 + si] = r["dist"].astype(np.float64)
    left, right, desc, el_after = oracle_mod.nj_tree(n, el)
    h = hashlib.sha256()
    for a in (np.asarray(left, "<f8"), np.asarray(right, "<f8"), np.asarray(desc, "<i4"), np.asarray(el_after, "<f8")):
        h.update(np.ascontiguousarray(a).tobytes())
    assert h.digest() == x["nj_sha256"]
