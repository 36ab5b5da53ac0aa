"""The oracle restatement (oracle/oracle.c) against distance matrices written by
the unmodified reference on its own fixtures, partial ranges, synthetic sets and
edge cases (tests/golden/). Bit-exact: the reference stores a float in a double."""
import os
import subprocess

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


@pytest.fixture(scope="module")
def oracle_1000_97(oracle_mod):
    """The oracle's whole DistMatrix of the reference's 1000 x 97 test set
    (499,500 pairs), computed once for the tests below."""
    g = load_big_golden("big_1000_97")
    n = len(g["seqs"])
    pairs = range_pairs(n, *g["range"])
    r = oracle_mod.align_pairs(g["seqs"], g["matrix"], g["params"], pairs)
    el = np.zeros(g["n_elements"])
    si, sj = pairs[:, 0].astype(np.int64), pairs[:, 1].astype(np.int64)
    el[(sj * (sj + 1)) // 2 + si] = r["dist"].astype(np.float64)
    return g, el


def test_oracle_matches_reference_on_1000_97(oracle_1000_97):
    """The oracle on the reference's own 1000 x 97 test set, all 499,500
    pairs: the DistMatrix it fills hashes to what the unmodified reference
    filled (the larger compact fixtures are checked on the GPU only)."""
    import hashlib

    g, el = oracle_1000_97
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


def test_oracle_tree_matches_reference_on_1000_97(oracle_mod, oracle_1000_97):
    """The oracle's guide tree on the reference's 1000 x 97 DistMatrix (itself
    checked by hash above) hashes to what the unmodified NJTree leaves."""
    import hashlib

    from conftest import load_big_extra

    g, el = oracle_1000_97
    x = load_big_extra("big_1000_97")
    n = len(g["seqs"])
    left, right, desc, el_after = oracle_mod.nj_tree(n, el.copy())
    h = hashlib.sha256()
    for a in (np.asarray(left, "<f8"), np.asarray(right, "<f8"), np.asarray(desc, "<i4"), np.asarray(el_after, "<f8")):
        h.update(np.ascontiguousarray(a).tobytes())
    assert h.digest() == x["nj_sha256"]


REF_TREE = os.environ.get("CLUSTALW_REF_ROOT", "/root/reference")
SHIPPED_DND = {
    # fixture -> the reference's shipped input / guide-tree pair (its own CPU outputs)
    "fixture_100_97": "test_data/correct/100_97",
    "fixture_100_498": "test_data/correct/100_498",
    "fixture_100_1002": "test_data/correct/100_1002",
    "fixture_100_1523": "test_data/correct/100_1523",
    "sequential_100_500": "CPU/clustalw-2.0.11/src/sequential/100_500",
    "sequential_100_1000": "CPU/clustalw-2.0.11/src/sequential/100_1000",
    "sequential_100_1800": "CPU/clustalw-2.0.11/src/sequential/100_1800",
    "big_1000_97": "test_data/correct/1000_97",
}


def _dnd_from(elements, n, base, tmp_path):
    from oracle import oracle as O

    dist = tmp_path / "in.dist"
    out = tmp_path / "out.dnd"
    with open(dist, "wb") as f:
        f.write(np.int32(n).tobytes())
        f.write(np.asarray(elements, "<f8").tobytes())
    subprocess.run([O.REF_HARNESS, "--dnd", base + ".fa", str(dist), str(out)], check=True,
                   stdout=subprocess.DEVNULL)
    return out.read_text()


@pytest.mark.skipif(not os.path.isdir(os.path.join(REF_TREE, "test_data")), reason="reference tree not present")
@pytest.mark.parametrize("name", sorted(SHIPPED_DND))
def test_distances_reproduce_the_shipped_guide_trees(name, tmp_path, oracle_mod, request):
    """The reference's shipped guide-tree files (.dnd, its own CPU outputs for
    these inputs) come out byte for byte when the reference's own tree code
    (UnRootedClusterTree::treeFromDistMatrix through oracle/_ref/refharness
    --dnd) runs on the DistMatrix the oracle reproduces: the stored fixture
    (equal to the oracle's, tested above) or, for 1000_97, the oracle's own."""
    from oracle import oracle as O

    if not os.path.exists(O.REF_HARNESS):
        pytest.skip("reference harness not built")
    base = os.path.join(REF_TREE, SHIPPED_DND[name])
    if name == "big_1000_97":
        g, el = request.getfixturevalue("oracle_1000_97")
        n = len(g["seqs"])
    else:
        g = load_golden(name)
        el, n = g["elements"], len(g["seqs"])
    with open(base + ".dnd") as f:
        want = f.read()
    assert _dnd_from(el, n, base, tmp_path) == want
