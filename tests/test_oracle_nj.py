"""The guide-tree restatement (oracle.c cwo_nj_tree) against the unmodified
reference NJTree::generateTree (tree/NJTree.cpp:161-748), run by
tests/golden/make_golden.py on the reference's own distance matrices, small
matrices (N = 3, 4, 5, 9) and a matrix full of ties. Bit-exact: branch lengths,
the treeDesc membership table and the distance matrix the reference leaves
behind (it joins in place)."""
import numpy as np
import pytest

from conftest import load_nj_golden, nj_golden_names


def same_bits(a, b):
    return np.array_equal(np.asarray(a, np.float64).view(np.int64), np.asarray(b, np.float64).view(np.int64))


@pytest.mark.parametrize("name", nj_golden_names())
def test_nj_oracle_matches_reference(name, oracle_mod):
    g = load_nj_golden(name)
    n = int(g["n"])
    left, right, desc, after = oracle_mod.nj_tree(n, g["elements"])
    assert same_bits(left, g["left"])
    assert same_bits(right, g["right"])
    assert np.array_equal(desc, g["desc"])
    assert same_bits(after, g["elements_after"])


def test_nj_golden_has_ties():
    """The tie fixture really exercises the first-minimum rule: several pairs
    share the minimum of the first cycle's criterion."""
    g = load_nj_golden("nj_ties_30")
    n = int(g["n"])
    el = g["elements"]

    def d(i, j):
        a, b = max(i, j) - 1, min(i, j) - 1
        return el[a * (a + 1) // 2 + b]

    r = [0.0] + [sum(d(i, j) for j in range(1, n + 1) if j != i) for i in range(1, n + 1)]
    s = sum(d(i, j) for j in range(1, n + 1) for i in range(1, j))
    tot = [(n - 2) * d(i, j) + 2 * s - r[i] - r[j] for j in range(2, n + 1) for i in range(1, j)]
    assert sum(1 for t in tot if t == min(tot)) > 1


@pytest.mark.parametrize("name", nj_golden_names())
def test_nj_report_matches_reference(name, oracle_mod):
    """The verbose cycle report the host mirror writes (from the joins and
    branch lengths) is the reference's own report, character for character."""
    from clustalw_gb300.tree import _REPORT_HEAD, nj_report

    g = load_nj_golden(name)
    n = int(g["n"])
    left, right, _, _, joins = oracle_mod.nj_tree(n, g["elements"], want_joins=True)
    assert _REPORT_HEAD + nj_report(n, joins, left, right) == str(g["report"])


@pytest.mark.parametrize("d", [0.0412371047, 0.0, 0.5, 1.0])
def test_two_sequence_tree_matches_reference(d, tmp_path, oracle_mod):
    """Two sequences: the reference writes one report line and returns before
    touching the tree (NJTree.cpp:218-229); the mirror's NJTree does the same
    without a device call. Report text against the unmodified reference."""
    import io
    import os

    from clustalw_gb300.pairwise import DistMatrix
    from clustalw_gb300.tree import NJTree, PhyloTree, SeqInfo

    if not os.path.exists(oracle_mod.REF_HARNESS):
        pytest.skip("reference harness not built")
    el = np.zeros(6)
    el[1] = float(np.float32(d))  # getIndex(1, 2): the float the pairwise stage stores
    *_, report = oracle_mod.run_reference_nj(2, el, str(tmp_path), report=True)
    dm = DistMatrix(3)
    dm.getElements()[:] = el
    tree, out = PhyloTree(), io.StringIO()
    nj = NJTree(gpu=object())  # never used for two sequences
    nj.setVerbose(True)
    nj.generateTree(tree, dm, SeqInfo(1, 2, 2), out)
    assert out.getvalue() == report
    assert len(tree.leftBranch) == 0 and len(tree.rightBranch) == 0
