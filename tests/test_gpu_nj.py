"""GPU guide tree (include/cwgpu_nj.h) against the reference NJTree::generateTree
(tree/NJTree.cpp:161-748): bit-exact on the reference-generated fixtures and,
at sizes the reference-pinned oracle finishes in seconds, on seeded matrices
including tie-heavy ones. Every comparison is of the raw float64 bits."""
import numpy as np
import pytest

from conftest import load_nj_golden, nj_golden_names

pytestmark = pytest.mark.gpu


def same_bits(a, b):
    return np.array_equal(np.asarray(a, np.float64).view(np.int64), np.asarray(b, np.float64).view(np.int64))


@pytest.fixture(scope="module")
def nj():
    from clustalw_gb300.tree import NJGpu

    g = NJGpu(0)
    yield g
    g.close()


def random_matrix(n, seed, ties=False):
    """Packed DistMatrix of n sequences: float32-valued distances (what the
    pairwise stage stores) with clustered structure; with ties=True many equal
    values and zero distances."""
    rng = np.random.default_rng(seed)
    el = np.zeros((n + 1) * (n + 2) // 2)
    pos = rng.normal(size=(n, 3))
    grp = rng.integers(0, max(2, n // 8), size=n)
    for j in range(2, n + 1):
        a = j - 1
        i = np.arange(1, j)
        if ties:
            v = np.where(grp[i - 1] == grp[j - 1], 0.0, 0.05 * (1 + (grp[i - 1] + grp[j - 1]) % 5))
        else:
            v = np.linalg.norm(pos[i - 1] - pos[j - 1], axis=1) / 6.0 + rng.uniform(0, 0.05, size=j - 1)
        el[a * (a + 1) // 2 + (i - 1)] = np.minimum(v, 1.0).astype(np.float32)
    return el


def check(nj, oracle_mod, n, el):
    want = oracle_mod.nj_tree(n, el.copy(), want_joins=True)
    got_el = el.copy()
    left, right, desc, joins = nj.tree(n, got_el, want_joins=True)
    assert same_bits(left, want[0])
    assert same_bits(right, want[1])
    assert np.array_equal(desc, want[2])
    assert same_bits(got_el, want[3])
    assert np.array_equal(joins, want[4])
    return joins


@pytest.mark.parametrize("name", nj_golden_names())
def test_gpu_nj_matches_reference_fixtures(nj, name):
    g = load_nj_golden(name)
    n = int(g["n"])
    el = g["elements"].copy()
    left, right, desc, _ = nj.tree(n, el)
    assert same_bits(left, g["left"])
    assert same_bits(right, g["right"])
    assert np.array_equal(desc, g["desc"])
    assert same_bits(el, g["elements_after"])


@pytest.mark.parametrize("n,seed,ties", [(3, 1, False), (4, 2, True), (17, 3, False), (150, 4, True),
                                         (257, 5, False), (600, 6, False), (600, 7, True),
                                         (1000, 8, False)])
def test_gpu_nj_matches_oracle_seeded(nj, oracle_mod, n, seed, ties):
    check(nj, oracle_mod, n, random_matrix(n, seed, ties))


def test_gpu_nj_node_arrays_in_global_memory(nj, oracle_mod):
    """Above about 4,370 sequences CTA 0's per-node arrays (sums, joins, the
    two lists of valid nodes) no longer fit shared memory and live in global
    memory; the tree is still the oracle's."""
    check(nj, oracle_mod, 4400, random_matrix(4400, 9))


def test_gpu_nj_bounded_wait_ends_with_timeout_status(nj, oracle_mod):
    """A wait between CTAs whose counter nothing raises ends at its limit
    (here 2 ms) with the timeout status instead of hanging, and the handle
    still builds a correct tree afterwards."""
    import time

    t = time.perf_counter()
    assert nj.wait_probe(2_000_000)
    assert time.perf_counter() - t < 5.0
    check(nj, oracle_mod, 40, random_matrix(40, 12))


def test_gpu_nj_first_join_is_first_minimum(nj):
    """The first cycle's join is the first minimum of the criterion in the
    reference's scan order, recomputed here in float64 with the same
    expression order."""
    n = 40
    el = random_matrix(n, 11, ties=True)

    def d(i, j):
        a, b = max(i, j) - 1, min(i, j) - 1
        return el[a * (a + 1) // 2 + b]

    rows = [0.0] * (n + 1)
    cols = [0.0] * (n + 1)
    for j in range(1, n + 1):
        s = 0.0
        for i in range(1, j):
            s = s + d(i, j)
        rows[j] = s
        s = 0.0
        for i in range(j + 1, n + 1):
            s = s + d(j, i)
        cols[j] = s
    sumd = 0.0
    for j in range(1, n + 1):
        sumd = sumd + cols[j]
    f = float(n - 2)
    best, arg = 99999.0 * 2.0 * f, None
    for jj in range(2, n + 1):
        for ii in range(1, jj):
            t = f * d(ii, jj) + 2.0 * sumd - (cols[ii] + rows[ii]) - (cols[jj] + rows[jj])
            if t < best:
                best, arg = t, (ii, jj)
    _, _, _, joins = nj.tree(n, el.copy(), want_joins=True)
    assert tuple(joins[0]) == arg


@pytest.mark.parametrize("name", ["nj_fixture_100_97", "nj_ties_30", "nj_random_4"])
def test_gpu_nj_verbose_report_matches_reference(nj, name):
    """NJTree.generateTree with a report stream writes the reference's own
    verbose report (NJTree.cpp:209-236, 413-470, 694-740)."""
    import io

    from clustalw_gb300.pairwise import DistMatrix
    from clustalw_gb300.tree import NJTree, PhyloTree, SeqInfo

    g = load_nj_golden(name)
    n = int(g["n"])
    dm = DistMatrix(n + 1)
    dm.getElements()[:] = g["elements"]
    algo = NJTree(gpu=nj)
    algo.setVerbose(True)
    out = io.StringIO()
    algo.generateTree(PhyloTree(), dm, SeqInfo(1, n, n), out)
    assert out.getvalue() == str(g["report"])


def test_gpu_nj_two_sequences_untouched(nj):
    from clustalw_gb300.tree import NJTree, PhyloTree, SeqInfo
    from clustalw_gb300.pairwise import DistMatrix

    dm = DistMatrix(3)
    dm.SetAt(1, 2, 0.25)
    before = dm.getElements().copy()
    tree = PhyloTree()
    NJTree(gpu=nj).generateTree(tree, dm, SeqInfo(1, 2, 2))
    assert same_bits(dm.getElements(), before)
    assert tree.leftBranch.size == 0


def test_gpu_nj_plugin_interface(nj, oracle_mod):
    """NJTree.generateTree through the ClusterTreeAlgorithm mirror."""
    from clustalw_gb300.tree import NJTree, PhyloTree, SeqInfo
    from clustalw_gb300.pairwise import DistMatrix

    n = 120
    el = random_matrix(n, 21)
    dm = DistMatrix(n + 1)
    dm.getElements()[:] = el
    tree = PhyloTree()
    NJTree(gpu=nj).generateTree(tree, dm, SeqInfo(1, n, n))
    want = oracle_mod.nj_tree(n, el.copy())
    assert same_bits(tree.leftBranch, want[0]) and same_bits(tree.rightBranch, want[1])
    assert np.array_equal(tree.treeDesc, want[2])
    assert same_bits(dm.getElements(), want[3])


def test_gpu_nj_device_entry_point(nj, oracle_mod):
    torch = pytest.importorskip("torch")
    n = 300
    el = random_matrix(n, 31)
    want = oracle_mod.nj_tree(n, el.copy())
    dev = torch.device("cuda:0")
    d_in = torch.from_numpy(el).to(dev)
    d_out = torch.empty_like(d_in)
    d_left = torch.empty(n + 2, dtype=torch.float64, device=dev)
    d_right = torch.empty(n + 2, dtype=torch.float64, device=dev)
    d_desc = torch.empty((n + 1) * (n + 1), dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    for _ in range(2):  # the input stays untouched, so the call repeats
        nj.tree_device(n, d_in.data_ptr(), d_out.data_ptr(), d_left.data_ptr(), d_right.data_ptr(),
                       d_desc.data_ptr())
        assert same_bits(d_left.cpu().numpy(), want[0])
        assert same_bits(d_right.cpu().numpy(), want[1])
        assert np.array_equal(d_desc.cpu().numpy().reshape(n + 1, n + 1), want[2])
        assert same_bits(d_out.cpu().numpy(), want[3])
    assert same_bits(d_in.cpu().numpy(), el)
    pairs, secs = nj.last_stats()
    assert pairs == sum((n - k + 1) * (n - k) // 2 for k in range(1, n - 2)) and secs > 0


def test_gpu_nj_rejects_bad_sizes(nj):
    from clustalw_gb300.native import CwgpuError

    with pytest.raises(CwgpuError):
        nj.tree(1, np.zeros(3))
    buf = np.zeros(4)
    for n in (-1, 0, 16385):  # rejected before any pointer is read
        assert nj._lib.cwgpu_nj_tree(nj._h, n, buf.ctypes.data, buf.ctypes.data, buf.ctypes.data,
                                     buf.ctypes.data, None) == 1


def seq(x, s0=0.0):
    s = s0
    for v in x:
        s = s + float(v)  # one IEEE double addition per term, in order
    return s


def adversarial_terms(seed):
    rng = np.random.default_rng(seed)
    out = []
    # float32-valued distances: sums that round late, with exact ties
    out.append(rng.uniform(0, 1, 5000).astype(np.float32).astype(np.float64))
    # multiples of 0.05 and zeros: many rounding ties
    out.append((0.05 * rng.integers(0, 20, 4000)).astype(np.float32).astype(np.float64))
    # every term exactly half an ulp of the running sum: a tie at each step
    x = [1.0]
    for _ in range(300):
        x.append(2.0 ** -53)
    x += [2.0 ** -52 * 3] * 50
    out.append(np.array(x))
    # binade crossings from a tiny start, spread exponents, subnormals
    out.append(np.concatenate([[5e-324, 1e-310, 1e-300], np.logspace(-30, 10, 700)]))
    # negative terms, -0.0, a term larger than the sum, zeros
    y = rng.normal(size=1000)
    y[::37] = -0.0
    y[::53] = 0.0
    y[500] = 1e12
    out.append(y)
    # long chains of large and small magnitudes
    out.append(np.concatenate([rng.uniform(1e6, 2e6, 300), rng.uniform(0, 1e-9, 3000), rng.uniform(0, 1, 3000)]))
    # infinities and a NaN
    z = rng.uniform(0, 1, 200)
    z[100] = np.inf
    out.append(z)
    w = rng.uniform(0, 1, 100)
    w[10] = np.nan
    out.append(w)
    return out


@pytest.mark.parametrize("seed", [0, 1])
def test_gpu_sequential_sum_replay(nj, seed):
    """The warp replay of the reference's sequential sums, on terms built to
    hit every slow path: rounding ties, binade crossings, subnormals,
    negative terms, -0.0, infinities and NaN, and arbitrary starting sums."""
    for x in adversarial_terms(seed):
        for s0 in (0.0, 0.3, 1e-320):
            want = seq(x, s0)
            got = nj.seq_sum(x, s0)
            if np.isnan(want):
                assert np.isnan(got)
            else:
                assert np.float64(got).view(np.int64) == np.float64(want).view(np.int64)
    for count in range(0, 70):
        x = np.random.default_rng(count).uniform(0, 1, count)
        assert nj.seq_sum(x) == seq(x)
    # a long sum of float32-valued terms (ties and late rounding)
    x = np.random.default_rng(seed).uniform(0, 1, 9000).astype(np.float32).astype(np.float64)
    assert np.float64(nj.seq_sum(x, 0.3)).view(np.int64) == np.float64(seq(x, 0.3)).view(np.int64)
