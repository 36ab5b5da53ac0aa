"""GPU quick k-tuple distances (cwgpu_fast_*) against the reference
FastPairwiseAlign::pairwiseAlign (pairwise/FastPairwiseAlign.cpp:20-400):
bit-exact on the reference-generated fixtures and, with other parameter sets,
against the reference-pinned oracle on seeded sets, including tie-heavy
repeats (the reference's quicksort decides the selected diagonals) and the
"(Partial alignment)" fragment cut-off."""
import numpy as np
import pytest

from conftest import fast_golden_names, load_fast_golden, quick_limit_names, range_pairs, sym_index

pytestmark = pytest.mark.gpu


def same_bits(a, b):
    return np.array_equal(np.asarray(a, np.float64).view(np.int64), np.asarray(b, np.float64).view(np.int64))


@pytest.fixture(scope="module")
def ctx():
    from clustalw_gb300 import native

    c = native.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("name", fast_golden_names())
def test_gpu_fast_matches_reference_fixtures(name):
    """Through the FastPairwiseAlign plugin mirror, as Clustal::align calls it."""
    from clustalw_gb300.native import FastParams
    from clustalw_gb300.pairwise import Alignment, DistMatrix, FastPairwiseAlign

    g = load_fast_golden(name)
    n = len(g["seqs"])
    aln = Alignment(g["seqs"])
    dm = DistMatrix(n + 1)
    FastPairwiseAlign(FastParams.from_dict(g["fast_params"])).pairwiseAlign(aln, dm, *g["range"])
    assert same_bits(dm.getElements(), g["elements"]), f"{np.count_nonzero(dm.getElements() != g['elements'])} differ"


@pytest.mark.parametrize("name", quick_limit_names())
def test_gpu_fast_at_the_length_limit(ctx, oracle_mod, name):
    """The quick path at its 8191-residue limit (protein ktup 1, DNA ktup 2: an
    8191-residue sequence, a mutated copy and a fragment), against the
    DistMatrix the unmodified FastPairwiseAlign filled, bit for bit, and the
    oracle's per-pair score, fragment count and partial flag."""
    from clustalw_gb300.native import FastParams

    g = load_fast_golden(name)
    n = len(g["seqs"])
    assert max(len(s) for s in g["seqs"]) == 8191
    ctx.upload_seqs(g["seqs"])
    el = np.zeros_like(g["elements"])
    ctx.fast_pairwise_align(FastParams.from_dict(g["fast_params"]), *g["range"], el, n + 1)
    assert same_bits(el, g["elements"]), f"{np.count_nonzero(el != g['elements'])} differ"
    check(ctx, oracle_mod, g["seqs"], g["fast_params"])


def check(ctx, oracle_mod, seqs, fp, pairs=None):
    from clustalw_gb300 import native

    n = len(seqs)
    pairs = range_pairs(n, 0, n, 0, n) if pairs is None else pairs
    ctx.upload_seqs(seqs)
    got, st = ctx.fast_align_pairs(pairs, native.FastParams.from_dict(fp), stats=True)
    want = oracle_mod.fast_pairs(seqs, fp, pairs)
    assert same_bits(got, want["dist"]), f"{np.count_nonzero(got != want['dist'])} of {len(pairs)} differ"
    assert np.array_equal(st["score"], want["score"])
    assert np.array_equal(st["frags"], want["frags"])
    assert np.array_equal(st["partial"], want["partial"])
    return st


def params(dna=0, ktup=1, window=5, window_gap=3, signif=5, percent=1, seqs=()):
    return dict(dna=dna, ktup=ktup, window=window, window_gap=window_gap, signif=signif, percent=percent, max_aa=24,
                max_aln_length=2 * max((len(s) for s in seqs), default=0))


@pytest.mark.parametrize("variant", [
    dict(), dict(ktup=2), dict(window=1), dict(window=9, signif=2), dict(signif=12), dict(window_gap=1),
    dict(window_gap=9), dict(percent=0),
])
def test_gpu_fast_protein_parameters(ctx, oracle_mod, variant):
    from clustalw_gb300 import synth

    seqs = synth.protein_family(24, 160, 31) + synth.protein_family(8, 40, 32)
    check(ctx, oracle_mod, seqs, params(seqs=seqs, **variant))


@pytest.mark.parametrize("ktup", [1, 2, 3, 4])
def test_gpu_fast_dna_ktup(ctx, oracle_mod, ktup):
    from clustalw_gb300 import synth

    seqs = synth.dna_family(20, 300, 41)
    check(ctx, oracle_mod, seqs, params(dna=1, ktup=ktup, window=4, window_gap=5, signif=4, seqs=seqs))


def test_gpu_fast_ties_need_the_reference_sort(ctx, oracle_mod):
    """Repeats give many diagonals with equal hit counts at the boundary of
    the top positions, where the reference's quicksort decides."""
    rng = np.random.default_rng(5)
    unit = rng.integers(0, 20, 7)
    seqs = []
    for k in range(16):
        s = np.tile(unit, 12 + k % 5)
        s[rng.integers(0, len(s), 3)] = rng.integers(0, 20, 3)
        seqs.append(s.astype(np.int8))
    check(ctx, oracle_mod, seqs, params(seqs=seqs))
    check(ctx, oracle_mod, seqs, params(signif=3, window=2, seqs=seqs))


def test_gpu_fast_partial_cutoff(ctx, oracle_mod):
    """A small max_aln_length makes the fragment count reach the reference's
    cut-off (2 * maxAlnLength) mid-pair."""
    from clustalw_gb300 import synth

    seqs = synth.protein_family(10, 300, 51)
    fp = params(seqs=seqs)
    fp["max_aln_length"] = 40
    st = check(ctx, oracle_mod, seqs, fp)
    assert st["partial"].sum() > 0


def test_gpu_fast_long_family(ctx, oracle_mod):
    """Long sequences: thousands of fragments per pair."""
    from clustalw_gb300 import synth

    seqs = synth.protein_family(8, 1523, 61)
    st = check(ctx, oracle_mod, seqs, params(seqs=seqs))
    assert st["frags"].max() > 1000


@pytest.mark.parametrize("ktup,window,signif,partial", [(2, 5, 5, False), (3, 20, 10, False), (2, 20, 10, True)])
def test_gpu_fast_list_tiers(ctx, oracle_mod, ktup, window, signif, partial):
    """The fragment list spans its three tiers (registers, shared records,
    global overflow): DNA families with wide windows give more fragments
    than fit the shared records (about lmax of them), with deep putFrag
    insertions among many off-diagonal fragments; the last case fills the
    list up to the reference's cut-off."""
    from clustalw_gb300 import synth

    seqs = synth.dna_family(6, 1200, 71)
    st = check(ctx, oracle_mod, seqs, params(dna=1, ktup=ktup, window=window, window_gap=5, signif=signif, seqs=seqs))
    assert st["frags"].max() > 1.3 * max(len(s) for s in seqs)
    assert bool(st["partial"].any()) == partial


def test_gpu_fast_device_entry_point(ctx, oracle_mod):
    torch = pytest.importorskip("torch")
    from clustalw_gb300 import native, synth

    seqs = synth.protein_family(30, 200, 71)
    fp = params(seqs=seqs)
    n = len(seqs)
    pairs = range_pairs(n, 0, n, 0, n)
    ctx.upload_seqs(seqs)
    want = oracle_mod.fast_pairs(seqs, fp, pairs)
    dev = torch.device("cuda:0")
    d_pairs = torch.from_numpy(pairs.astype(np.int32)).to(dev)
    order = np.argsort(-np.array([len(seqs[a]) * len(seqs[b]) for a, b in pairs]), kind="stable").astype(np.int32)
    d_order = torch.from_numpy(order).to(dev)
    d_dist = torch.zeros(len(pairs), dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    ctx.fast_align_pairs_device(native.FastParams.from_dict(fp), d_pairs.data_ptr(), d_order.data_ptr(), len(pairs),
                                d_dist.data_ptr())
    ctx.synchronize()
    assert same_bits(d_dist.cpu().numpy(), want["dist"])


def test_gpu_fast_range_and_errors(ctx, oracle_mod):
    from clustalw_gb300 import native, synth
    from clustalw_gb300.native import CwgpuError

    seqs = synth.protein_family(12, 90, 81)
    n = len(seqs)
    fp = params(seqs=seqs)
    ctx.upload_seqs(seqs)
    el = np.zeros((n + 1) * (n + 2) // 2)
    ctx.fast_pairwise_align(native.FastParams.from_dict(fp), 2, 9, 4, 11, el, n + 1)
    pairs = range_pairs(n, 2, 9, 4, 11)
    want = np.zeros_like(el)
    want[sym_index(pairs)] = oracle_mod.fast_pairs(seqs, fp, pairs)["dist"]
    assert same_bits(el, want)
    with pytest.raises(CwgpuError):  # wrong matrix size
        ctx.fast_pairwise_align(native.FastParams.from_dict(fp), 0, n, 0, n, el, n)
    with pytest.raises(CwgpuError):  # iEnd < iStart
        ctx.fast_pairwise_align(native.FastParams.from_dict(fp), 5, 2, 0, n, el, n + 1)
    with pytest.raises(CwgpuError):  # too many k-tuple codes
        ctx.fast_align_pairs([[0, 1]], native.FastParams.from_dict(dict(fp, ktup=4)))
