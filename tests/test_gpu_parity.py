"""GPU parity: the sm_103a kernels, called through the C ABI, against the
reference's distance matrices (golden fixtures, bit-exact) and against the
oracle's per-pair intermediates (forward max score, end cell, start cell,
Myers-Miller score, identity and match counts)."""
import numpy as np
import pytest

from conftest import (big_golden_names, golden_names, load_big_extra, load_big_golden, load_golden,
                      pw_variant_names, range_pairs)

pytestmark = pytest.mark.gpu

STAT_FIELDS = ["fwd_score", "se1", "se2", "sb1", "sb2", "mm_score", "n_ident", "n_match"]


@pytest.fixture(scope="module")
def ctx():
    from clustalw_gb300 import native

    c = native.Context(0)
    yield c
    c.close()


def setup(ctx, g):
    ctx.set_matrix(g["matrix"])
    ctx.set_params(g["params"])
    ctx.upload_seqs(g["seqs"])


@pytest.mark.parametrize("name", golden_names())
def test_distmatrix_bit_exact_vs_reference(ctx, name):
    g = load_golden(name)
    setup(ctx, g)
    n = len(g["seqs"])
    elements = np.zeros_like(g["elements"])
    ctx.pairwise_align(*g["range"], elements, n + 1)
    bad = np.nonzero(elements != g["elements"])[0]
    assert len(bad) == 0, f"{name}: {len(bad)} of {len(elements)} entries differ, first {bad[:5]}"


@pytest.mark.parametrize("name", golden_names())
def test_pair_stats_vs_oracle(ctx, oracle_mod, name):
    g = load_golden(name)
    setup(ctx, g)
    pairs = range_pairs(len(g["seqs"]), *g["range"])
    if len(pairs) == 0:
        pytest.skip("empty range")
    dist, st = ctx.align_pairs(pairs, stats=True)
    want = oracle_mod.align_pairs(g["seqs"], g["matrix"], g["params"], pairs)
    assert np.array_equal(dist, want["dist"])
    for f in STAT_FIELDS:
        bad = np.nonzero(st[f] != want[f])[0]
        assert len(bad) == 0, f"{name}.{f}: {len(bad)} pairs differ, e.g. pair {pairs[bad[0]]}: gpu {st[f][bad[0]]} oracle {want[f][bad[0]]}"


@pytest.mark.parametrize("name", pw_variant_names())
def test_distmatrix_other_matrices_and_gap_penalties(ctx, oracle_mod, name):
    """The reference's DistMatrix under the BLOSUM, PAM and identity pairwise
    matrices and non-default gap penalties (protein and DNA, one DNA set with
    gap extension 0), read as FullPairwiseAlign.cpp:69-94, 129-148 read them:
    bit-exact through the range call, and every per-pair intermediate equals
    the oracle's. These stress the shifted E/F carry (gap open + extension)
    and the int16 score profile with other matrix ranges."""
    g = load_golden(name)
    setup(ctx, g)
    n = len(g["seqs"])
    elements = np.zeros_like(g["elements"])
    ctx.pairwise_align(*g["range"], elements, n + 1)
    bad = np.nonzero(elements != g["elements"])[0]
    assert len(bad) == 0, f"{name}: {len(bad)} of {len(elements)} entries differ, first {bad[:5]}"
    pairs = range_pairs(n, *g["range"])
    dist, st = ctx.align_pairs(pairs, stats=True)
    want = oracle_mod.align_pairs(g["seqs"], g["matrix"], g["params"], pairs)
    assert np.array_equal(dist, want["dist"])
    for f in STAT_FIELDS:
        bad = np.nonzero(st[f] != want[f])[0]
        assert len(bad) == 0, f"{name}.{f}: pair {pairs[bad[0]]} gpu {st[f][bad[0]]} oracle {want[f][bad[0]]}"


def test_plain_form_matches_batched(ctx):
    g = load_golden("synth_uneven_40")
    setup(ctx, g)
    pairs = range_pairs(len(g["seqs"]), 0, 40, 0, 40)[::7]
    d1, s1 = ctx.align_pairs(pairs, stats=True)
    d2, s2 = ctx.align_pairs(pairs, stats=True, plain=True)
    assert np.array_equal(d1, d2)
    assert np.array_equal(s1, s2)


def test_plan_replay_is_idempotent(ctx):
    g = load_golden("synth_protein_60x97")
    setup(ctx, g)
    pairs = range_pairs(60, 0, 60, 0, 60)
    plan = ctx.plan(pairs)
    plan.launch()
    a = plan.results()
    plan.launch()
    plan.launch()
    b = plan.results()
    plan.close()
    assert np.array_equal(a, b)


def test_swapped_pair_order(ctx, oracle_mod):
    """(sj, si) is a different alignment problem (seq1/seq2 roles swap); both
    orders must match the oracle."""
    g = load_golden("synth_uneven_40")
    setup(ctx, g)
    pairs = range_pairs(40, 0, 40, 0, 40)[:200][:, ::-1].copy()
    dist, st = ctx.align_pairs(pairs, stats=True)
    want = oracle_mod.align_pairs(g["seqs"], g["matrix"], g["params"], pairs)
    assert np.array_equal(dist, want["dist"])
    for f in STAT_FIELDS:
        assert np.array_equal(st[f], want[f]), f


@pytest.mark.parametrize("name", ["synth_uneven_40", "fixture_100_97", "synth_long_6x3000", "edge_protein"])
def test_cell_counts_match_oracle(ctx, oracle_mod, name):
    """The kernel's algorithmic cell counters equal the reference's own
    inner-loop iteration counts (forwardPass, reversePass up to its break, diff)."""
    g = load_golden(name)
    setup(ctx, g)
    pairs = range_pairs(len(g["seqs"]), *g["range"])
    plan = ctx.plan(pairs)
    plan.launch()
    fwd, rev, dif = plan.cell_counts()
    plan.close()
    want = oracle_mod.align_pairs(g["seqs"], g["matrix"], g["params"], pairs)
    assert (fwd, rev, dif) == (int(want["cells_fwd"].sum()), int(want["cells_rev"].sum()), int(want["cells_diff"].sum()))


def test_short_and_long_pair_kernels_at_the_boundary(ctx, oracle_mod):
    """Pairs whose first sequence has <= 128 residues run in the 4-rows-per-lane
    kernel, the rest in the 8-row kernel, both inside one plan. Lengths around
    the 128-row split and the 32/64-row stripe edges, in both pair orders,
    must match the oracle field for field."""
    from clustalw_gb300 import load_matrix, synth

    matrix, params = load_matrix("protein")
    base = synth.protein_family(16, 300, seed=11)
    lens = [1, 2, 31, 32, 33, 63, 64, 65, 127, 128, 129, 130, 255, 256, 257, 300]
    seqs = [s[:L] if len(s) >= L else np.concatenate([s, s])[:L] for s, L in zip(base, lens)]
    ctx.set_matrix(matrix)
    ctx.set_params(params)
    ctx.upload_seqs(seqs)
    pairs = range_pairs(len(seqs), 0, len(seqs), 0, len(seqs))
    pairs = np.concatenate([pairs, pairs[:, ::-1]]).astype(np.int32)
    plan = ctx.plan(pairs)
    assert plan.kernel_count() == 2
    plan.launch()
    dist, st = plan.results(stats=True)
    fwd, rev, dif = plan.cell_counts()
    plan.close()
    want = oracle_mod.align_pairs(seqs, matrix, params, pairs)
    assert np.array_equal(dist.view(np.int32), want["dist"].view(np.int32))
    for f in STAT_FIELDS:
        bad = np.nonzero(st[f] != want[f])[0]
        assert len(bad) == 0, f"{f}: pair {pairs[bad[0]]} gpu {st[f][bad[0]]} oracle {want[f][bad[0]]}"
    assert (fwd, rev, dif) == (int(want["cells_fwd"].sum()), int(want["cells_rev"].sum()), int(want["cells_diff"].sum()))
    d_plain, s_plain = ctx.align_pairs(pairs, stats=True, plain=True)
    assert np.array_equal(d_plain, dist) and np.array_equal(s_plain, st)


@pytest.mark.parametrize("name,kernels", [("fixture_100_97", 1), ("fixture_100_498", 1), ("synth_uneven_40", 2)])
def test_plan_kernel_count(ctx, name, kernels):
    g = load_golden(name)
    setup(ctx, g)
    plan = ctx.plan(range_pairs(len(g["seqs"]), *g["range"]))
    assert plan.kernel_count() == kernels
    plan.close()


def test_one_shot_calls_reuse_buffers(ctx, oracle_mod):
    """cwgpu_align_pairs keeps grow-only device arrays in the context: calls of
    growing and shrinking sizes, with and without stats, and a re-upload of
    other sequences in between, all give the oracle's results."""
    g = load_golden("synth_uneven_40")
    setup(ctx, g)
    pairs = range_pairs(40, 0, 40, 0, 40)
    want = oracle_mod.align_pairs(g["seqs"], g["matrix"], g["params"], pairs)
    for sl in (slice(0, 50), slice(0, len(pairs)), slice(100, 130), slice(0, 1)):
        d = ctx.align_pairs(pairs[sl])
        assert np.array_equal(d, want["dist"][sl])
        d, st = ctx.align_pairs(pairs[sl], stats=True)
        assert np.array_equal(d, want["dist"][sl]) and np.array_equal(st["mm_score"], want["mm_score"][sl])
    h = load_golden("synth_protein_60x97")
    setup(ctx, h)
    p2 = range_pairs(60, 0, 60, 0, 60)
    d = ctx.align_pairs(p2)
    assert np.array_equal(d, oracle_mod.align_pairs(h["seqs"], h["matrix"], h["params"], p2)["dist"])


@pytest.mark.parametrize("short_rows", [0, 64, 300, 65535])
def test_short_rows_knob_keeps_results(ctx, oracle_mod, short_rows):
    """The short-pair threshold moves pairs between the 4-row and 8-row
    kernels (0: none short, 65535: all short); results stay the oracle's."""
    g = load_golden("synth_uneven_40")
    setup(ctx, g)
    pairs = range_pairs(40, 0, 40, 0, 40)
    old = ctx.get_tuning()
    ctx.set_tuning(old[0], old[1], short_rows)
    try:
        d, st = ctx.align_pairs(pairs, stats=True)
        plan = ctx.plan(pairs)
        kernels = plan.kernel_count()
        plan.launch()
        d2 = plan.results()
        plan.close()
    finally:
        ctx.set_tuning(*old)
    want = oracle_mod.align_pairs(g["seqs"], g["matrix"], g["params"], pairs)
    assert np.array_equal(d, want["dist"]) and np.array_equal(d2, want["dist"])
    for f in STAT_FIELDS:
        assert np.array_equal(st[f], want[f]), f
    assert kernels == (1 if short_rows in (0, 65535) else 2)


def test_autotune_picks_all_knobs(ctx):
    from clustalw_gb300 import autotune

    g = load_golden("synth_uneven_40")
    setup(ctx, g)
    pairs = range_pairs(40, 0, 40, 0, 40)
    lens = [len(s) for s in g["seqs"]]
    before = ctx.align_pairs(pairs)
    choice, timings = autotune.tune(ctx, lens, pairs, target_cells=2e8, use_cache=False, repeats=1)
    assert len(choice) == 3 and ctx.get_tuning() == tuple(choice)
    assert len({c[2] for c in timings}) >= 2  # short-pair thresholds were timed
    assert np.array_equal(ctx.align_pairs(pairs), before)
    ctx.set_tuning(32, 16, 128)


def test_short_pair_kernel_dna(ctx, oracle_mod):
    """DNA (IUB, dense alphabet of 4-5 codes) through the 4-row kernel:
    a family of ~100 residues, every pair short."""
    from clustalw_gb300 import load_matrix, synth

    matrix, params = load_matrix("dna")
    seqs = synth.dna_family(30, 100, seed=21)
    assert max(len(s) for s in seqs) <= 128
    ctx.set_matrix(matrix)
    ctx.set_params(params)
    ctx.upload_seqs(seqs)
    pairs = range_pairs(len(seqs), 0, len(seqs), 0, len(seqs))
    plan = ctx.plan(pairs)
    assert plan.kernel_count() == 1
    plan.launch()
    dist, st = plan.results(stats=True)
    plan.close()
    want = oracle_mod.align_pairs(seqs, matrix, params, pairs)
    assert np.array_equal(dist, want["dist"])
    for f in STAT_FIELDS:
        assert np.array_equal(st[f], want[f]), f


def test_maximum_length_sequences(oracle_mod):
    """Sequences at the length limit (CWGPU_MAX_SEQ_LEN = 65,535 residues): a
    300-residue fragment (long-pair kernel) and a 99-residue one (short-pair
    kernel) against the full-length sequence in both orders, and a pair of
    about 16,000 residues whose Myers-Miller stage recurses 14 levels deep;
    every distance and intermediate equals the oracle's. One residue more is
    rejected at upload. A context of its own: its scratch rows are sized for
    65,536 columns."""
    from clustalw_gb300 import load_matrix, native, synth

    seqs = synth.length_limit_set()
    assert len(seqs[0]) == 65535 and len(seqs[4]) <= 128 < len(seqs[1])
    matrix, params = load_matrix("protein")
    c = native.Context(0)
    try:
        c.set_matrix(matrix)
        c.set_params(params)
        with pytest.raises(native.CwgpuError):
            c.upload_seqs([np.resize(seqs[0], 65536)])
        c.upload_seqs(seqs)
        pairs = np.array([[0, 1], [1, 0], [4, 0], [0, 4], [2, 3], [3, 2]], dtype=np.int32)
        dist, st = c.align_pairs(pairs, stats=True)
    finally:
        c.close()
    want = oracle_mod.align_pairs(seqs, matrix, params, pairs)
    assert np.array_equal(dist, want["dist"])
    for f in STAT_FIELDS:
        assert np.array_equal(st[f], want[f]), f
    assert want["se1"][4] - want["sb1"][4] > 8192  # the deep Myers-Miller box


@pytest.mark.parametrize("name", big_golden_names())
def test_full_size_reference_fixture(ctx, name):
    """The reference's own 1000-sequence test sets (test_data/correct), the
    whole DistMatrix through the drop-in range call: its SHA-256 equals that
    of the matrix the unmodified reference filled, and so do sampled entries.
    Then the guide tree on it and the quick k-tuple distances of the same
    set, each against what the unmodified NJTree / FastPairwiseAlign leave."""
    import hashlib

    g = load_big_golden(name)
    setup(ctx, g)
    n = len(g["seqs"])
    elements = np.zeros(g["n_elements"])
    ctx.pairwise_align(*g["range"], elements, n + 1)
    assert np.array_equal(elements[g["sample_idx"]].view(np.int64), g["sample_val"].view(np.int64))
    assert hashlib.sha256(np.ascontiguousarray(elements, dtype="<f8").tobytes()).digest() == g["sha256"]
    x = load_big_extra(name)
    if x is None:
        return
    # The guide tree on that matrix, as the reference's NJTree leaves it.
    from clustalw_gb300.tree import NJGpu

    nj = NJGpu(0)
    left, right, desc, _ = nj.tree(n, elements)
    nj.close()
    h = hashlib.sha256()
    for a in (left.astype("<f8"), right.astype("<f8"), desc.astype("<i4"), elements.astype("<f8")):
        h.update(np.ascontiguousarray(a).tobytes())
    assert h.digest() == x["nj_sha256"]
    # The quick k-tuple distances of the same sequences, as FastPairwiseAlign fills them.
    quick = np.zeros(g["n_elements"])
    ctx.fast_pairwise_align(x["fast_params"], *g["range"], quick, n + 1)
    assert np.array_equal(quick[x["fast_sample_idx"]].view(np.int64), x["fast_sample_val"].view(np.int64))
    assert hashlib.sha256(np.ascontiguousarray(quick, dtype="<f8").tobytes()).digest() == x["fast_sha256"]
