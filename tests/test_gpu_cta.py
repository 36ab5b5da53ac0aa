"""The one-CTA-per-pair form (k_pairwise_cta): the warps of a CTA share a
pair's forwardPass and reversePass stripes and its large Myers-Miller frames.
Its DistMatrix must equal the reference's and every per-pair intermediate and
cell count the oracle's, for every warp count and frame threshold; launches
with few long pairs take it by default; its hand-over wait ends at its bound
with the timeout status and leaves the context usable."""
import numpy as np
import pytest

from conftest import load_golden, range_pairs

pytestmark = pytest.mark.gpu

STAT_FIELDS = ["fwd_score", "se1", "se2", "sb1", "sb2", "mm_score", "n_ident", "n_match"]
ALWAYS = 2**31 - 1


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


def check_vs_oracle(ctx, oracle_mod, g, pairs):
    plan = ctx.plan(pairs)
    plan.launch()
    dist, st = plan.results(stats=True)
    cells = plan.cell_counts()
    plan.close()
    want = oracle_mod.align_pairs(g["seqs"], g["matrix"], g["params"], pairs)
    assert np.array_equal(dist.view(np.int32), want["dist"].view(np.int32))
    for f in STAT_FIELDS:
        bad = np.nonzero(st[f] != want[f])[0]
        assert len(bad) == 0, f"{f}: pair {pairs[bad[0]]} gpu {st[f][bad[0]]} oracle {want[f][bad[0]]}"
    assert cells == (int(want["cells_fwd"].sum()), int(want["cells_rev"].sum()), int(want["cells_diff"].sum()))


@pytest.mark.parametrize("name", ["synth_long_6x3000", "fixture_100_1523", "limit_deep_16384", "edge_protein",
                                  "synth_uneven_40", "range_100_97_cols49"])
def test_cta_form_bit_exact(ctx, oracle_mod, name):
    """Every long pair through the CTA form: the range call's DistMatrix equals
    the reference's, and intermediates and cell counts equal the oracle's."""
    g = load_golden(name)
    setup(ctx, g)
    old = ctx.get_cta_tuning()
    ctx.set_cta_tuning(max_pairs=ALWAYS)
    try:
        n = len(g["seqs"])
        elements = np.zeros_like(g["elements"])
        ctx.pairwise_align(*g["range"], elements, n + 1)
        assert np.array_equal(elements, g["elements"])
        pairs = range_pairs(n, *g["range"])
        if len(pairs):
            check_vs_oracle(ctx, oracle_mod, g, pairs)
    finally:
        ctx.set_cta_tuning(*old)


@pytest.mark.parametrize("warps,large_rows", [(2, 768), (4, 256), (8, 2), (8, 65535), (16, 512), (16, 768), (8, 0),
                                             (16, 0), (4, 0)])
def test_cta_form_knobs_keep_results(ctx, oracle_mod, warps, large_rows):
    """Warps per CTA and the size from which the CTA divides a frame together
    change only the schedule (large_rows 2: every frame with 64 columns or
    more, two at a time whenever two are waiting; 65535: none, every frame to
    one warp; 0: the automatic threshold)."""
    g = load_golden("synth_long_6x3000")
    setup(ctx, g)
    old = ctx.get_cta_tuning()
    ctx.set_cta_tuning(ALWAYS, warps, large_rows)
    try:
        pairs = range_pairs(6, 0, 6, 0, 6)
        pairs = np.concatenate([pairs, pairs[:, ::-1]]).astype(np.int32)
        check_vs_oracle(ctx, oracle_mod, g, pairs)
    finally:
        ctx.set_cta_tuning(*old)


def test_cta_form_on_a_family_with_both_kernels(ctx, oracle_mod):
    """A plan whose long pairs take the CTA form while its short pairs (first
    sequence of at most 128 residues) run in the short-pair kernel beside it."""
    from clustalw_gb300 import load_matrix, synth

    matrix, params = load_matrix("protein")
    seqs = synth.protein_family(6, 900, 5) + synth.protein_family(6, 90, 6)
    g = dict(seqs=seqs, matrix=matrix, params=params)
    setup(ctx, g)
    pairs = range_pairs(12, 0, 12, 0, 12)
    pairs = np.concatenate([pairs, pairs[:, ::-1]]).astype(np.int32)
    plan = ctx.plan(pairs)
    assert plan.kernel_count() == 2
    plan.close()
    check_vs_oracle(ctx, oracle_mod, g, pairs)


def test_one_column_call_takes_the_cta_form_by_default(ctx):
    """sequencesAlignToProfile recomputes one column of pairs (Clustal.cpp:404-416):
    N-1 long pairs, fewer than the long-pair kernel's warps, so by default they
    run one CTA per pair; the results equal the one-warp form's."""
    g = load_golden("fixture_100_1523")
    setup(ctx, g)
    n = len(g["seqs"])
    pairs = range_pairs(n, 0, n, n - 2, n)
    assert len(pairs) == n - 1
    assert ctx.get_cta_tuning() == (-1, 0, 0)  # defaults: automatic threshold, warps and frame size
    plan = ctx.plan(pairs)
    assert plan.pair_ctas()
    plan.close()
    d_cta, s_cta = ctx.align_pairs(pairs, stats=True)
    old = ctx.get_cta_tuning()
    ctx.set_cta_tuning(max_pairs=0)
    try:
        plan = ctx.plan(pairs)
        assert not plan.pair_ctas()
        plan.close()
        d_warp, s_warp = ctx.align_pairs(pairs, stats=True)
    finally:
        ctx.set_cta_tuning(*old)
    assert np.array_equal(d_cta, d_warp) and np.array_equal(s_cta, s_warp)


def test_cta_tuning_rejects_bad_values(ctx):
    from clustalw_gb300.native import CwgpuError

    for bad in [(-2, 8, 768), (10, 3, 768), (10, 32, 768), (10, 8, 1), (10, 8, 70000)]:
        with pytest.raises(CwgpuError):
            ctx.set_cta_tuning(*bad)


def test_cta_hand_over_wait_times_out_and_context_stays_usable(ctx, oracle_mod):
    """The wait a warp makes for its predecessor's row, run on a progress word
    nothing raises, ends after its 2 ms bound with the timeout status."""
    assert ctx.cta_wait_probe(2_000_000)
    g = load_golden("synth_long_6x3000")
    setup(ctx, g)
    old = ctx.get_cta_tuning()
    ctx.set_cta_tuning(max_pairs=ALWAYS)
    try:
        check_vs_oracle(ctx, oracle_mod, g, range_pairs(6, 0, 6, 0, 6)[:5])
    finally:
        ctx.set_cta_tuning(*old)
