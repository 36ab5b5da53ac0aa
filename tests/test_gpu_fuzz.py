"""Seeded random inputs through every form of the pair kernels, against the
oracle: alphabets of 1 to 25 residue codes (so the remapped alphabet the
score profile is built on varies), symmetric pairwise matrices over the int16
range (negative entries included), random gap penalties under the protein and
the DNA rules (gap extension 0 included), lengths from 0 to 400 residues
(both kernels, partial and full stripes, empty sequences), internal gap codes,
random tiny-frame and short-pair thresholds. The one-shot call, a plan, the
one-CTA-per-pair form (every warp count) and the plain per-pair form all give
the oracle's distances and per-pair intermediates bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STAT_FIELDS = ["fwd_score", "se1", "se2", "sb1", "sb2", "mm_score", "n_ident", "n_match"]
ALWAYS = 2**31 - 1
GAP1, GAP2 = 30, 31
LENGTHS = [0, 1, 2, 3, 7, 16, 31, 33, 64, 97, 127, 128, 129, 130, 200, 255, 256, 257, 400]


@pytest.fixture(scope="module")
def ctx():
    from clustalw_gb300 import native

    c = native.Context(0)
    yield c
    c.close()


def random_case(seed):
    rng = np.random.default_rng(seed)
    K = int(rng.integers(1, 26))
    alphabet = np.sort(rng.choice(25, size=K, replace=False))
    m = rng.integers(-1500, 3001, size=(32, 32))
    m = np.triu(m) + np.triu(m, 1).T
    if seed % 3 == 0:  # an identity-like matrix: many ties
        m = np.where(np.eye(32, dtype=bool), int(rng.integers(1, 200)), 0)
    matrix = m.astype(np.int32)
    dna = int(rng.integers(0, 2))
    params = dict(dna=dna, int_scale=int(rng.choice([10, 100])), mat_avg=int(rng.integers(0, 60)),
                  gap_pos1=GAP1, gap_pos2=GAP2,
                  pw_gap_open=float(np.float32(rng.choice([0.0, 1.0, 5.0, 10.0, 15.0, 25.0, 40.0]))),
                  pw_gap_extend=float(np.float32(rng.choice([0.0, 0.05, 0.1, 1.0, 6.66]))),
                  gap_open_scale=float(np.float32(rng.uniform(0.5, 2.0))),
                  gap_extend_scale=float(np.float32(rng.uniform(0.5, 2.0))))
    n = int(rng.integers(2, 24))
    root = rng.choice(alphabet, size=400)
    seqs = []
    for _ in range(n):
        L = int(rng.choice(LENGTHS))
        if rng.random() < 0.7:  # a mutated piece of the shared root, so alignments are long
            start = int(rng.integers(0, 401 - L)) if L < 400 else 0
            s = root[start : start + L].copy()
            sub = rng.random(L) < rng.uniform(0.0, 0.5)
            s[sub] = rng.choice(alphabet, size=int(sub.sum()))
        else:
            s = rng.choice(alphabet, size=L)
        if L > 4 and rng.random() < 0.3:  # internal gap codes (not residues: nres, identities)
            s[rng.integers(0, L, size=max(1, L // 20))] = rng.choice([GAP1, GAP2])
        seqs.append(s.astype(np.int8))
    pairs = np.array([(i, j) for i in range(n) for j in range(i + 1, n)], dtype=np.int32)
    pairs = np.concatenate([pairs, pairs[rng.random(len(pairs)) < 0.3][:, ::-1]]).astype(np.int32)
    tuning = [(0, 0, 0), (32, 16, 128), (16, 8, 64), (64, 16, 300), (32, 12, 65535)][seed % 5]
    return matrix, params, seqs, pairs, tuning


def check(got, want, what):
    dist, st = got
    assert np.array_equal(dist.view(np.int32), want["dist"].view(np.int32)), what
    for f in STAT_FIELDS:
        bad = np.nonzero(st[f] != want[f])[0]
        assert len(bad) == 0, f"{what} {f}: {len(bad)} pairs, first gpu {st[f][bad[0]]} oracle {want[f][bad[0]]}"


@pytest.mark.parametrize("seed", range(48))
def test_random_inputs_every_form(ctx, oracle_mod, seed):
    matrix, params, seqs, pairs, tuning = random_case(seed)
    ctx.set_matrix(matrix)
    ctx.set_params(params)
    ctx.upload_seqs(seqs)
    old_t, old_c = ctx.get_tuning(), ctx.get_cta_tuning()
    try:
        ctx.set_tuning(*tuning)
        want = oracle_mod.align_pairs(seqs, matrix, params, pairs)
        check(ctx.align_pairs(pairs, stats=True), want, "one-shot")
        plan = ctx.plan(pairs)
        plan.launch()
        got = plan.results(stats=True)
        plan.close()
        check(got, want, "plan")
        for warps in (4, 8, 16):
            ctx.set_cta_tuning(ALWAYS, warps, 2 if warps == 8 else 1024)
            check(ctx.align_pairs(pairs, stats=True), want, f"cta{warps}")
        ctx.set_cta_tuning(*old_c)
        few = pairs[:12]
        dist, st = ctx.align_pairs(few, stats=True, plain=True)
        check((dist, st), want[: len(few)], "plain")
    finally:
        ctx.set_tuning(*old_t)
        ctx.set_cta_tuning(*old_c)
