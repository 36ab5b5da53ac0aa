"""CPU-side checks of the C ABI: the library builds for sm_103a, loads, exports
every function include/*.h declares, and its host-only helpers (no device
work) agree with the oracle."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import REPO, load_golden


def declared_functions():
    inc = os.path.join(REPO, "include")
    text = "\n".join(open(os.path.join(inc, h)).read() for h in sorted(os.listdir(inc)) if h.endswith(".h"))
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cwgpu_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from clustalw_gb300 import native

    return native.load()


def test_header_declares_core_entry_points():
    names = declared_functions()
    for must in ["cwgpu_create", "cwgpu_pairwise_align", "cwgpu_align_pairs", "cwgpu_align_pairs_plain", "cwgpu_plan_create",
                 "cwgpu_nj_tree"]:
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    from clustalw_gb300 import native

    for name in declared_functions():
        assert hasattr(lib, name), f"{name} declared in include/ but not exported"
        assert name in native.SIGNATURES, f"{name} has no ctypes signature"


def test_gap_penalties_match_oracle(lib, oracle_mod):
    from clustalw_gb300 import native

    for g in ["fixture_100_97", "fixture_100_1002", "synth_uneven_40"]:
        p = load_golden(g)["params"]
        for n, m in [(1, 1), (2, 7), (97, 96), (498, 498), (1523, 1600), (3000, 2999), (65535, 65535)]:
            assert native.gap_penalties(p, n, m) == oracle_mod.gap_penalties(p, n, m)
    # matAvg <= 0 protein branch (2 * (int)(...)).
    p = dict(load_golden("fixture_100_97")["params"], mat_avg=0)
    for n in [5, 50, 500]:
        assert native.gap_penalties(p, n, n) == oracle_mod.gap_penalties(p, n, n)


def test_range_pair_count(lib):
    from clustalw_gb300 import native
    from conftest import range_pairs

    for rng in [(0, 10, 0, 10), (0, 10, 4, 10), (3, 7, 0, 10), (5, 5, 0, 10), (0, 100, 0, 100), (8, 20, 9, 30)]:
        assert native.range_pair_count(10, *rng) == len(range_pairs(10, *rng))
    big = 2**31 - 1  # column start at INT32_MAX selects no column (no 32-bit wrap)
    assert native.range_pair_count(10, 0, 10, big, big) == 0
    assert native.range_pair_count(10, 0, big, 0, big) == 45
    assert native.range_pair_count(70000, 0, 70000, 0, 70000) == 70000 * 69999 // 2


def test_status_strings(lib):
    for code in range(10):
        assert lib.cwgpu_status_string(code)


def test_autotune_helpers_cpu():
    from clustalw_gb300 import autotune, synth

    rng = np.random.default_rng(3)
    lens = rng.integers(30, 2000, size=200)
    pairs = synth.all_pairs(200)
    s = autotune.stratified_sample(lens, pairs, 5e8)
    assert len(s) > 0 and s.shape[1] == 2
    work = lens[s[:, 0]].astype(np.int64) * lens[s[:, 1]]
    assert work.min() < np.median(lens) ** 2 < work.max()
    assert autotune.length_profile(lens) == autotune.length_profile(lens.copy())
    assert autotune.length_profile([1523] * 10) != autotune.length_profile([97] * 10)


def test_autotune_environment_override(tmp_path, monkeypatch):
    """$CLUSTALW_GB300_TUNING beats the cache and the search; unset or empty
    means no override; a malformed value is an error."""
    from clustalw_gb300 import autotune, synth

    class FakeCtx:
        t = (32, 16, 128)

        def set_tuning(self, m, n, r=None):
            self.t = (m, n, r)

        def get_tuning(self):
            return self.t

    monkeypatch.setattr(autotune, "_time_sample", lambda *a: pytest.fail("timed despite the override"))
    monkeypatch.setenv("XDG_CACHE_HOME", str(tmp_path))
    monkeypatch.delenv(autotune.ENV_VAR, raising=False)
    assert autotune.env_override() is None
    monkeypatch.setenv(autotune.ENV_VAR, " ")
    assert autotune.env_override() is None
    monkeypatch.setenv(autotune.ENV_VAR, "16, 8,256")
    assert autotune.env_override() == (16, 8, 256)
    ctx = FakeCtx()
    lens = np.array([100] * 10)
    assert autotune.tune(ctx, lens, synth.all_pairs(10), gpu_name="fake") == ((16, 8, 256), {})
    assert ctx.get_tuning() == (16, 8, 256)
    for bad in ("16,8", "a,b,c", "1,2,3,4"):
        monkeypatch.setenv(autotune.ENV_VAR, bad)
        with pytest.raises(ValueError):
            autotune.env_override()


def test_context_applies_the_tuning_override(monkeypatch):
    """native.Context sets $CLUSTALW_GB300_TUNING on its new handle, and only
    when it is set (a stand-in library on the CPU: no device call)."""
    from clustalw_gb300 import autotune, native

    class FakeLib:
        def __init__(self):
            self.tuning = []

        def cwgpu_create(self, device, handle):
            return 0

        def cwgpu_destroy(self, handle):
            pass

        def cwgpu_set_tuning(self, handle, ref):
            t = ref._obj
            self.tuning.append((t.tiny_m, t.tiny_n, t.short_rows))
            return 0

    fake = FakeLib()
    monkeypatch.setattr(native, "load", lambda build=True: fake)
    monkeypatch.delenv(autotune.ENV_VAR, raising=False)
    native.Context(0).close()
    assert fake.tuning == []
    monkeypatch.setenv(autotune.ENV_VAR, "64,16,192")
    native.Context(0).close()
    assert fake.tuning == [(64, 16, 192)]


def test_autotune_search_and_cache_cpu(tmp_path, monkeypatch):
    """The tuner's search on a stand-in context with a known cost model: the
    tiny-frame candidates first, then only the short-pair thresholds that
    split the sample differently, the fastest kept and cached."""
    from clustalw_gb300 import autotune, synth

    class FakeCtx:
        def __init__(self):
            self.t = (32, 16, 128)
            self.timed = []

        def set_tuning(self, m, n, r=None):
            self.t = (m, n, self.t[2] if r is None else r)

        def get_tuning(self):
            return self.t

    def cost(t):  # best at (16, 16) and 192 rows
        return abs(t[0] - 16) + abs(t[1] - 16) + abs(t[2] - 192) / 64 + 1.0

    def fake_time(ctx, sample, repeats):
        ctx.timed.append(ctx.t)
        return cost(ctx.t)

    monkeypatch.setattr(autotune, "_time_sample", fake_time)
    monkeypatch.setenv("XDG_CACHE_HOME", str(tmp_path))
    monkeypatch.delenv(autotune.ENV_VAR, raising=False)
    lens = np.array([100] * 20 + [150] * 20 + [1000] * 20)
    pairs = synth.all_pairs(len(lens))
    ctx = FakeCtx()
    choice, timings = autotune.tune(ctx, lens, pairs, gpu_name="fake", target_cells=1e9)
    assert choice == (16, 16, 192) and ctx.get_tuning() == choice
    tiny = [t for t in ctx.timed if t[2] == 128]
    assert len(tiny) == len(autotune.CANDIDATES)
    # 0 and 64 split the sample the same way (no first sequence is that short): one of them is timed
    assert sum(1 for t in ctx.timed if t[2] in (0, 64)) == 1
    # cached: a second call does not time anything
    ctx2 = FakeCtx()
    choice2, timings2 = autotune.tune(ctx2, lens, pairs, gpu_name="fake", target_cells=1e9)
    assert choice2 == choice and timings2 == {} and ctx2.timed == [] and ctx2.get_tuning() == choice


def test_autotune_cta_choice_cpu(monkeypatch):
    """tune_cta on a stand-in context: the whole launch is timed one warp per
    pair and with each CTA width, and the threshold is set so that a launch of
    this many long pairs takes the faster form; launches with many long pairs
    are not timed."""
    from clustalw_gb300 import autotune, synth

    class FakeCtx:
        def __init__(self):
            self.cta = (-1, 0, 512)
            self.timed = []

        def get_tuning(self):
            return (32, 16, 128)

        def get_cta_tuning(self):
            return self.cta

        def set_cta_tuning(self, p, w, r):
            self.cta = (p, w, r)

    def fake_time(cost):
        def f(ctx, sample, repeats):
            ctx.timed.append(ctx.cta)
            return cost(ctx.cta)
        return f

    lens = np.array([1500] * 10 + [100] * 5)
    pairs = synth.all_pairs(len(lens))  # 95 long pairs (first sequence > 128), 10 short
    # CTA form with 8 warps fastest
    monkeypatch.setattr(autotune, "_time_sample", fake_time(lambda t: 1.0 if t[0] == 0 else abs(t[1] - 8) + 0.5))
    ctx = FakeCtx()
    choice, timings = autotune.tune_cta(ctx, lens, pairs)
    assert choice == (95, 8, 512) and ctx.cta == choice and len(timings) == 1 + len(autotune.CTA_WARPS)
    # one warp per pair fastest: the threshold falls below this launch
    monkeypatch.setattr(autotune, "_time_sample", fake_time(lambda t: 0.5 if t[0] == 0 else 1.0))
    ctx = FakeCtx()
    choice, _ = autotune.tune_cta(ctx, lens, pairs)
    assert choice[0] == 94 and ctx.cta == choice
    # many long pairs: untimed
    ctx = FakeCtx()
    big = np.array([1500] * 100)
    choice, timings = autotune.tune_cta(ctx, big, synth.all_pairs(100))
    assert timings == {} and ctx.timed == [] and choice == (-1, 0, 512)


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """No CPU fallback: without the built library the package raises instead
    of computing anything."""
    from clustalw_gb300 import _build, native

    monkeypatch.setattr(native, "_lib", None)
    monkeypatch.setattr(_build, "LIB_PATH", str(tmp_path / "absent" / "libcwgpu.so"))
    with pytest.raises(RuntimeError, match="missing"):
        native.load(build=False)


def test_bench_distmatrix_packing_matches_symmatrix():
    """bench.py fills the reference's packed SymMatrix from a pair list the
    way FullPairwiseAlign's SetAt does (float distance stored as double)."""
    import bench
    from clustalw_gb300 import synth
    from clustalw_gb300.pairwise import DistMatrix

    n = 7
    pairs = synth.all_pairs(n)
    dist = np.linspace(0.05, 0.95, len(pairs)).astype(np.float32)
    el = bench.packed_distmatrix(n, pairs, dist)
    dm = DistMatrix(n + 1)
    for (i, j), d in zip(pairs, dist):
        dm.SetAt(int(i) + 1, int(j) + 1, float(np.float64(d)))
    assert np.array_equal(el, dm.getElements())
