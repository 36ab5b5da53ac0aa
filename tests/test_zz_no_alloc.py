"""The allocation-free entry point, cwgpu_align_pairs_noalloc, called through
the C ABI with device buffers the caller owns (allocated here with torch, as a
framework that owns all device memory would). It serves callers that cannot
call cudaMalloc themselves; its results must equal those of the allocating
entry point cwgpu_align_pairs, bit for bit (the same tolerance, zero, that the
other parity tests use for distances and integer statistics), on two calls in a
row that share the library's static scratch array. Collected last on purpose."""
import ctypes

import numpy as np
import pytest

from conftest import load_fast_golden, load_golden, range_pairs

pytestmark = pytest.mark.gpu


def _device_inputs(torch, g):
    from clustalw_gb300 import native

    codes, offsets, lens = native.pack_sequences(g["seqs"])
    dev = torch.device("cuda", 0)
    return dict(
        codes=torch.from_numpy(codes).to(dev),
        offsets=torch.from_numpy(offsets).to(dev),
        lens=torch.from_numpy(lens).to(dev),
        matrix=torch.from_numpy(np.ascontiguousarray(g["matrix"].reshape(-1).astype(np.int32))).to(dev),
        max_len=int(lens.max()),
    )


def _call(lib, d, params, pairs_dev, npairs, dist_dev, stats_dev, max_len=None, stream=None):
    return lib.cwgpu_align_pairs_noalloc(
        d["codes"].data_ptr(),
        d["offsets"].data_ptr(),
        d["lens"].data_ptr(),
        int(d["lens"].numel()),
        int(d["max_len"] if max_len is None else max_len),
        d["matrix"].data_ptr(),
        ctypes.byref(params),
        pairs_dev.data_ptr(),
        int(npairs),
        dist_dev.data_ptr(),
        stats_dev.data_ptr() if stats_dev is not None else None,
        stream,
    )


@pytest.mark.parametrize("name", ["synth_uneven_40", "fixture_100_97", "edge_protein"])
def test_noalloc_matches_allocating_entry_point_twice(name):
    torch = pytest.importorskip("torch")
    from clustalw_gb300 import native

    g = load_golden(name)
    pairs = range_pairs(len(g["seqs"]), 0, len(g["seqs"]), 0, len(g["seqs"]))
    with native.Context(0) as ctx:
        ctx.set_matrix(g["matrix"])
        ctx.set_params(g["params"])
        ctx.upload_seqs(g["seqs"])
        want_dist, want_stats = ctx.align_pairs(pairs, stats=True)

    lib = native.load()
    params = native.Params.from_dict(g["params"])
    d = _device_inputs(torch, g)
    pairs_dev = torch.from_numpy(pairs).to("cuda")
    for call in range(2):
        dist_dev = torch.full((len(pairs),), float("nan"), dtype=torch.float32, device="cuda")
        stats_dev = torch.full((len(pairs), 8), -7, dtype=torch.int32, device="cuda")
        rc = _call(lib, d, params, pairs_dev, len(pairs), dist_dev, stats_dev)
        assert rc == 0, f"call {call}: status {rc}"
        got_dist = dist_dev.cpu().numpy()
        got_stats = stats_dev.cpu().numpy().copy().view(native.PAIR_STATS_DTYPE).reshape(-1)
        assert np.array_equal(got_dist, want_dist), f"call {call}: distances differ"
        assert np.array_equal(got_stats, want_stats), f"call {call}: statistics differ"


def test_noalloc_rejects_lengths_above_its_limit():
    torch = pytest.importorskip("torch")
    from clustalw_gb300 import native

    g = load_golden("synth_uneven_40")
    lib = native.load()
    d = _device_inputs(torch, g)
    pairs = range_pairs(len(g["seqs"]), 0, 3, 0, 3)
    pairs_dev = torch.from_numpy(pairs).to("cuda")
    dist_dev = torch.zeros(len(pairs), dtype=torch.float32, device="cuda")
    params = native.Params.from_dict(g["params"])
    rc = _call(lib, d, params, pairs_dev, len(pairs), dist_dev, None, max_len=8192)
    assert rc == 1  # CWGPU_ERR_ARG
    # A stated max_len below a real length is caught by the device-side check.
    rc = _call(lib, d, params, pairs_dev, len(pairs), dist_dev, None, max_len=2)
    assert rc == 1


def test_noalloc_at_its_length_limit_and_on_a_caller_stream():
    """A caller with a fixed limit passes max_len = CWGPU_NOALLOC_MAX_LEN
    (8191) whatever its sequences are: that changes the row stride, the slot
    count and the grid (about 31 CTAs at 8191). Short sequences at that
    max_len, on a caller-owned stream, must still equal the allocating entry
    point bit for bit; then 8191-residue sequences (a sequence, a mutated copy
    and a fragment) must equal the oracle in every intermediate."""
    torch = pytest.importorskip("torch")
    from clustalw_gb300 import load_matrix, native
    from oracle import oracle as O

    g = load_golden("synth_uneven_40")
    pairs = range_pairs(len(g["seqs"]), 0, len(g["seqs"]), 0, len(g["seqs"]))
    with native.Context(0) as ctx:
        ctx.set_matrix(g["matrix"])
        ctx.set_params(g["params"])
        ctx.upload_seqs(g["seqs"])
        want_dist, want_stats = ctx.align_pairs(pairs, stats=True)
    lib = native.load()
    params = native.Params.from_dict(g["params"])
    d = _device_inputs(torch, g)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        pairs_dev = torch.from_numpy(pairs).to("cuda")
        dist_dev = torch.full((len(pairs),), float("nan"), dtype=torch.float32, device="cuda")
        stats_dev = torch.full((len(pairs), 8), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()  # inputs made on both streams are in place before the call
    rc = _call(lib, d, params, pairs_dev, len(pairs), dist_dev, stats_dev, max_len=8191, stream=stream.cuda_stream)
    assert rc == 0
    assert np.array_equal(dist_dev.cpu().numpy(), want_dist)
    assert np.array_equal(stats_dev.cpu().numpy().copy().view(native.PAIR_STATS_DTYPE).reshape(-1), want_stats)

    q = load_fast_golden("quicklimit_protein_8191")
    seqs = q["seqs"]
    assert max(len(s) for s in seqs) == 8191
    matrix, prot = load_matrix("protein")
    lp = np.array([[0, 1], [1, 0], [0, 2], [2, 1]], dtype=np.int32)
    want = O.align_pairs(seqs, matrix, prot, lp)
    d = _device_inputs(torch, dict(seqs=seqs, matrix=matrix))
    lp_dev = torch.from_numpy(lp).to("cuda")
    dist_dev = torch.full((len(lp),), float("nan"), dtype=torch.float32, device="cuda")
    stats_dev = torch.full((len(lp), 8), -7, dtype=torch.int32, device="cuda")
    rc = _call(lib, d, native.Params.from_dict(prot), lp_dev, len(lp), dist_dev, stats_dev, max_len=8191)
    assert rc == 0
    assert np.array_equal(dist_dev.cpu().numpy(), want["dist"])
    got = stats_dev.cpu().numpy().copy().view(native.PAIR_STATS_DTYPE).reshape(-1)
    for f in native.PAIR_STATS_DTYPE.names:
        assert np.array_equal(got[f], want[f]), f


def test_noalloc_rejects_bad_matrix_entries_and_offsets():
    """A matrix entry outside int16 (the score profile's range) is refused with
    CWGPU_ERR_MATRIX before any pair is aligned, as cwgpu_set_matrix refuses it
    on the host; a negative sequence offset is refused with CWGPU_ERR_ARG
    instead of being read. A good call afterwards is unaffected."""
    torch = pytest.importorskip("torch")
    from clustalw_gb300 import native

    g = load_golden("synth_uneven_40")
    lib = native.load()
    params = native.Params.from_dict(g["params"])
    pairs = range_pairs(len(g["seqs"]), 0, 4, 0, 4)
    pairs_dev = torch.from_numpy(pairs).to("cuda")
    dist_dev = torch.full((len(pairs),), float("nan"), dtype=torch.float32, device="cuda")
    d = _device_inputs(torch, g)
    bad = dict(d)
    m = g["matrix"].reshape(-1).astype(np.int32).copy()
    m[33] = 40000
    bad["matrix"] = torch.from_numpy(m).to("cuda")
    assert _call(lib, bad, params, pairs_dev, len(pairs), dist_dev, None) == 8  # CWGPU_ERR_MATRIX
    assert bool(torch.isnan(dist_dev).all())
    bad = dict(d)
    offs = d["offsets"].clone()
    offs[1] = -64
    bad["offsets"] = offs
    assert _call(lib, bad, params, pairs_dev, len(pairs), dist_dev, None) == 1  # CWGPU_ERR_ARG
    assert _call(lib, d, params, pairs_dev, len(pairs), dist_dev, None) == 0
