"""ctypes bindings of the C ABI declared in include/cwgpu.h.

There is no fallback: if lib/libcwgpu.so cannot be loaded, or a call fails,
an exception is raised. Nothing here computes an alignment on the CPU.
"""
import ctypes
import os

import numpy as np

from . import _build

NUMRES = 32

STATUS = {
    0: "CWGPU_OK",
    1: "CWGPU_ERR_ARG",
    2: "CWGPU_ERR_CUDA",
    3: "CWGPU_ERR_OOM",
    4: "CWGPU_ERR_STATE",
    5: "CWGPU_ERR_RANGE",
    6: "CWGPU_ERR_TIMEOUT",
    7: "CWGPU_ERR_DEVICE",
    8: "CWGPU_ERR_MATRIX",
    9: "CWGPU_ERR_NOT_FOUND",
}


class CwgpuError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class Params(ctypes.Structure):
    """cwgpu_params: the scalars FullPairwiseAlign::pairwiseAlign reads."""

    _fields_ = [
        ("dna", ctypes.c_int32),
        ("pw_gap_open", ctypes.c_float),
        ("pw_gap_extend", ctypes.c_float),
        ("int_scale", ctypes.c_int32),
        ("gap_open_scale", ctypes.c_float),
        ("gap_extend_scale", ctypes.c_float),
        ("mat_avg", ctypes.c_int32),
        ("gap_pos1", ctypes.c_int32),
        ("gap_pos2", ctypes.c_int32),
    ]

    @classmethod
    def from_dict(cls, d):
        p = cls()
        for name, _ in cls._fields_:
            setattr(p, name, d[name])
        return p

    def to_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


PAIR_STATS_DTYPE = np.dtype(
    [
        ("fwd_score", "<i4"),
        ("se1", "<i4"),
        ("se2", "<i4"),
        ("sb1", "<i4"),
        ("sb2", "<i4"),
        ("mm_score", "<i4"),
        ("n_ident", "<i4"),
        ("n_match", "<i4"),
    ]
)

class FastParams(ctypes.Structure):
    """cwgpu_fast_params: what FastPairwiseAlign::pairAlign reads from userParameters."""

    _fields_ = [(k, ctypes.c_int32) for k in
                ("dna", "ktup", "window", "window_gap", "signif", "percent", "max_aa", "max_aln_length")]

    @classmethod
    def from_dict(cls, d):
        return cls(*[int(d.get(k, 0)) for k, _ in cls._fields_])

    @classmethod
    def defaults(cls, dna, max_aln_length=0):
        """The reference's defaults after setDNAParams/setProtParams
        (UserParameters.cpp:86-94, 133)."""
        if dna:
            return cls(1, 2, 4, 5, 4, 1, 24, max_aln_length)
        return cls(0, 1, 5, 3, 5, 1, 24, max_aln_length)


FAST_STATS_DTYPE = np.dtype([("score", "<i4"), ("frags", "<i4"), ("partial", "<i4"), ("pad", "<i4")])


class Tuning(ctypes.Structure):
    """cwgpu_tuning: tiny-frame thresholds of the Myers-Miller stage."""

    _fields_ = [("tiny_m", ctypes.c_int32), ("tiny_n", ctypes.c_int32), ("short_rows", ctypes.c_int32)]


class CtaTuning(ctypes.Structure):
    """cwgpu_cta_tuning: when and how long pairs run one CTA per pair."""

    _fields_ = [("max_pairs", ctypes.c_int32), ("warps", ctypes.c_int32), ("large_rows", ctypes.c_int32)]


class ServerOpts(ctypes.Structure):
    _fields_ = [
        ("memory_budget_bytes", ctypes.c_int64),
        ("max_jobs", ctypes.c_int32),
        ("max_seq_len", ctypes.c_int32),
        ("round_cells", ctypes.c_double),
        ("max_items_per_round", ctypes.c_int64),
        ("policy", ctypes.c_int32),
        ("srpt_age_ms", ctypes.c_int32),
    ]


class ServerStats(ctypes.Structure):
    _fields_ = [
        ("jobs_queued", ctypes.c_int64),
        ("jobs_running", ctypes.c_int64),
        ("jobs_done", ctypes.c_int64),
        ("rounds", ctypes.c_int64),
        ("pairs", ctypes.c_int64),
        ("bytes_in_use", ctypes.c_int64),
        ("cells", ctypes.c_int64 * 3),
    ]


_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64

# name -> (restype, argtypes); every function include/*.h declares.
SIGNATURES = {
    "cwgpu_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_vp)]),
    "cwgpu_destroy": (None, [_vp]),
    "cwgpu_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "cwgpu_last_error": (ctypes.c_char_p, [_vp]),
    "cwgpu_set_matrix": (ctypes.c_int, [_vp, _vp]),
    "cwgpu_set_params": (ctypes.c_int, [_vp, ctypes.POINTER(Params)]),
    "cwgpu_upload_seqs": (ctypes.c_int, [_vp, _i32, _vp, _vp, _vp]),
    "cwgpu_gap_penalties": (
        ctypes.c_int,
        [ctypes.POINTER(Params), _i32, _i32, ctypes.POINTER(_i32), ctypes.POINTER(_i32)],
    ),
    "cwgpu_range_pair_count": (_i64, [_i32, _i32, _i32, _i32, _i32]),
    "cwgpu_pairwise_align": (ctypes.c_int, [_vp, _i32, _i32, _i32, _i32, _vp, _i32, _vp]),
    "cwgpu_align_pairs": (ctypes.c_int, [_vp, _vp, _i64, _vp, _vp]),
    "cwgpu_align_pairs_plain": (ctypes.c_int, [_vp, _vp, _i64, _vp, _vp]),
    "cwgpu_plan_create": (ctypes.c_int, [_vp, _vp, _i64, ctypes.POINTER(_vp)]),
    "cwgpu_plan_launch": (ctypes.c_int, [_vp, _vp]),
    "cwgpu_plan_results": (ctypes.c_int, [_vp, _vp, _vp]),
    "cwgpu_plan_device_dist": (_vp, [_vp]),
    "cwgpu_plan_cell_counts": (ctypes.c_int, [_vp, _vp]),
    "cwgpu_plan_kernel_count": (ctypes.c_int, [_vp]),
    "cwgpu_plan_pair_ctas": (ctypes.c_int, [_vp]),
    "cwgpu_plan_destroy": (None, [_vp]),
    "cwgpu_synchronize": (ctypes.c_int, [_vp]),
    "cwgpu_set_tuning": (ctypes.c_int, [_vp, ctypes.POINTER(Tuning)]),
    "cwgpu_get_tuning": (ctypes.c_int, [_vp, ctypes.POINTER(Tuning)]),
    "cwgpu_set_cta_tuning": (ctypes.c_int, [_vp, ctypes.POINTER(CtaTuning)]),
    "cwgpu_get_cta_tuning": (ctypes.c_int, [_vp, ctypes.POINTER(CtaTuning)]),
    "cwgpu_cta_wait_probe": (ctypes.c_int, [_vp, _i64, ctypes.POINTER(ctypes.c_int32)]),
    "cwgpu_server_create": (
        ctypes.c_int,
        [ctypes.c_int, _vp, ctypes.POINTER(Params), ctypes.POINTER(ServerOpts), ctypes.POINTER(_vp)],
    ),
    "cwgpu_server_destroy": (None, [_vp]),
    "cwgpu_server_submit": (ctypes.c_int, [_vp, _i32, _vp, _vp, _vp, _i32, ctypes.POINTER(_i64)]),
    "cwgpu_server_poll": (ctypes.c_int, [_vp, _i64, ctypes.POINTER(_i32)]),
    "cwgpu_server_wait": (ctypes.c_int, [_vp, _i64, _i32]),
    "cwgpu_server_result": (ctypes.c_int, [_vp, _i64, _vp, _vp, _vp]),
    "cwgpu_server_release": (ctypes.c_int, [_vp, _i64]),
    "cwgpu_server_query": (ctypes.c_int, [_vp, ctypes.POINTER(ServerStats)]),
    "cwgpu_align_pairs_noalloc": (
        ctypes.c_int,
        [_vp, _vp, _vp, _i32, _i32, _vp, ctypes.POINTER(Params), _vp, _i64, _vp, _vp, _vp],
    ),
    "cwgpu_fast_pairwise_align": (
        ctypes.c_int,
        [_vp, ctypes.POINTER(FastParams), _i32, _i32, _i32, _i32, _vp, _i32, _vp],
    ),
    "cwgpu_fast_align_pairs": (ctypes.c_int, [_vp, ctypes.POINTER(FastParams), _vp, _i64, _vp, _vp]),
    "cwgpu_fast_align_pairs_device": (
        ctypes.c_int,
        [_vp, ctypes.POINTER(FastParams), _vp, _vp, _i64, _vp, _vp, _vp],
    ),
    # include/cwgpu_nj.h
    "cwgpu_nj_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_vp)]),
    "cwgpu_nj_destroy": (None, [_vp]),
    "cwgpu_nj_last_error": (ctypes.c_char_p, [_vp]),
    "cwgpu_nj_tree": (ctypes.c_int, [_vp, _i32, _vp, _vp, _vp, _vp, _vp]),
    "cwgpu_nj_tree_device": (ctypes.c_int, [_vp, _i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "cwgpu_nj_last_stats": (ctypes.c_int, [_vp, ctypes.POINTER(_i64), ctypes.POINTER(ctypes.c_double)]),
    "cwgpu_nj_seq_sum": (ctypes.c_int, [_vp, _vp, _i64, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]),
    "cwgpu_nj_wait_probe": (ctypes.c_int, [_vp, _i64, ctypes.POINTER(ctypes.c_int32)]),
}

_lib = None


def load(build=True):
    """Load lib/libcwgpu.so (building it first if it is missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    if build:
        _build.build()
    if not os.path.exists(_build.LIB_PATH):
        raise RuntimeError(f"GB300 library missing: {_build.LIB_PATH}")
    lib = ctypes.CDLL(_build.LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def _ptr(a):
    """Address of a contiguous numpy array's data (None for None). A writable
    array takes the cheaper buffer route; read-only or empty ones .ctypes."""
    if a is None:
        return None
    try:
        return ctypes.addressof(ctypes.c_char.from_buffer(a))
    except (TypeError, ValueError, BufferError):
        return a.ctypes.data


def gap_penalties(params, n, m):
    """Host-side gap penalties (no device work)."""
    lib = load()
    p = params if isinstance(params, Params) else Params.from_dict(params)
    go, ge = _i32(), _i32()
    rc = lib.cwgpu_gap_penalties(ctypes.byref(p), int(n), int(m), ctypes.byref(go), ctypes.byref(ge))
    if rc:
        raise CwgpuError(rc, "cwgpu_gap_penalties")
    return go.value, ge.value


def range_pair_count(nseqs, i_start, i_end, j_start, j_end):
    return int(load().cwgpu_range_pair_count(nseqs, i_start, i_end, j_start, j_end))


def pack_sequences(seqs):
    """list of code arrays -> (codes int8, offsets int64, lens int32)."""
    lens = np.array([len(s) for s in seqs], dtype=np.int32)
    offsets = np.zeros(len(seqs), dtype=np.int64)
    if len(seqs) > 1:
        offsets[1:] = np.cumsum(lens[:-1], dtype=np.int64)
    codes = np.zeros(max(1, int(lens.sum())), dtype=np.int8)
    for s, o in zip(seqs, offsets):
        codes[o : o + len(s)] = np.asarray(s, dtype=np.int8)
    return codes, offsets, lens


class Context:
    """One cwgpu_context on one CUDA device."""

    def __init__(self, device=0):
        self._lib = load()
        h = _vp()
        rc = self._lib.cwgpu_create(int(device), ctypes.byref(h))
        if rc:
            raise CwgpuError(rc, "cwgpu_create")
        self._h = h
        self.nseqs = 0
        from .autotune import env_override  # the knobs' environment override, if set

        forced = env_override()
        if forced is not None:
            self.set_tuning(*forced)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.cwgpu_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc, what):
        if rc:
            msg = self._lib.cwgpu_last_error(self._h)
            raise CwgpuError(rc, f"{what}: {msg.decode() if msg else ''}")

    @property
    def handle(self):
        return self._h

    def set_matrix(self, matrix):
        m = np.ascontiguousarray(np.asarray(matrix, dtype=np.int32).reshape(NUMRES * NUMRES))
        self._check(self._lib.cwgpu_set_matrix(self._h, _ptr(m)), "cwgpu_set_matrix")

    def set_params(self, params):
        p = params if isinstance(params, Params) else Params.from_dict(params)
        self._check(self._lib.cwgpu_set_params(self._h, ctypes.byref(p)), "cwgpu_set_params")

    def upload_seqs(self, seqs=None, packed=None):
        codes, offsets, lens = packed if packed is not None else pack_sequences(seqs)
        codes = np.ascontiguousarray(codes, dtype=np.int8)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        lens = np.ascontiguousarray(lens, dtype=np.int32)
        self._check(
            self._lib.cwgpu_upload_seqs(self._h, len(lens), _ptr(codes), _ptr(offsets), _ptr(lens)),
            "cwgpu_upload_seqs",
        )
        self.nseqs = len(lens)

    def align_pairs(self, pairs, stats=False, plain=False):
        pr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
        n = len(pr)
        dist = np.zeros(max(n, 1), dtype=np.float32)
        st = np.zeros(max(n, 1), dtype=PAIR_STATS_DTYPE) if stats else None
        fn = self._lib.cwgpu_align_pairs_plain if plain else self._lib.cwgpu_align_pairs
        self._check(fn(self._h, _ptr(pr), n, _ptr(dist), _ptr(st)), "cwgpu_align_pairs")
        return (dist[:n], st[:n]) if stats else dist[:n]

    def fast_align_pairs(self, pairs, fparams, stats=False):
        """Quick k-tuple distances (FastPairwiseAlign) of pairs [P, 2]: float64."""
        pr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
        n = len(pr)
        fp = fparams if isinstance(fparams, FastParams) else FastParams.from_dict(fparams)
        dist = np.zeros(max(n, 1), dtype=np.float64)
        st = np.zeros(max(n, 1), dtype=FAST_STATS_DTYPE) if stats else None
        self._check(self._lib.cwgpu_fast_align_pairs(self._h, ctypes.byref(fp), _ptr(pr), n, _ptr(dist), _ptr(st)),
                    "cwgpu_fast_align_pairs")
        return (dist[:n], st[:n]) if stats else dist[:n]

    def fast_align_pairs_device(self, fparams, d_pairs, d_order, npairs, d_dist, d_stats=None, stream=None):
        fp = fparams if isinstance(fparams, FastParams) else FastParams.from_dict(fparams)
        self._check(self._lib.cwgpu_fast_align_pairs_device(self._h, ctypes.byref(fp), d_pairs, d_order, int(npairs),
                                                            d_dist, d_stats, stream), "cwgpu_fast_align_pairs_device")

    def fast_pairwise_align(self, fparams, i_start, i_end, j_start, j_end, elements, dist_size, stats=False):
        npairs = range_pair_count(self.nseqs, i_start, i_end, j_start, j_end)
        fp = fparams if isinstance(fparams, FastParams) else FastParams.from_dict(fparams)
        st = np.zeros(max(npairs, 1), dtype=FAST_STATS_DTYPE) if stats else None
        rc = self._lib.cwgpu_fast_pairwise_align(self._h, ctypes.byref(fp), i_start, i_end, j_start, j_end,
                                                 _ptr(elements), int(dist_size), _ptr(st))
        self._check(rc, "cwgpu_fast_pairwise_align")
        return st[:npairs] if stats else None

    def pairwise_align(self, i_start, i_end, j_start, j_end, elements, dist_size, stats=False):
        npairs = range_pair_count(self.nseqs, i_start, i_end, j_start, j_end)
        st = np.zeros(max(npairs, 1), dtype=PAIR_STATS_DTYPE) if stats else None
        rc = self._lib.cwgpu_pairwise_align(
            self._h, i_start, i_end, j_start, j_end, _ptr(elements), int(dist_size), _ptr(st)
        )
        self._check(rc, "cwgpu_pairwise_align")
        return st[:npairs] if stats else None

    def plan(self, pairs):
        return Plan(self, pairs)

    def set_tuning(self, tiny_m, tiny_n, short_rows=None):
        """Sets the knobs of cwgpu_tuning; short_rows None keeps the current value."""
        if short_rows is None:
            short_rows = self.get_tuning()[2]
        t = Tuning(int(tiny_m), int(tiny_n), int(short_rows))
        self._check(self._lib.cwgpu_set_tuning(self._h, ctypes.byref(t)), "cwgpu_set_tuning")

    def get_tuning(self):
        t = Tuning()
        self._check(self._lib.cwgpu_get_tuning(self._h, ctypes.byref(t)), "cwgpu_get_tuning")
        return t.tiny_m, t.tiny_n, t.short_rows

    def set_cta_tuning(self, max_pairs=None, warps=None, large_rows=None):
        """Sets the knobs of cwgpu_cta_tuning; None keeps the current value."""
        cur = self.get_cta_tuning()
        t = CtaTuning(*(int(v if v is not None else c) for v, c in zip((max_pairs, warps, large_rows), cur)))
        self._check(self._lib.cwgpu_set_cta_tuning(self._h, ctypes.byref(t)), "cwgpu_set_cta_tuning")

    def get_cta_tuning(self):
        t = CtaTuning()
        self._check(self._lib.cwgpu_get_cta_tuning(self._h, ctypes.byref(t)), "cwgpu_get_cta_tuning")
        return t.max_pairs, t.warps, t.large_rows

    def cta_wait_probe(self, timeout_ns):
        """True if the CTA form's hand-over wait, run on a word nothing raises,
        ended at its limit with the timeout status."""
        out = ctypes.c_int32(0)
        self._check(self._lib.cwgpu_cta_wait_probe(self._h, int(timeout_ns), ctypes.byref(out)),
                    "cwgpu_cta_wait_probe")
        return bool(out.value)

    def synchronize(self):
        self._check(self._lib.cwgpu_synchronize(self._h), "cwgpu_synchronize")


class Plan:
    """cwgpu_plan: a device-resident pair list with a captured persistent launch."""

    def __init__(self, ctx, pairs):
        self.ctx = ctx
        self._lib = ctx._lib
        pr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
        self.npairs = len(pr)
        h = _vp()
        ctx._check(self._lib.cwgpu_plan_create(ctx.handle, _ptr(pr), self.npairs, ctypes.byref(h)), "cwgpu_plan_create")
        self._h = h

    def launch(self, stream=None):
        self.ctx._check(self._lib.cwgpu_plan_launch(self._h, stream), "cwgpu_plan_launch")

    def results(self, stats=False):
        dist = np.zeros(max(self.npairs, 1), dtype=np.float32)
        st = np.zeros(max(self.npairs, 1), dtype=PAIR_STATS_DTYPE) if stats else None
        self.ctx._check(self._lib.cwgpu_plan_results(self._h, _ptr(dist), _ptr(st)), "cwgpu_plan_results")
        return (dist[: self.npairs], st[: self.npairs]) if stats else dist[: self.npairs]

    def cell_counts(self):
        """(forward, reverse, diff) cell updates of the last run, as the reference counts them."""
        c = np.zeros(3, dtype=np.int64)
        self.ctx._check(self._lib.cwgpu_plan_cell_counts(self._h, _ptr(c)), "cwgpu_plan_cell_counts")
        return tuple(int(x) for x in c)

    def kernel_count(self):
        """Kernels one launch of this plan runs (long-pair and/or short-pair)."""
        return int(self._lib.cwgpu_plan_kernel_count(self._h))

    def pair_ctas(self):
        """True if the plan's long pairs run one CTA per pair."""
        return bool(self._lib.cwgpu_plan_pair_ctas(self._h))

    def device_dist_ptr(self):
        return self._lib.cwgpu_plan_device_dist(self._h)

    def close(self):
        if getattr(self, "_h", None):
            self._lib.cwgpu_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
