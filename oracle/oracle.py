"""ctypes wrapper of the oracle restatement (oracle/oracle.c) and a reader for
the reference harness output (oracle/ref_harness.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() to
check the GPU results and by bench.py's CPU-baseline leg. The product never imports it.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_HARNESS = os.path.join(HERE, "_ref", "refharness")

NUMRES = 32

PAIR_RESULT_DTYPE = np.dtype(
    [
        ("fwd_score", "<i4"),
        ("se1", "<i4"),
        ("se2", "<i4"),
        ("sb1", "<i4"),
        ("sb2", "<i4"),
        ("mm_score", "<i4"),
        ("n_ident", "<i4"),
        ("n_match", "<i4"),
        ("print_ptr", "<i4"),
        ("gap_open", "<i4"),
        ("gap_extend", "<i4"),
        ("dist", "<f4"),
        ("cells_fwd", "<i8"),
        ("cells_rev", "<i8"),
        ("cells_diff", "<i8"),
    ]
)
assert PAIR_RESULT_DTYPE.itemsize == 72


class Params(ctypes.Structure):
    """Mirror of cwo_params (oracle.c): the scalars FullPairwiseAlign reads."""

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


def build():
    """Compile oracle/oracle.c (and the reference harness when the reference is present)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    subprocess.run(["sh", os.path.join(HERE, "build_ref.sh")], check=True, stdout=subprocess.DEVNULL)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.cwo_align_pairs.restype = ctypes.c_int
        L.cwo_align_pairs.argtypes = [
            ctypes.c_void_p,
            ctypes.c_void_p,
            ctypes.c_void_p,
            ctypes.c_int32,
            ctypes.c_void_p,
            ctypes.POINTER(Params),
            ctypes.c_void_p,
            ctypes.c_int64,
            ctypes.c_void_p,
            ctypes.c_int32,
        ]
        L.cwo_nj_tree.restype = ctypes.c_int
        L.cwo_nj_tree.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                  ctypes.c_void_p]
        L.cwo_fast_pairs.restype = ctypes.c_int
        L.cwo_fast_pairs.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                     ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                     ctypes.c_int32]
        L.cwo_gap_penalties.restype = None
        L.cwo_gap_penalties.argtypes = [
            ctypes.POINTER(Params),
            ctypes.c_int,
            ctypes.c_int,
            ctypes.POINTER(ctypes.c_int32),
            ctypes.POINTER(ctypes.c_int32),
        ]
        _lib = L
    return _lib


def params_from(d):
    """Build Params from a dict with the field names of Params."""
    p = Params()
    for name, _ in Params._fields_:
        setattr(p, name, d[name])
    return p


def pack_sequences(seqs):
    """Concatenate a list of int code arrays into (codes int8, offsets int64, lens int32)."""
    lens = np.array([len(s) for s in seqs], dtype=np.int32)
    offsets = np.zeros(len(seqs), dtype=np.int64)
    if len(seqs) > 1:
        offsets[1:] = np.cumsum(lens[:-1], dtype=np.int64)
    codes = np.zeros(int(lens.sum()) + 1, dtype=np.int8)
    for s, o in zip(seqs, offsets):
        codes[o : o + len(s)] = np.asarray(s, dtype=np.int8)
    return codes, offsets, lens


def align_pairs(seqs, matrix, params, pairs, nthreads=None):
    """Run the oracle on `pairs` (array [P, 2] of 0-based (si, sj)); returns a
    structured array of PAIR_RESULT_DTYPE."""
    codes, offsets, lens = pack_sequences(seqs)
    mat = np.ascontiguousarray(np.asarray(matrix, dtype=np.int32).reshape(NUMRES, NUMRES))
    pr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
    out = np.zeros(len(pr), dtype=PAIR_RESULT_DTYPE)
    p = params_from(params) if isinstance(params, dict) else params
    if nthreads is None:
        nthreads = os.cpu_count() or 1
    rc = lib().cwo_align_pairs(
        codes.ctypes.data,
        offsets.ctypes.data,
        lens.ctypes.data,
        len(seqs),
        mat.ctypes.data,
        ctypes.byref(p),
        pr.ctypes.data,
        len(pr),
        out.ctypes.data,
        int(nthreads),
    )
    if rc != 0:
        raise RuntimeError(f"cwo_align_pairs failed with {rc}")
    return out


FAST_RESULT_DTYPE = np.dtype([("dist", "<f8"), ("score", "<i4"), ("frags", "<i4"), ("partial", "<i4"), ("pad", "<i4")])
assert FAST_RESULT_DTYPE.itemsize == 24


class FastParams(ctypes.Structure):
    """Mirror of cwo_fast_params: what FastPairwiseAlign::pairAlign reads."""

    _fields_ = [(k, ctypes.c_int32) for k in
                ("dna", "ktup", "window", "window_gap", "signif", "percent", "max_aa", "max_aln_length")]


def fast_pairs(seqs, fparams, pairs, nthreads=None):
    """k-tuple quick distances (oracle.c cwo_fast_pairs) for pairs [P, 2] of
    0-based (si, sj); returns a structured array of FAST_RESULT_DTYPE."""
    codes, offsets, lens = pack_sequences(seqs)
    pr = np.ascontiguousarray(np.asarray(pairs, dtype=np.int32).reshape(-1, 2))
    out = np.zeros(len(pr), dtype=FAST_RESULT_DTYPE)
    p = FastParams(*[int(fparams[k]) for k, _ in FastParams._fields_])
    rc = lib().cwo_fast_pairs(codes.ctypes.data, offsets.ctypes.data, lens.ctypes.data, len(seqs), ctypes.byref(p),
                              pr.ctypes.data, len(pr), out.ctypes.data, int(nthreads or os.cpu_count() or 1))
    if rc != 0:
        raise RuntimeError(f"cwo_fast_pairs failed with {rc}")
    return out


def nj_tree(n, elements, want_joins=False):
    """NJTree::generateTree restated (oracle.c cwo_nj_tree). Returns
    (left_branch[n+2], right_branch[n+2], tree_desc[(n+1),(n+1)], elements_after)
    and, with want_joins, the (mini, minj) of every cycle as a fifth item."""
    d = np.ascontiguousarray(np.array(elements, dtype=np.float64))
    left = np.zeros(n + 2, dtype=np.float64)
    right = np.zeros(n + 2, dtype=np.float64)
    desc = np.zeros((n + 1) * (n + 1), dtype=np.int32)
    joins = np.zeros((max(n - 3, 0) + 1, 2), dtype=np.int32)
    rc = lib().cwo_nj_tree(int(n), d.ctypes.data, left.ctypes.data, right.ctypes.data, desc.ctypes.data,
                           joins.ctypes.data)
    if rc != 0:
        raise RuntimeError("cwo_nj_tree failed")
    out = (left, right, desc.reshape(n + 1, n + 1), d)
    return out + (joins[: max(n - 3, 0)],) if want_joins else out


def run_reference_nj(n, elements, workdir, report=False):
    """Run the reference NJTree through the harness (built here only). With
    report=True also returns the reference's verbose cycle report as text."""
    inp = os.path.join(workdir, "nj_in.bin")
    out = os.path.join(workdir, "nj_out.bin")
    rep = os.path.join(workdir, "nj_report.txt")
    with open(inp, "wb") as f:
        f.write(np.int32(n).tobytes())
        f.write(np.asarray(elements, dtype="<f8").tobytes())
    subprocess.run([REF_HARNESS, "--nj", inp, out] + ([rep] if report else []), check=True, stdout=subprocess.DEVNULL)
    with open(out, "rb") as f:
        buf = f.read()
    off = 4
    left = np.frombuffer(buf, "<f8", n + 2, off).copy()
    off += 8 * (n + 2)
    right = np.frombuffer(buf, "<f8", n + 2, off).copy()
    off += 8 * (n + 2)
    desc = np.frombuffer(buf, "<i4", (n + 1) * (n + 1), off).copy().reshape(n + 1, n + 1)
    off += 4 * (n + 1) * (n + 1)
    nel = (n + 1) * (n + 2) // 2
    el = np.frombuffer(buf, "<f8", nel, off).copy()
    off += 8 * nel
    secs = float(np.frombuffer(buf, "<f8", 1, off)[0])
    if report:
        with open(rep) as f:
            return left, right, desc, el, secs, f.read()
    return left, right, desc, el, secs


def gap_penalties(params, n, m):
    p = params_from(params) if isinstance(params, dict) else params
    go = ctypes.c_int32()
    ge = ctypes.c_int32()
    lib().cwo_gap_penalties(ctypes.byref(p), int(n), int(m), ctypes.byref(go), ctypes.byref(ge))
    return go.value, ge.value


def range_pairs(nseqs, i_start, i_end, j_start, j_end):
    """The (si, sj) enumeration of FullPairwiseAlign.cpp:97,110 in loop order."""
    out = []
    for si in range(max(0, i_start), min(nseqs, i_end)):
        for sj in range(max(si + 1, j_start + 1), min(nseqs, j_end)):
            out.append((si, sj))
    return np.array(out, dtype=np.int32).reshape(-1, 2)


def sym_index(i, j):
    """SymMatrix::getIndex (general/SymMatrix.h:166-197) for 1-based i != j, both > 0."""
    a, b = i - 1, j - 1
    if a < b:
        a, b = b, a
    return (a * (a + 1)) // 2 + b


def read_ref_output(path):
    """Parse the binary written by oracle/ref_harness.cpp."""
    with open(path, "rb") as f:
        buf = f.read()
    assert buf[:8] in (b"CWREF01\0", b"CWREF02\0"), "bad magic"
    fast = buf[:8] == b"CWREF02\0"
    off = 8
    hdr = np.frombuffer(buf, dtype="<i4", count=7, offset=off)
    off += 28
    n, dna, int_scale, mat_avg, gp1, gp2, max_aln = (int(x) for x in hdr)
    fl = np.frombuffer(buf, dtype="<f4", count=4, offset=off)
    off += 16
    fast_params = None
    if fast:
        kp = np.frombuffer(buf, dtype="<i4", count=6, offset=off)
        off += 24
        fast_params = dict(dna=dna, ktup=int(kp[0]), window=int(kp[1]), window_gap=int(kp[2]), signif=int(kp[3]),
                           percent=int(kp[4]), max_aa=int(kp[5]), max_aln_length=max_aln)
    matrix = np.frombuffer(buf, dtype="<i4", count=NUMRES * NUMRES, offset=off).reshape(NUMRES, NUMRES).copy()
    off += 4 * NUMRES * NUMRES
    lens = np.frombuffer(buf, dtype="<i4", count=n, offset=off).copy()
    off += 4 * n
    seqs = []
    for L in lens:
        seqs.append(np.frombuffer(buf, dtype="<i4", count=int(L), offset=off).astype(np.int8))
        off += 4 * int(L)
    rng = np.frombuffer(buf, dtype="<i4", count=4, offset=off).copy()
    off += 16
    nel = (n + 1) * (n + 2) // 2
    elements = np.frombuffer(buf, dtype="<f8", count=nel, offset=off).copy()
    off += 8 * nel
    secs = float(np.frombuffer(buf, dtype="<f8", count=1, offset=off)[0])
    params = dict(
        dna=dna,
        pw_gap_open=float(fl[0]),
        pw_gap_extend=float(fl[1]),
        int_scale=int_scale,
        gap_open_scale=float(fl[2]),
        gap_extend_scale=float(fl[3]),
        mat_avg=mat_avg,
        gap_pos1=gp1,
        gap_pos2=gp2,
    )
    return dict(
        n=n,
        params=params,
        matrix=matrix,
        seqs=seqs,
        range=rng,
        elements=elements,
        seconds=secs,
        max_aln_length=max_aln,
        fast_params=fast_params,
    )


def run_reference(fasta, out_bin, rng=None, fast=False, overrides=None):
    """Run the reference harness (needs oracle/_ref/refharness, built here only);
    fast=True runs FastPairwiseAlign instead of FullPairwiseAlign. overrides:
    {"CWREF_PWMATRIX": "blosum"|"pam"|"gonnet"|"id", "CWREF_PWGAPOPEN": "...",
    "CWREF_PWGAPEXT": "..."}, applied as the reference's -pwmatrix, -pwgapopen
    and -pwgapext options would be."""
    if not os.path.exists(REF_HARNESS):
        raise FileNotFoundError(REF_HARNESS)
    cmd = [REF_HARNESS] + (["--fast"] if fast else []) + [fasta, out_bin]
    if rng is not None:
        cmd += [str(int(x)) for x in rng]
    env = dict(os.environ, **overrides) if overrides else None
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, env=env)
    return read_ref_output(out_bin)
