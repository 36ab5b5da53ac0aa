"""The C++ drop-ins (cuda-clustalw_gb300/host/GpuFullPairwiseAlign.cpp,
GpuFastPairwiseAlign.cpp, GpuNJTree.cpp) compiled against stand-in headers
(tests/dropin_shim: only the reference interfaces they use, so no reference
tree is needed) and linked with

* the GB300 library (lib/libcwgpu.so), on the GPU: the DistMatrix each
  pairwise drop-in fills equals the reference's stored one bit for bit, the
  guide-tree drop-in leaves the reference's branch lengths, tree description,
  joined matrix and verbose cycle report, and the lines the pairwise drop-ins
  print equal those of the same drop-ins linked with the oracle test double;
* the oracle test double (tests/dropin_stub_cwgpu.c), on the CPU: the same
  comparisons with the stand-in headers, which checks this harness itself.

tests/test_dropin_run.py runs the same drop-ins against the unmodified
reference headers and objects on the CPU (where the reference tree exists)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import REPO, load_fast_golden, load_golden, load_nj_golden

HOST = os.path.join(REPO, "cuda-clustalw_gb300", "host")
SOURCES = [os.path.join(HOST, f) for f in ("GpuFullPairwiseAlign.cpp", "GpuFastPairwiseAlign.cpp", "GpuNJTree.cpp")]
# -ffp-contract=off: no fused multiply-adds (the default of gcc on Arm), as the
# oracle itself is built (oracle/Makefile) and the reference computes on x86.
CXX = ["g++", "-std=gnu++98", "-O1", "-ffp-contract=off", "-I" + os.path.join(REPO, "tests", "dropin_shim"),
       "-I" + os.path.join(REPO, "include"), "-I" + HOST, os.path.join(REPO, "tests", "dropin_shim_main.cpp"), *SOURCES]


def build_stub(d):
    stub = str(d / "stub.o")
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-c", "-I" + os.path.join(REPO, "include"),
                    os.path.join(REPO, "tests", "dropin_stub_cwgpu.c"), "-o", stub], check=True)
    out = str(d / "dropin_shim_stub")
    subprocess.run([*CXX, stub, "-lm", "-o", out], check=True)
    return out


def build_gpu(d):
    from clustalw_gb300 import _build

    _build.build()
    out = str(d / "dropin_shim_gpu")
    subprocess.run([*CXX, "-L" + _build.LIB_DIR, "-lcwgpu", "-Wl,-rpath," + _build.LIB_DIR, "-o", out], check=True)
    return out


@pytest.fixture(scope="module")
def stub_bin(tmp_path_factory):
    return build_stub(tmp_path_factory.mktemp("shim_stub"))


@pytest.fixture(scope="module")
def gpu_bin(tmp_path_factory):
    return build_gpu(tmp_path_factory.mktemp("shim_gpu"))


def seq_text(seqs):
    return f"{len(seqs)}\n" + "".join(f"{len(s)} " + " ".join(str(int(c)) for c in s) + "\n" for s in seqs)


def full_input(g, display):
    p = g["params"]
    i0, i1, j0, j1 = g["range"]
    text = f"full 0 {i0} {i1} {j0} {j1} {int(display)}\n"
    text += f"{p['dna']} {p['int_scale']} {p['mat_avg']} {p['gap_pos1']} {p['gap_pos2']}\n"
    text += " ".join(float(p[k]).hex() for k in ("pw_gap_open", "pw_gap_extend", "gap_open_scale",
                                                   "gap_extend_scale")) + "\n"
    text += " ".join(str(int(v)) for v in np.asarray(g["matrix"]).ravel()) + "\n"
    return text + seq_text(g["seqs"])


def fast_input(g, display):
    fp = g["fast_params"]
    i0, i1, j0, j1 = g["range"]
    text = f"fast 0 {i0} {i1} {j0} {j1} {int(display)}\n"
    text += " ".join(str(fp[k]) for k in ("dna", "ktup", "window", "window_gap", "signif", "percent", "max_aa",
                                          "max_aln_length")) + "\n"
    return text + seq_text(g["seqs"])


def run(binary, text, tmp_path, tag):
    inp, out, rep = tmp_path / f"{tag}.in", tmp_path / f"{tag}.out", tmp_path / f"{tag}.report"
    inp.write_text(text)
    r = subprocess.run([binary, str(inp), str(out), str(rep)], capture_output=True, check=True)
    vals = out.read_text().split()
    return vals, r.stdout, rep.read_text() if rep.exists() else ""


def as_doubles(vals):
    return np.array([float.fromhex(v) for v in vals], dtype=np.float64)


def same_bits(a, b):
    return np.array_equal(np.asarray(a, np.float64).view(np.int64), np.asarray(b, np.float64).view(np.int64))


FULL_CPU = [("edge_protein", True), ("range_100_97_cols49", True), ("synth_dna_40x300", False)]
FAST_CPU = [("fast_edge_dna", True), ("fast_synth_protein_60x97", True)]
NJ_CPU = ["nj_random_3", "nj_random_5", "nj_ties_30", "nj_synth_uneven_40"]


def check_nj(binary, name, tmp_path):
    g = load_nj_golden(name)
    n = int(g["n"])
    text = f"nj 0 1 {n}\n" + " ".join(float(v).hex() for v in g["elements"]) + "\n"
    vals, _, report = run(binary, text, tmp_path, name)
    k = 0
    left = as_doubles(vals[k : k + n + 2]); k += n + 2
    right = as_doubles(vals[k : k + n + 2]); k += n + 2
    desc = np.array(vals[k : k + (n + 1) ** 2], dtype=np.int64).reshape(n + 1, n + 1); k += (n + 1) ** 2
    after = as_doubles(vals[k:])
    m = len(g["left"])
    assert same_bits(left[:m], g["left"]) and same_bits(right[:m], g["right"])
    assert np.array_equal(desc[: g["desc"].shape[0], : g["desc"].shape[1]], g["desc"])
    assert same_bits(after, g["elements_after"])
    assert report == str(g["report"])


@pytest.mark.parametrize("name,display", FULL_CPU)
def test_full_dropin_on_the_test_double(stub_bin, name, display, tmp_path):
    g = load_golden(name)
    vals, stdout, _ = run(stub_bin, full_input(g, display), tmp_path, name)
    assert same_bits(as_doubles(vals), g["elements"])
    if display:
        assert stdout.count(b"Sequences (") > 0


@pytest.mark.parametrize("name,display", FAST_CPU)
def test_fast_dropin_on_the_test_double(stub_bin, name, display, tmp_path):
    g = load_fast_golden(name)
    vals, _, _ = run(stub_bin, fast_input(g, display), tmp_path, name)
    assert same_bits(as_doubles(vals), g["elements"])


@pytest.mark.parametrize("name", NJ_CPU)
def test_nj_dropin_on_the_test_double(stub_bin, name, tmp_path):
    check_nj(stub_bin, name, tmp_path)


@pytest.mark.gpu
@pytest.mark.parametrize("name,display", FULL_CPU + [("fixture_100_97", False), ("fixture_100_1523", False),
                                                     ("range_100_97_block", True), ("limit_deep_16384", False)])
def test_full_dropin_on_the_gpu(gpu_bin, stub_bin, name, display, tmp_path):
    g = load_golden(name)
    text = full_input(g, display)
    vals, stdout, _ = run(gpu_bin, text, tmp_path, name + "_gpu")
    assert same_bits(as_doubles(vals), g["elements"])
    if display:  # the per-pair info lines and the matrix print, as with the oracle behind the ABI
        _, want, _ = run(stub_bin, text, tmp_path, name + "_stub")
        assert stdout == want and stdout.count(b"Sequences (") > 0


@pytest.mark.gpu
@pytest.mark.parametrize("name,display", FAST_CPU + [("fast_100_1523", False), ("fast_100_97_block", True)])
def test_fast_dropin_on_the_gpu(gpu_bin, stub_bin, name, display, tmp_path):
    g = load_fast_golden(name)
    text = fast_input(g, display)
    vals, stdout, _ = run(gpu_bin, text, tmp_path, name + "_gpu")
    assert same_bits(as_doubles(vals), g["elements"])
    if display:
        _, want, _ = run(stub_bin, text, tmp_path, name + "_stub")
        assert stdout == want


@pytest.mark.gpu
@pytest.mark.parametrize("name", NJ_CPU + ["nj_fixture_100_97", "nj_sequential_100_1800"])
def test_nj_dropin_on_the_gpu(gpu_bin, name, tmp_path):
    check_nj(gpu_bin, name, tmp_path)
