"""The C++ drop-ins (cuda-clustalw_gb300/host/GpuFullPairwiseAlign.cpp,
GpuFastPairwiseAlign.cpp, GpuNJTree.cpp) run in a clustalw2-like process next
to the reference classes they replace, and leave exactly what those leave: the
DistMatrix, everything printed (per-pair lines and the matrix print with
display on), the guide tree and its verbose report, byte for byte.

The GPU library is replaced here by tests/dropin_stub_cwgpu.c, which answers
the same C ABI calls with the oracle restatement, so this checks the drop-ins'
own host code (what they read from the reference's globals, the SeqArray
flattening, ranges, DistMatrix writes, printing) on a host without a GPU; the
GPU tests check the library against the oracle and the reference. Runs only
where the reference tree and its objects (oracle/build_ref.sh) are present."""
import glob
import os
import subprocess

import pytest

from conftest import REPO, load_fast_golden, load_golden

REF_SRC = os.environ.get("CLUSTALW_REF_SRC", "/root/reference/CPU/clustalw-2.0.11/src")
REF_TREE = os.path.dirname(os.path.dirname(os.path.dirname(REF_SRC)))
pytestmark = pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference sources not present")


@pytest.fixture(scope="module")
def runner(tmp_path_factory, oracle_mod):
    objs = glob.glob(os.path.join(REPO, "oracle", "_ref", "obj", "*.o"))
    if not objs:
        pytest.skip("oracle/build_ref.sh did not build the reference objects")
    d = tmp_path_factory.mktemp("dropin_run")
    stub = str(d / "stub.o")
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-c", "-I" + os.path.join(REPO, "include"),
                    os.path.join(REPO, "tests", "dropin_stub_cwgpu.c"), "-o", stub], check=True)
    host = os.path.join(REPO, "cuda-clustalw_gb300", "host")
    out = str(d / "dropin_run")
    subprocess.run(["g++", "-std=gnu++98", "-w", "-DOS_UNIX=1", "-I" + REF_SRC,
                    "-I" + os.path.join(REPO, "oracle", "_ref", "include"), "-I" + os.path.join(REPO, "include"),
                    "-I" + os.path.join(REPO, "oracle"),
                    "-I" + host, os.path.join(host, "GpuFullPairwiseAlign.cpp"),
                    os.path.join(host, "GpuFastPairwiseAlign.cpp"), os.path.join(host, "GpuNJTree.cpp"),
                    os.path.join(REPO, "tests", "dropin_run_main.cpp"), *objs, stub, "-lpthread", "-lm", "-o", out],
                   check=True)
    return out


def fasta_of(name, tmp_path):
    from clustalw_gb300 import synth

    if name.startswith("shipped:"):
        return os.path.join(REF_TREE, name.split(":", 1)[1])
    if name.startswith("first2:"):  # two sequences: the tree's early return
        seqs = load_golden(name.split(":", 1)[1])["seqs"][:2]
    else:
        seqs = (load_fast_golden(name) if name.startswith("fast_") else load_golden(name))["seqs"]
    path = tmp_path / "in.fa"
    path.write_text(synth.to_fasta(seqs))
    return str(path)


def run_both(runner, kind, fasta, tmp_path, rng=(), overrides=None):
    outs = {}
    env = dict(os.environ, **(overrides or {}))
    for impl in ("ref", "dropin"):
        bin_path = tmp_path / f"{impl}_{kind}.bin"
        r = subprocess.run([runner, impl, kind, fasta, str(bin_path), *map(str, rng)], capture_output=True,
                           check=True, env=env)
        report = bin_path.with_name(bin_path.name + ".report")
        outs[impl] = (bin_path.read_bytes(), r.stdout, report.read_bytes() if report.exists() else b"")
    return outs


@pytest.mark.parametrize("kind", ["full", "fast"])
@pytest.mark.parametrize("source,rng", [("shipped:test_data/correct/100_97.fa", ()),
                                        ("shipped:test_data/correct/100_97.fa", (10, 30, 5, 60)),
                                        ("edge_protein", ()), ("fast_edge_dna", ()),
                                        ("synth_dna_40x300", (0, 40, 20, 40))])
def test_dropin_leaves_what_the_reference_leaves(runner, kind, source, rng, tmp_path):
    outs = run_both(runner, kind, fasta_of(source, tmp_path), tmp_path, rng)
    assert outs["ref"][1].count(b"Sequences (") > 0  # display on: the per-pair lines were printed
    assert outs["dropin"][0] == outs["ref"][0]  # DistMatrix
    assert outs["dropin"][1] == outs["ref"][1]  # standard output


@pytest.mark.parametrize("source", ["shipped:test_data/correct/100_97.fa", "edge_protein", "synth_uneven_40",
                                    "first2:fixture_100_97"])
def test_dropin_tree_leaves_what_the_reference_leaves(runner, source, tmp_path):
    outs = run_both(runner, "nj", fasta_of(source, tmp_path), tmp_path)
    assert len(outs["ref"][2]) > 0  # the verbose report was written
    assert outs["dropin"] == outs["ref"]  # tree, joined matrix, standard output, report


@pytest.mark.parametrize("kind,source,overrides", [
    ("full", "shipped:test_data/correct/100_97.fa", {"CWREF_PWMATRIX": "blosum", "CWREF_PWGAPOPEN": "3",
                                                     "CWREF_PWGAPEXT": "0.5"}),
    ("full", "shipped:test_data/correct/100_97.fa", {"CWREF_PWMATRIX": "id"}),
    ("full", "synth_dna_40x300", {"CWREF_PWGAPOPEN": "40", "CWREF_PWGAPEXT": "0"}),
    ("fast", "shipped:test_data/correct/100_97.fa", {"CWREF_KTUP": "2", "CWREF_WINDOW": "9", "CWREF_SIGNIF": "2"}),
    ("fast", "shipped:test_data/correct/100_97.fa", {"CWREF_PERCENT": "0", "CWREF_WINDOWGAP": "9"}),
    ("fast", "synth_dna_40x300", {"CWREF_KTUP": "3"}),
])
def test_dropin_reads_the_reference_settings(runner, kind, source, overrides, tmp_path):
    """Under non-default pairwise matrices, gap penalties and quick-distance
    settings (set in userParameters / subMatrix, as clustalw2's options do) the
    drop-ins still leave what the reference classes leave: they read those
    settings where the reference reads them."""
    outs = run_both(runner, kind, fasta_of(source, tmp_path), tmp_path, overrides=overrides)
    assert outs["dropin"][0] == outs["ref"][0]
    assert outs["dropin"][1] == outs["ref"][1]
