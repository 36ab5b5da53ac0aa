"""The whole clustalw2 program with the drop-ins bound in by the maintainer's
two-line edit (in a temporary copy of Clustal.cpp, `new
FullPairwiseAlign()` becomes `new GpuFullPairwiseAlign(0)` and `new
FastPairwiseAlign()` becomes `new GpuFastPairwiseAlign(0)`; every other
reference source compiles unchanged), writes the reference's shipped alignment
and guide tree (test_data/correct/*.aln, *.dnd) byte for byte, and with
-QUICKTREE the same files as the unmodified program.

The GPU library is replaced by tests/dropin_stub_cwgpu.c (the oracle behind the
same C ABI), so this checks the binding and the drop-ins' host code on a host
without a GPU. Runs only where the reference tree is present."""
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

import pytest

from conftest import REPO

REF_SRC = os.environ.get("CLUSTALW_REF_SRC", "/root/reference/CPU/clustalw-2.0.11/src")
REF_TREE = os.path.dirname(os.path.dirname(os.path.dirname(REF_SRC)))
CORRECT = os.path.join(REF_TREE, "test_data", "correct")
pytestmark = pytest.mark.skipif(not os.path.isdir(CORRECT), reason="reference tree not present")


def bind_dropins(text):
    """The maintainer's edit of Clustal.cpp: construct the drop-ins where the
    reference constructs FullPairwiseAlign and FastPairwiseAlign."""
    text = text.replace("new FullPairwiseAlign()", "new GpuFullPairwiseAlign(0)")
    text = text.replace("new FastPairwiseAlign()", "new GpuFastPairwiseAlign(0)")
    return text.replace('#include "pairwise/FastPairwiseAlign.h"',
                        '#include "pairwise/FastPairwiseAlign.h"\n#include "GpuFullPairwiseAlign.h"\n'
                        '#include "GpuFastPairwiseAlign.h"', 1)


@pytest.fixture(scope="module")
def programs():
    d = os.path.join(REPO, "oracle", "_ref", "pipeline")  # build outputs of reference code stay under oracle/_ref
    os.makedirs(d, exist_ok=True)
    host = os.path.join(REPO, "cuda-clustalw_gb300", "host")
    inc = os.path.join(d, "include")
    os.makedirs(inc, exist_ok=True)
    with open(os.path.join(inc, "clustalw_version.h"), "w") as f:
        f.write('#define CLUSTALW_NAME "ClustalW"\n#define CLUSTALW_VERSION "2.0.11"\n')
    flags = ["-O2", "-std=gnu++98", "-w", "-DOS_UNIX=1", "-I" + REF_SRC, "-I" + inc,
             "-I" + os.path.join(REPO, "include"), "-I" + host]
    with open(os.path.join(REF_SRC, "Clustal.cpp")) as f:
        original = f.read()
    bound = bind_dropins(original)
    assert bound.count("GpuFullPairwiseAlign(0)") == 4 and bound.count("GpuFastPairwiseAlign(0)") == 4
    # the edited Clustal.cpp is compiled from standard input: no copy of it is written
    subprocess.run(["g++", *flags, "-x", "c++", "-c", "-", "-o", os.path.join(d, "clustal_bound.o")],
                   input=bound.encode(), check=True)
    units = []
    for root, _, files in os.walk(REF_SRC):
        for name in files:
            if name.endswith(".cpp") and os.path.join(root, name) != os.path.join(REF_SRC, "Clustal.cpp"):
                units.append(os.path.join(root, name))
    jobs = [(u, os.path.join(d, "u%03d.o" % k)) for k, u in enumerate(sorted(units))]
    jobs += [(os.path.join(REF_SRC, "Clustal.cpp"), os.path.join(d, "clustal_ref.o")),
             (os.path.join(host, "GpuFullPairwiseAlign.cpp"), os.path.join(d, "gfull.o")),
             (os.path.join(host, "GpuFastPairwiseAlign.cpp"), os.path.join(d, "gfast.o"))]

    def compile_one(job):
        subprocess.run(["g++", *flags, "-c", job[0], "-o", job[1]], check=True)

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        list(ex.map(compile_one, jobs))
    stub = os.path.join(d, "stub.o")
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-c", "-I" + os.path.join(REPO, "include"),
                    os.path.join(REPO, "tests", "dropin_stub_cwgpu.c"), "-o", stub], check=True)
    common = [o for _, o in jobs[:len(units)]]
    ref_bin, bound_bin = os.path.join(d, "clustalw2"), os.path.join(d, "clustalw2_dropin")
    subprocess.run(["g++", *common, os.path.join(d, "clustal_ref.o"), "-lm", "-o", ref_bin], check=True)
    subprocess.run(["g++", *common, os.path.join(d, "clustal_bound.o"), os.path.join(d, "gfull.o"),
                    os.path.join(d, "gfast.o"), stub, "-lpthread", "-lm", "-o", bound_bin], check=True)
    return ref_bin, bound_bin


def run(binary, fasta, workdir, *opts):
    os.makedirs(workdir, exist_ok=True)
    fa = os.path.join(workdir, os.path.basename(fasta))
    shutil.copy(fasta, fa)
    subprocess.run([binary, "-INFILE=" + fa, "-ALIGN", "-QUIET", *opts], check=True, capture_output=True,
                   cwd=workdir)
    stem = fa[:-3]
    with open(stem + ".aln", "rb") as a, open(stem + ".dnd", "rb") as t:
        return a.read(), t.read()


@pytest.mark.parametrize("fx", ["100_97", "100_498"])
def test_bound_program_writes_the_shipped_outputs(programs, fx, tmp_path):
    aln, dnd = run(programs[1], os.path.join(CORRECT, fx + ".fa"), str(tmp_path))
    with open(os.path.join(CORRECT, fx + ".aln"), "rb") as f:
        assert aln == f.read()
    with open(os.path.join(CORRECT, fx + ".dnd"), "rb") as f:
        assert dnd == f.read()


def test_bound_program_quicktree_matches_the_unmodified_program(programs, tmp_path):
    fa = os.path.join(CORRECT, "100_97.fa")
    want = run(programs[0], fa, str(tmp_path / "ref"), "-QUICKTREE")
    got = run(programs[1], fa, str(tmp_path / "bound"), "-QUICKTREE")
    assert got == want
