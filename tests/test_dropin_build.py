"""The C++ drop-ins (cuda-clustalw_gb300/host/GpuFullPairwiseAlign.cpp,
GpuFastPairwiseAlign.cpp and GpuNJTree.cpp) compile against the reference's own headers as C++98 and link
against the reference's objects plus lib/libcwgpu.so. Runs only where the reference tree and its
objects (oracle/build_ref.sh) are present."""
import glob
import os
import subprocess

import pytest

from conftest import REPO

REF_SRC = os.environ.get("CLUSTALW_REF_SRC", "/root/reference/CPU/clustalw-2.0.11/src")


@pytest.mark.skipif(not os.path.isdir(REF_SRC), reason="reference sources not present")
def test_dropin_compiles_and_links(tmp_path, oracle_mod):
    from clustalw_gb300 import _build

    lib = _build.build()
    objs = [o for o in glob.glob(os.path.join(REPO, "oracle", "_ref", "obj", "*.o"))]
    assert objs, "oracle/build_ref.sh did not build the reference objects"
    inc = ["-I" + REF_SRC, "-I" + os.path.join(REPO, "oracle", "_ref", "include"), "-I" + os.path.join(REPO, "include"),
           "-I" + os.path.join(REPO, "cuda-clustalw_gb300", "host")]
    out = str(tmp_path / "dropin")
    cmd = ["g++", "-std=gnu++98", "-w", "-DOS_UNIX=1", *inc,
           os.path.join(REPO, "cuda-clustalw_gb300", "host", "GpuFullPairwiseAlign.cpp"),
           os.path.join(REPO, "cuda-clustalw_gb300", "host", "GpuNJTree.cpp"),
           os.path.join(REPO, "cuda-clustalw_gb300", "host", "GpuFastPairwiseAlign.cpp"),
           os.path.join(REPO, "tests", "dropin_link_main.cpp"), *objs,
           "-L" + os.path.dirname(lib), "-lcwgpu", "-Wl,-rpath," + os.path.dirname(lib), "-o", out]
    subprocess.run(cmd, check=True)
    assert os.path.exists(out)
