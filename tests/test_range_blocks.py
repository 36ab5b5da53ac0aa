"""The range calls cut the reference's pair loops (FullPairwiseAlign.cpp:97,110)
into blocks of whole rows (cuda-clustalw_gb300/csrc/cwgpu_ranges.h): the blocks,
joined, are the loop order exactly; each holds at most the block limit unless a
single row is longer; `first` counts the pairs before the block; an empty range
still makes one call. Host code only: built with g++ and run on the CPU."""
import os
import subprocess

import numpy as np
import pytest

from conftest import REPO, range_pairs

INT32_MAX = 2**31 - 1


@pytest.fixture(scope="module")
def blocks_bin(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("ranges") / "range_blocks")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(REPO, "cuda-clustalw_gb300", "csrc"),
                    os.path.join(REPO, "tests", "range_blocks_main.cpp"), "-o", out], check=True)
    return out


def run_cases(binary, cases):
    text = "".join(" ".join(str(v) for v in c) + "\n" for c in cases)
    lines = subprocess.run([binary], input=text, capture_output=True, text=True, check=True).stdout.splitlines()
    result, k = [], 0
    while k < len(lines):
        assert lines[k] == "case"
        k += 1
        blocks = []
        while k < len(lines) and lines[k].startswith("block"):
            _, first, np_ = lines[k].split()
            vals = np.array(lines[k + 1].split(), dtype=np.int64).reshape(-1, 2)
            assert len(vals) == int(np_)
            blocks.append((int(first), vals))
            k += 2
        result.append(blocks)
    assert len(result) == len(cases)
    return result


def test_blocks_follow_the_reference_loop_order(blocks_bin):
    rng = np.random.default_rng(3)
    cases = [(10, 0, 10, 0, 10, 1), (10, 0, 10, 0, 10, 9), (10, 0, 10, 0, 10, 100), (10, 0, 10, 4, 10, 5),
             (10, 3, 7, 0, 10, 4), (10, 5, 5, 0, 10, 4), (10, 0, 100, 0, 100, 7), (10, 8, 20, 9, 30, 1),
             (0, 0, 0, 0, 0, 4), (1, 0, 1, 0, 1, 4), (10, 0, 10, 9, 10, 3), (10, 0, 10, 0, 10, 1 << 28)]
    for _ in range(60):
        n = int(rng.integers(0, 40))
        i0 = int(rng.integers(0, n + 3))
        i1 = int(rng.integers(i0, n + 5))
        j0 = int(rng.integers(0, n + 3))
        j1 = int(rng.integers(j0, n + 5))
        cases.append((n, i0, i1, j0, j1, int(rng.integers(1, 60))))
    for case, blocks in zip(cases, run_cases(blocks_bin, cases)):
        n, i0, i1, j0, j1, mx = case
        want = range_pairs(n, i0, i1, j0, j1).astype(np.int64)
        assert len(blocks) >= 1
        if len(want) == 0:
            assert [(f, len(v)) for f, v in blocks] == [(0, 0)], case
            continue
        got = np.concatenate([v for _, v in blocks])
        assert np.array_equal(got, want), case
        seen = 0
        for first, v in blocks:
            assert first == seen and len(v) > 0, case
            rows = np.unique(v[:, 0])
            assert len(v) <= mx or len(rows) == 1, case  # over the limit only as a single row
            seen += len(v)
        for (_, a), (_, b) in zip(blocks, blocks[1:]):
            assert a[-1, 0] < b[0, 0], case  # whole rows: no row is split across blocks
            # greedy: the next block's first row would have overflowed this one
            assert len(a) + np.count_nonzero(b[:, 0] == b[0, 0]) > mx, case


def test_extreme_column_start_selects_nothing(blocks_bin):
    (blocks,) = run_cases(blocks_bin, [(10, 0, 10, INT32_MAX, INT32_MAX, 4)])
    assert [(f, len(v)) for f, v in blocks] == [(0, 0)]
