"""Host-only pieces of the library, built with g++ and run on the CPU:

* the length key of the pair kernels' work order (cuda-clustalw_gb300/csrc/
  cwgpu_order.h): 16 * floor(log2 L) plus the 4 bits below the leading one,
  non-decreasing in L;
* the work order itself: a permutation of the call's pairs, the long-pair
  kernel's pairs (first sequence longer than short_rows) first, each part by
  non-increasing key sum, ties in call order;
* the device layout of the residue codes (cwgpu_layout.h): guard bytes, then
  per sequence its remapped codes and the same reversed, each zero-padded to 16
  bytes, then guard bytes. The pair kernels read residues without bounds
  checks on the strength of this layout."""
import os
import subprocess

import numpy as np
import pytest

from conftest import REPO

GUARD = 64


@pytest.fixture(scope="module")
def host_bin(tmp_path_factory):
    out = str(tmp_path_factory.mktemp("host_order") / "host_order")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(REPO, "cuda-clustalw_gb300", "csrc"),
                    os.path.join(REPO, "tests", "host_order_main.cpp"), "-o", out], check=True)
    return out


def run(binary, text):
    return subprocess.run([binary], input=text, capture_output=True, text=True, check=True).stdout.splitlines()


def key_of(L):
    if L <= 0:
        return 0
    e = L.bit_length() - 1
    m = (L >> (e - 4)) & 15 if e >= 4 else (L << (4 - e)) & 15
    return 16 * e + m


def test_length_key(host_bin):
    Ls = list(range(0, 300)) + [511, 512, 513, 1000, 1523, 4095, 4096, 65534, 65535]
    out = run(host_bin, "".join(f"key {L}\n" for L in Ls))
    keys = [int(line.split()[1]) for line in out]
    assert keys == [key_of(L) for L in Ls]
    assert all(0 <= k < 256 for k in keys)
    for L, k in zip(Ls, keys):
        if L > 0:  # a float's exponent and 4 mantissa bits: 16 log2 L - 2.4 < k <= 16 log2 L
            assert 16 * np.log2(L) - 2.4 < k <= 16 * np.log2(L) + 1e-9
    assert all(key_of(L) <= key_of(L + 1) for L in range(0, 70000))


@pytest.mark.parametrize("seed,short_rows", [(0, 128), (1, 0), (2, 65535), (3, 300)])
def test_work_order(host_bin, seed, short_rows):
    rng = np.random.default_rng(seed)
    n = 60
    lens = rng.integers(0, 3000, n)
    lens[:5] = [0, 1, 128, 129, 2000]
    np_ = 1500
    pairs = rng.integers(0, n, (np_, 2))
    text = f"order {n} {short_rows} {np_}\n" + " ".join(map(str, lens)) + "\n" + " ".join(map(str, pairs.ravel())) + "\n"
    out = run(host_bin, text)
    nlong = int(out[0].split()[1])
    order = np.array(out[1].split(), dtype=np.int64)
    assert sorted(order.tolist()) == list(range(np_))
    long_ = lens[pairs[:, 0]] > short_rows
    assert nlong == int(long_.sum())
    assert long_[order[:nlong]].all() and not long_[order[nlong:]].any()
    keysum = np.array([key_of(int(lens[a])) + key_of(int(lens[b])) for a, b in pairs])
    for part in (order[:nlong], order[nlong:]):
        ks = keysum[part]
        assert (np.diff(ks) <= 0).all()
        for k in np.unique(ks):  # ties keep the call order
            assert (np.diff(part[ks == k]) > 0).all()


def test_layout(host_bin):
    rng = np.random.default_rng(5)
    lens = np.array([0, 1, 15, 16, 17, 31, 97, 0, 200, 3])
    remap = rng.permutation(32) - 1  # includes -1, as the library's unused codes
    codes = [rng.integers(0, 32, L) for L in lens]
    text = f"layout {len(lens)}\n" + " ".join(map(str, lens)) + "\n" + " ".join(map(str, remap)) + "\n"
    text += " ".join(str(c) for s in codes for c in s) + "\n"
    out = run(host_bin, text)
    offs = np.array(out[0].split()[1:], dtype=np.int64)
    got = np.array(out[1].split()[1:], dtype=np.int64)
    want, o = [0] * GUARD, []
    for L, c in zip(lens, codes):
        pad = (L + 15) // 16 * 16
        o.append(len(want))
        fwd = [int(remap[x]) for x in c]
        want += fwd + [0] * (pad - L) + fwd[::-1] + [0] * (pad - L)
    want += [0] * GUARD
    assert offs.tolist() == o
    assert got.tolist() == want
    assert all(x % 16 == 0 for x in o)
