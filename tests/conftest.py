import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (REPO, os.path.join(REPO, "cuda-clustalw_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def load_golden(name):
    """A golden fixture written by tests/golden/make_golden.py from the reference."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    lens = z["lens"]
    offs = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int64) if len(lens) else np.zeros(0, np.int64)
    seqs = [z["codes"][o : o + L].astype(np.int8) for o, L in zip(offs, lens)]
    pi, pf = z["params_int"], z["params_float"]
    params = dict(
        dna=int(pi[0]),
        int_scale=int(pi[1]),
        mat_avg=int(pi[2]),
        gap_pos1=int(pi[3]),
        gap_pos2=int(pi[4]),
        pw_gap_open=float(pf[0]),
        pw_gap_extend=float(pf[1]),
        gap_open_scale=float(pf[2]),
        gap_extend_scale=float(pf[3]),
    )
    return dict(
        name=name,
        seqs=seqs,
        matrix=z["matrix"],
        params=params,
        range=tuple(int(x) for x in z["range"]),
        elements=z["elements"],
    )


def golden_names():
    """Full-pairwise fixtures with the default parameters (guide-tree fixtures
    start with nj_, quick k-tuple fixtures with fast_ or quicklimit_, other
    pairwise parameters with pwparams_, compact full-size ones with big_, the
    benchmark workloads' whole-set hashes with bench_)."""
    return sorted(f[:-4] for f in os.listdir(GOLDEN)
                  if f.endswith(".npz")
                  and not f.startswith(("nj_", "fast_", "quicklimit_", "quickparams_", "pwparams_", "big_", "bench_")))


def pw_variant_names():
    """Full-pairwise fixtures under the other protein pairwise matrices (BLOSUM,
    PAM, identity) and non-default gap penalties (protein and DNA)."""
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.startswith("pwparams_") and f.endswith(".npz"))


def big_golden_names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN)
                  if f.startswith("big_") and not f.startswith("big_extra_") and f.endswith(".npz"))


def load_big_extra(name):
    """Tree and quick-distance hashes for a compact full-size fixture
    (tests/golden/make_big_golden.py --extras); None if not generated."""
    path = os.path.join(GOLDEN, name.replace("big_", "big_extra_", 1) + ".npz")
    if not os.path.exists(path):
        return None
    z = np.load(path)
    return dict(nj_sha256=bytes(z["nj_sha256"]), fast_sha256=bytes(z["fast_sha256"]),
                fast_params=dict(zip(FAST_KEYS, (int(v) for v in z["fast_params"]))),
                fast_sample_idx=z["fast_sample_idx"], fast_sample_val=z["fast_sample_val"])


def load_big_golden(name):
    """A compact fixture written by tests/golden/make_big_golden.py: the
    reference's 1000-sequence test set, the SHA-256 of the DistMatrix the
    reference filled and a sample of its entries."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    lens = z["lens"]
    offs = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int64)
    seqs = [z["codes"][o : o + L].astype(np.int8) for o, L in zip(offs, lens)]
    pi, pf = z["params_int"], z["params_float"]
    params = dict(dna=int(pi[0]), int_scale=int(pi[1]), mat_avg=int(pi[2]), gap_pos1=int(pi[3]),
                  gap_pos2=int(pi[4]), pw_gap_open=float(pf[0]), pw_gap_extend=float(pf[1]),
                  gap_open_scale=float(pf[2]), gap_extend_scale=float(pf[3]))
    return dict(name=name, seqs=seqs, matrix=z["matrix"], params=params, range=tuple(int(x) for x in z["range"]),
                sha256=bytes(z["elements_sha256"]), n_elements=int(z["n_elements"]),
                sample_idx=z["sample_idx"], sample_val=z["sample_val"])


FAST_KEYS = ("dna", "ktup", "window", "window_gap", "signif", "percent", "max_aa", "max_aln_length")


def fast_golden_names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.startswith("fast_") and f.endswith(".npz"))


def quick_limit_names():
    """Quick-distance fixtures at the quick path's 8191-residue limit."""
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.startswith("quicklimit_") and f.endswith(".npz"))


def quick_variant_names():
    """Quick-distance fixtures under non-default ktup, window, window gap,
    significance and percent settings."""
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.startswith("quickparams_") and f.endswith(".npz"))


def load_fast_golden(name):
    """A quick-distance fixture: FastPairwiseAlign::pairwiseAlign of the reference
    (pairwise/FastPairwiseAlign.cpp:20-139) on the stored sequences."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    lens = z["lens"]
    offs = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int64) if len(lens) else np.zeros(0, np.int64)
    seqs = [z["codes"][o : o + L].astype(np.int8) for o, L in zip(offs, lens)]
    fp = dict(zip(FAST_KEYS, (int(v) for v in z["fast_params"])))
    return dict(name=name, seqs=seqs, fast_params=fp, range=[int(v) for v in z["range"]], elements=z["elements"])


def nj_golden_names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.startswith("nj_") and f.endswith(".npz"))


def load_nj_golden(name):
    """A guide-tree fixture: the reference NJTree::generateTree run on a packed
    DistMatrix (tree/NJTree.cpp:161-748)."""
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def range_pairs(n, i0, i1, j0, j1):
    out = [(si, sj) for si in range(max(0, i0), min(n, i1)) for sj in range(max(si + 1, j0 + 1), min(n, j1))]
    return np.array(out, dtype=np.int32).reshape(-1, 2)


def sym_index(pairs):
    """SymMatrix::getIndex for 1-based (si+1, sj+1), si < sj."""
    i = pairs[:, 0].astype(np.int64)
    j = pairs[:, 1].astype(np.int64)
    return (j * (j + 1)) // 2 + i


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O

    O.build()
    return O
