"""Writes compact golden fixtures for the reference's own 1000-sequence test
sets: the UNMODIFIED reference (ClustalW 2.0.11 FullPairwiseAlign, built by
oracle/build_ref.sh) fills the full DistMatrix, and only the sequences, the
scoring scheme, the SHA-256 of the packed DistMatrix (little-endian doubles)
and a seeded sample of its entries are stored (the matrices themselves are
4 MB each).

The reference is single-threaded, so the rows are split into ranges balanced
by pair count and run as parallel processes of the harness; each range fills
only its own entries, which are disjoint, and the ranges are summed. For
1000_97 the merged matrix is checked against one full run.

With --extras it adds, per set, big_extra_<name>.npz: the SHA-256 of what
the unmodified reference NJTree leaves (branches, treeDesc, joined matrix) on
that DistMatrix, and the SHA-256 and a sample of the DistMatrix the unmodified
FastPairwiseAlign (quick k-tuple distances) fills. The DistMatrix for the tree
is recomputed with the oracle on all cores and used only if its hash equals
the stored reference hash.

Run from the repository root, where the reference tree is available:
    python tests/golden/make_big_golden.py [--extras] [names...]
"""
import hashlib
import os
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, REPO)

from oracle import oracle as O  # noqa: E402

REF_ROOT = os.environ.get("CLUSTALW_REF_ROOT", "/root/reference")
FIXTURES = os.path.join(REF_ROOT, "test_data", "correct")
OUT = os.path.dirname(os.path.abspath(__file__))
NAMES = ["1000_97", "1000_498", "1000_1002", "1000_1523"]


def row_ranges(n, k):
    """k contiguous row ranges [i0, i1) of the pair triangle with about equal pair counts."""
    pairs_before = np.concatenate([[0], np.cumsum(np.arange(n - 1, -1, -1))])  # pairs of rows < i
    total = pairs_before[-1]
    cuts = [0]
    for t in range(1, k):
        cuts.append(int(np.searchsorted(pairs_before, total * t / k)))
    cuts.append(n)
    cuts = sorted(set(cuts))
    return [(a, b) for a, b in zip(cuts[:-1], cuts[1:]) if b > a]


def run_ranges(fasta, n, k, workdir, fast=False):
    ranges = row_ranges(n, k)

    def one(idx_rng):
        idx, (a, b) = idx_rng
        return O.run_reference(fasta, os.path.join(workdir, f"part{idx}.bin"), (a, b, 0, n), fast=fast)

    with ThreadPoolExecutor(max_workers=k) as ex:
        parts = list(ex.map(one, enumerate(ranges)))
    el = np.zeros_like(parts[0]["elements"])
    for p in parts:
        el += p["elements"]
    return parts[0], el


def main(names):
    k = os.cpu_count() or 4
    for name in names:
        fasta = os.path.join(FIXTURES, name + ".fa")
        with tempfile.TemporaryDirectory() as d:
            # the sequence count, from a run over an empty range
            meta = O.run_reference(fasta, os.path.join(d, "meta.bin"), (0, 0, 0, 0))
            n = int(meta["n"])
            ref, el = run_ranges(fasta, n, k, d)
            if name == "1000_97":
                full = O.run_reference(fasta, os.path.join(d, "full.bin"))
                assert np.array_equal(full["elements"].view(np.int64), el.view(np.int64)), "range merge differs"
        seqs = ref["seqs"]
        lens = np.array([len(s) for s in seqs], dtype=np.int32)
        p = ref["params"]
        digest = hashlib.sha256(np.ascontiguousarray(el, dtype="<f8").tobytes()).digest()
        rng = np.random.default_rng(1)
        iu = np.triu_indices(n, 1)  # 0-based (si, sj), si < sj
        pick = rng.choice(len(iu[0]), size=min(2000, len(iu[0])), replace=False)
        si, sj = iu[0][pick].astype(np.int64) + 1, iu[1][pick].astype(np.int64) + 1
        idx = ((sj * (sj - 1)) // 2 + (si - 1)).astype(np.int64)  # SymMatrix::getIndex(si, sj) for si < sj, 1-based
        np.savez_compressed(
            os.path.join(OUT, "big_" + name + ".npz"),
            codes=np.concatenate(seqs).astype(np.int8),
            lens=lens,
            matrix=ref["matrix"].astype(np.int32),
            params_int=np.array([p["dna"], p["int_scale"], p["mat_avg"], p["gap_pos1"], p["gap_pos2"]], np.int32),
            params_float=np.array(
                [p["pw_gap_open"], p["pw_gap_extend"], p["gap_open_scale"], p["gap_extend_scale"]], np.float32
            ),
            range=np.array([0, n, 0, n], np.int32),
            max_aln_length=np.int32(ref["max_aln_length"]),
            elements_sha256=np.frombuffer(digest, dtype=np.uint8),
            n_elements=np.int64(len(el)),
            sample_idx=idx,
            sample_val=el[idx],
        )
        print(f"big_{name}: {n} seqs, {len(el)} elements, sha256 {digest.hex()[:16]}...")


def sample_of(n, el):
    rng = np.random.default_rng(1)
    iu = np.triu_indices(n, 1)  # 0-based (si, sj), si < sj
    pick = rng.choice(len(iu[0]), size=min(2000, len(iu[0])), replace=False)
    si, sj = iu[0][pick].astype(np.int64), iu[1][pick].astype(np.int64)
    idx = (sj * (sj + 1)) // 2 + si
    return idx, el[idx]


def sha(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return np.frombuffer(h.digest(), dtype=np.uint8)


def extras(names):
    k = os.cpu_count() or 4
    for name in names:
        z = np.load(os.path.join(OUT, "big_" + name + ".npz"))
        lens = z["lens"]
        offs = np.concatenate([[0], np.cumsum(lens)[:-1]]).astype(np.int64)
        seqs = [z["codes"][o : o + L].astype(np.int8) for o, L in zip(offs, lens)]
        pi, pf = z["params_int"], z["params_float"]
        params = dict(dna=int(pi[0]), int_scale=int(pi[1]), mat_avg=int(pi[2]), gap_pos1=int(pi[3]),
                      gap_pos2=int(pi[4]), pw_gap_open=float(pf[0]), pw_gap_extend=float(pf[1]),
                      gap_open_scale=float(pf[2]), gap_extend_scale=float(pf[3]))
        n = len(seqs)
        pairs = np.array(O.range_pairs(n, 0, n, 0, n), dtype=np.int32).reshape(-1, 2)
        r = O.align_pairs(seqs, z["matrix"], params, pairs)
        el = np.zeros(int(z["n_elements"]))
        el[(pairs[:, 1].astype(np.int64) * (pairs[:, 1] + 1)) // 2 + pairs[:, 0]] = r["dist"].astype(np.float64)
        assert bytes(sha(el.astype("<f8"))) == bytes(z["elements_sha256"]), "oracle DistMatrix differs from the reference's"
        fasta = os.path.join(FIXTURES, name + ".fa")
        with tempfile.TemporaryDirectory() as d:
            left, right, desc, el_after, _ = O.run_reference_nj(n, el, d)
            ref, el_fast = run_ranges(fasta, n, k, d, fast=True)
            if name == "1000_97":
                full = O.run_reference(fasta, os.path.join(d, "fast_full.bin"), fast=True)
                assert np.array_equal(full["elements"].view(np.int64), el_fast.view(np.int64)), "range merge differs"
        idx, val = sample_of(n, el_fast)
        fp = ref["fast_params"]
        np.savez_compressed(
            os.path.join(OUT, "big_extra_" + name + ".npz"),
            nj_sha256=sha(left.astype("<f8"), right.astype("<f8"), desc.astype("<i4"), el_after.astype("<f8")),
            fast_params=np.array([fp[k2] for k2 in ("dna", "ktup", "window", "window_gap", "signif", "percent",
                                                     "max_aa", "max_aln_length")], np.int32),
            fast_sha256=sha(el_fast.astype("<f8")),
            fast_sample_idx=idx,
            fast_sample_val=val,
        )
        print(f"big_extra_{name}: tree and quick distances of {n} sequences")


if __name__ == "__main__":
    args = sys.argv[1:]
    if args and args[0] == "--extras":
        extras(args[1:] or NAMES)
    else:
        main(args or NAMES)
