"""Writes the golden fixtures under tests/golden/ by running the UNMODIFIED
reference (ClustalW 2.0.11 FullPairwiseAlign, built by oracle/build_ref.sh)
through oracle/_ref/refharness.

Run from the repository root, where the reference tree is available:
    python tests/golden/make_golden.py
(--nj-only, --fast-only, --limits, --pw-variants or --sequential writes only the
guide-tree, quick-distance, length-limit, parameter-variant or src/sequential
fixtures.)

Each <name>.npz holds the encoded sequences exactly as the reference's reader
produced them, the pairwise matrix and scalars the reference used, the range,
and the reference's full packed DistMatrix (double). It also refreshes
cuda-clustalw_gb300/clustalw_gb300/data/pairwise_matrices.json (the default
protein and DNA pairwise matrices).
"""
import json
import os
import sys
import tempfile

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "cuda-clustalw_gb300"))

from clustalw_gb300 import synth  # noqa: E402
from oracle import oracle as O  # noqa: E402

REF_ROOT = os.environ.get("CLUSTALW_REF_ROOT", "/root/reference")
FIXTURES = os.path.join(REF_ROOT, "test_data", "correct")
OUT = os.path.dirname(os.path.abspath(__file__))


def save(name, ref):
    seqs = ref["seqs"]
    lens = np.array([len(s) for s in seqs], dtype=np.int32)
    codes = np.concatenate(seqs).astype(np.int8) if len(seqs) else np.zeros(0, np.int8)
    p = ref["params"]
    np.savez_compressed(
        os.path.join(OUT, name + ".npz"),
        codes=codes,
        lens=lens,
        matrix=ref["matrix"].astype(np.int32),
        params_int=np.array([p["dna"], p["int_scale"], p["mat_avg"], p["gap_pos1"], p["gap_pos2"]], np.int32),
        params_float=np.array(
            [p["pw_gap_open"], p["pw_gap_extend"], p["gap_open_scale"], p["gap_extend_scale"]], np.float32
        ),
        range=ref["range"].astype(np.int32),
        elements=ref["elements"],
        max_aln_length=np.int32(ref["max_aln_length"]),
    )
    print(f"{name}: {ref['n']} seqs, range {list(ref['range'])}, ref {ref['seconds']:.2f}s")


def run_fasta(text, name, rng=None, overrides=None):
    with tempfile.TemporaryDirectory() as d:
        fa = os.path.join(d, name + ".fa")
        with open(fa, "w") as f:
            f.write(text)
        return O.run_reference(fa, os.path.join(d, "out.bin"), rng, overrides=overrides)


def save_fast(name, ref):
    """k-tuple quick distances (FastPairwiseAlign) fixture: the sequences as
    the reference's reader encoded them, the userParameters values the call
    used, the range and the reference's DistMatrix."""
    seqs = ref["seqs"]
    lens = np.array([len(s) for s in seqs], dtype=np.int32)
    codes = np.concatenate(seqs).astype(np.int8) if len(seqs) else np.zeros(0, np.int8)
    fp = ref["fast_params"]
    np.savez_compressed(os.path.join(OUT, name + ".npz"), codes=codes, lens=lens,
                        fast_params=np.array([fp[k] for k in FAST_KEYS], np.int32),
                        range=ref["range"].astype(np.int32), elements=ref["elements"])
    print(f"{name}: {ref['n']} seqs, range {list(ref['range'])}, ref {ref['seconds']:.2f}s")


FAST_KEYS = ("dna", "ktup", "window", "window_gap", "signif", "percent", "max_aa", "max_aln_length")


def make_fast():
    """Quick (k-tuple) distances of the reference fixtures, a partial range,
    synthetic sets and the edge-case set."""
    with tempfile.TemporaryDirectory() as d:
        for fx in ["100_97", "100_498", "100_1002", "100_1523"]:
            save_fast("fast_" + fx, O.run_reference(os.path.join(FIXTURES, fx + ".fa"), os.path.join(d, "o.bin"),
                                                    fast=True))
        save_fast("fast_100_97_block", O.run_reference(os.path.join(FIXTURES, "100_97.fa"), os.path.join(d, "o.bin"),
                                                       (20, 60, 40, 70), fast=True))
        for fx in ["100_500", "100_1000", "100_1800"]:
            save_fast("fast_sequential_" + fx, O.run_reference(os.path.join(SEQUENTIAL, fx + ".fa"),
                                                               os.path.join(d, "o.bin"), fast=True))
    for name, text in fast_sets():
        with tempfile.TemporaryDirectory() as d:
            fa = os.path.join(d, "s.fa")
            with open(fa, "w") as f:
                f.write(text)
            save_fast("fast_" + name, O.run_reference(fa, os.path.join(d, "o.bin"), fast=True))


def fast_sets():
    uneven = []
    for f, L in enumerate([5, 30, 170, 600]):
        uneven += synth.protein_family(10, L, 100 + f)
    edge = ["W", "MA", "MKTAYIAKQRQISFVKSHFSRQ", "MKTAYIAKQRQISFVKSHFSRQ", "AAAAAAAAAAAAAAAAAAAA",
            "AAAAAAAAAAGAAAAAAAAA", "MK--LVAG-HHW", "----", "XXXXBZBZXX", "GGGGGGGG", "KR",
            "ACDEFGHIKLMNPQRSTVWY" * 12, "WWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWW", "MSLLTEVETPTRNGWECKCSDSSD", "P"]
    dna_edge = ["A", "AC", "ACGT" * 30, "ACGT" * 30, "AAAAAAAAAAAAAAAAAAAAAAAA", "ACGTNNNNACGT", "ACGU" * 10,
                "GATTACA" * 9, "TTTTTTTTTTGTTTTTTTTT", "CCGG"]
    return [
        ("synth_protein_60x97", synth.to_fasta(synth.protein_family(60, 97, 11))),
        ("synth_dna_40x300", synth.to_fasta(synth.dna_family(40, 300, 12))),
        ("synth_uneven_40", synth.to_fasta(uneven)),
        ("edge_protein", "".join(f">e{i}\n{x}\n" for i, x in enumerate(edge))),
        ("edge_dna", "".join(f">d{i}\n{x}\n" for i, x in enumerate(dna_edge))),
    ]


def save_nj(name, n, elements):
    """NJ fixture: inputs, the reference's tree and joined matrix, and its
    verbose cycle report (NJTree.cpp:209-236, 413-470, 694-740)."""
    with tempfile.TemporaryDirectory() as d:
        left, right, desc, el, secs, report = O.run_reference_nj(n, elements, d, report=True)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), n=np.int32(n), elements=np.asarray(elements, np.float64),
                        left=left, right=right, desc=desc, elements_after=el, report=np.array(report))
    print(f"{name}: NJ on {n} sequences, ref {secs:.4f}s")


def make_nj():
    """Guide trees (NJTree::generateTree) of the reference's own distance matrices,
    plus small and tie-heavy matrices."""
    import glob

    for path in (sorted(glob.glob(os.path.join(OUT, "fixture_*.npz"))) + [os.path.join(OUT, "synth_uneven_40.npz")]
                 + sorted(glob.glob(os.path.join(OUT, "sequential_*.npz")))):
        z = np.load(path)
        n = len(z["lens"])
        save_nj("nj_" + os.path.basename(path)[:-4], n, z["elements"])
    rng = np.random.default_rng(7)
    for n in (3, 4, 5, 9):
        el = np.zeros((n + 1) * (n + 2) // 2)
        for i in range(1, n + 1):
            for j in range(1, i):
                el[(i - 1) * i // 2 + (j - 1)] = float(np.float32(rng.uniform(0.05, 0.9)))
        save_nj(f"nj_random_{n}", n, el)
    # Ties: groups of identical sequences (distance 0) and repeated distances.
    n = 30
    grp = rng.integers(0, 6, size=n)
    el = np.zeros((n + 1) * (n + 2) // 2)
    for i in range(1, n + 1):
        for j in range(1, i):
            el[(i - 1) * i // 2 + (j - 1)] = 0.0 if grp[i - 1] == grp[j - 1] else float(np.float32(0.1 * (1 + (grp[i - 1] + grp[j - 1]) % 4)))
    save_nj("nj_ties_30", n, el)


def make_limits():
    """Sequences at the length limit (synth.length_limit_set): the 65,535-residue
    sequence with its 300- and 100-residue fragments, and the 16,384-residue
    pair whose Myers-Miller stage recurses 14 levels."""
    seqs = synth.length_limit_set()
    save("limit_65535", run_fasta(synth.to_fasta([seqs[0], seqs[1], seqs[4]]), "m"))
    save("limit_deep_16384", run_fasta(synth.to_fasta([seqs[2], seqs[3]]), "q"))


def make_quick_limits():
    """Quick distances at the quick path's length limit (8191 residues):
    protein (ktup 1) and DNA (ktup 2) sets of an 8191-residue sequence, a
    mutated copy of it and a fragment. Named quicklimit_*: only the oracle
    test reads them."""
    rng = np.random.default_rng(8191)

    def mutate(seq, rate, codes):
        seq = seq.copy()
        hit = rng.random(len(seq)) < rate
        seq[hit] = codes[rng.integers(0, len(codes), int(hit.sum()))]
        return seq[rng.random(len(seq)) >= 0.01]

    for tag, codes, probs in (("protein", synth.PROTEIN_CODES, synth.PROTEIN_PROBS),
                              ("dna", synth.DNA_CODES, synth.DNA_PROBS)):
        full = codes[rng.choice(len(codes), size=8191, p=probs)].astype(np.int8)
        seqs = [full, mutate(full, 0.15, codes), mutate(full[2000:2600], 0.1, codes)]
        with tempfile.TemporaryDirectory() as d:
            fa = os.path.join(d, "s.fa")
            with open(fa, "w") as f:
                f.write(synth.to_fasta(seqs))
            save_fast("quicklimit_" + tag + "_8191", O.run_reference(fa, os.path.join(d, "o.bin"), fast=True))


PW_VARIANTS = [
    # (name, protein?, overrides): the other protein pairwise matrices and
    # non-default gap penalties, as -pwmatrix / -pwgapopen / -pwgapext set them
    ("blosum", True, {"CWREF_PWMATRIX": "blosum"}),
    ("pam", True, {"CWREF_PWMATRIX": "pam"}),
    ("id", True, {"CWREF_PWMATRIX": "id"}),
    ("gonnet_go3_ge05", True, {"CWREF_PWGAPOPEN": "3.0", "CWREF_PWGAPEXT": "0.5"}),
    ("blosum_go25_ge1", True, {"CWREF_PWMATRIX": "blosum", "CWREF_PWGAPOPEN": "25", "CWREF_PWGAPEXT": "1"}),
    ("dna_go5_ge2", False, {"CWREF_PWGAPOPEN": "5", "CWREF_PWGAPEXT": "2"}),
    ("dna_go40_ge0", False, {"CWREF_PWGAPOPEN": "40", "CWREF_PWGAPEXT": "0"}),
]


def make_pw_variants():
    """Full-pairwise DistMatrices under the other pairwise matrices and gap
    penalties (named pwparams_*: only the oracle test reads them)."""
    prot = synth.to_fasta(synth.protein_family(30, 120, 41))
    dna = synth.to_fasta(synth.dna_family(30, 150, 42))
    for name, protein, ov in PW_VARIANTS:
        save("pwparams_" + name, run_fasta(prot if protein else dna, name, overrides=ov))


QUICK_VARIANTS = [
    # (name, protein?, overrides): the quick-distance settings the GPU tests vary
    ("prot_ktup2", True, {"CWREF_KTUP": "2"}),
    ("prot_window1", True, {"CWREF_WINDOW": "1"}),
    ("prot_window9_signif2", True, {"CWREF_WINDOW": "9", "CWREF_SIGNIF": "2"}),
    ("prot_signif12", True, {"CWREF_SIGNIF": "12"}),
    ("prot_windowgap1", True, {"CWREF_WINDOWGAP": "1"}),
    ("prot_windowgap9", True, {"CWREF_WINDOWGAP": "9"}),
    ("prot_percent0", True, {"CWREF_PERCENT": "0"}),
    ("dna_ktup1", False, {"CWREF_KTUP": "1"}),
    ("dna_ktup3", False, {"CWREF_KTUP": "3"}),
    ("dna_ktup4", False, {"CWREF_KTUP": "4"}),
]


def make_quick_variants():
    """Quick distances under non-default settings (named quickparams_*: only
    the oracle test reads them)."""
    prot = synth.to_fasta(synth.protein_family(24, 160, 31) + synth.protein_family(8, 40, 32))
    dna = synth.to_fasta(synth.dna_family(20, 300, 41))
    for name, protein, ov in QUICK_VARIANTS:
        with tempfile.TemporaryDirectory() as d:
            fa = os.path.join(d, "s.fa")
            with open(fa, "w") as f:
                f.write(prot if protein else dna)
            save_fast("quickparams_" + name, O.run_reference(fa, os.path.join(d, "o.bin"), fast=True, overrides=ov))


SEQUENTIAL = os.path.join(REF_ROOT, "CPU", "clustalw-2.0.11", "src", "sequential")


def make_sequential():
    """The reference's other shipped inputs, src/sequential/100_{500,1000,1800}.fa
    (protein; their .aln/.dnd are the reference's own CPU outputs): the whole
    DistMatrix, filled in row ranges on all host cores (each range writes only
    its own entries) and summed."""
    from make_big_golden import run_ranges

    k = os.cpu_count() or 4
    for fx in ["100_500", "100_1000", "100_1800"]:
        fasta = os.path.join(SEQUENTIAL, fx + ".fa")
        with tempfile.TemporaryDirectory() as d:
            n = int(O.run_reference(fasta, os.path.join(d, "meta.bin"), (0, 0, 0, 0))["n"])
            ref, el = run_ranges(fasta, n, k, d)
        ref = dict(ref, elements=el, range=np.array([0, n, 0, n], np.int32))
        save("sequential_" + fx, ref)


def main():
    O.build()
    mats = {}
    for fx in ["100_97", "100_498", "100_1002", "100_1523"]:
        with tempfile.TemporaryDirectory() as d:
            ref = O.run_reference(os.path.join(FIXTURES, fx + ".fa"), os.path.join(d, "o.bin"))
        save("fixture_" + fx, ref)
        kind = "dna" if ref["params"]["dna"] else "protein"
        mats.setdefault(kind, {"matrix": ref["matrix"].reshape(-1).tolist(), "params": ref["params"]})
        if fx == "100_97":
            n = ref["n"]
            # Partial ranges, as Clustal::sequencesAlignToProfile (Clustal.cpp:404-416) and
            # other callers pass them (FullPairwiseAlign.cpp:97,110).
            for tag, rng in [("cols49", (0, n, 49, n)), ("rows10_30", (10, 30, 0, n)), ("block", (20, 60, 40, 70))]:
                with tempfile.TemporaryDirectory() as d:
                    r2 = O.run_reference(os.path.join(FIXTURES, fx + ".fa"), os.path.join(d, "o.bin"), rng)
                save(f"range_{fx}_{tag}", r2)

    save("synth_protein_60x97", run_fasta(synth.to_fasta(synth.protein_family(60, 97, 11)), "p"))
    save("synth_dna_40x300", run_fasta(synth.to_fasta(synth.dna_family(40, 300, 12)), "d"))
    uneven = []
    for f, L in enumerate([5, 30, 170, 600]):
        uneven += synth.protein_family(10, L, 100 + f)
    save("synth_uneven_40", run_fasta(synth.to_fasta(uneven), "u"))
    save("synth_long_6x3000", run_fasta(synth.to_fasta(synth.protein_family(6, 3000, 13)), "l"))

    # Edge cases: length-1 and length-2 sequences, identical sequences, runs
    # that create ties, internal gaps, an all-gap sequence, ambiguity codes,
    # and a short-vs-long pair.
    edge = [
        "W",
        "MA",
        "MKTAYIAKQRQISFVKSHFSRQ",
        "MKTAYIAKQRQISFVKSHFSRQ",
        "AAAAAAAAAAAAAAAAAAAA",
        "AAAAAAAAAAGAAAAAAAAA",
        "MK--LVAG-HHW",
        "----",
        "XXXXBZBZXX",
        "GGGGGGGG",
        "KR",
        "ACDEFGHIKLMNPQRSTVWY" * 12,
        "WWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWWW",
        "MSLLTEVETPTRNGWECKCSDSSD",
        "P",
    ]
    text = "".join(f">e{i}\n{s}\n" for i, s in enumerate(edge))
    save("edge_protein", run_fasta(text, "e"))

    make_limits()
    make_nj()
    make_fast()
    make_quick_limits()
    make_pw_variants()
    make_quick_variants()
    make_sequential()

    os.makedirs(os.path.join(REPO, "cuda-clustalw_gb300", "clustalw_gb300", "data"), exist_ok=True)
    with open(os.path.join(REPO, "cuda-clustalw_gb300", "clustalw_gb300", "data", "pairwise_matrices.json"), "w") as f:
        json.dump(mats, f, indent=0)
    print("wrote pairwise_matrices.json with", sorted(mats))


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--nj-only":
        O.build()
        make_nj()
    elif len(sys.argv) > 1 and sys.argv[1] == "--fast-only":
        O.build()
        make_fast()
    elif len(sys.argv) > 1 and sys.argv[1] == "--limits":
        O.build()
        make_limits()
        make_quick_limits()
    elif len(sys.argv) > 1 and sys.argv[1] == "--sequential":
        O.build()
        make_sequential()
    elif len(sys.argv) > 1 and sys.argv[1] == "--pw-variants":
        O.build()
        make_pw_variants()
        make_quick_variants()
    else:
        main()
