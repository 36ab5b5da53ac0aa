"""The Python mirror of the reference's pairwise plugin interface
(clustalw_gb300.pairwise): SymMatrix index rule and bounds, the reference's
error behaviour for a wrong matrix size and bad ranges (message + exit 1, no
device work), residue encoding, and -- on the GPU -- pairwiseAlign filling a
DistMatrix exactly as the reference's FullPairwiseAlign did (golden fixtures,
full and partial ranges), with the same per-pair info lines; on the CPU, the
info lines built from per-pair identity counts equal the ones the unmodified
reference prints."""
import numpy as np
import pytest

from conftest import load_golden, sym_index


def test_symmatrix_index_rule():
    from clustalw_gb300.pairwise import SymMatrix

    m = SymMatrix(7)  # 6 sequences
    seen = set()
    for i in range(1, 7):
        for j in range(1, 7):
            k = m.getIndex(i, j)
            assert k == m.getIndex(j, i)
            if i != j:
                seen.add(k)
    assert m.getIndex(0, 3) == 0 and m.getIndex(3, 0) == 0
    assert len(seen) == 15
    pairs = np.array([(a, b) for a in range(6) for b in range(a + 1, 6)])
    assert sorted(seen) == sorted(sym_index(pairs).tolist())
    with pytest.raises(IndexError):
        m.getIndex(7, 1)
    m.SetAt(2, 5, 0.25)
    assert m.GetAt(5, 2) == 0.25


def test_reference_error_behaviour(capsys):
    from clustalw_gb300.pairwise import Alignment, DistMatrix, FullPairwiseAlign, PairwiseSettings

    g = load_golden("synth_uneven_40")
    aln = Alignment(g["seqs"][:5])
    fpa = FullPairwiseAlign(PairwiseSettings(g["matrix"], g["params"]))
    with pytest.raises(SystemExit) as e:
        fpa.pairwiseAlign(aln, DistMatrix(5), 0, 5, 0, 5)  # needs size 6
    assert e.value.code == 1
    assert "The distance matrix is not the right size!" in capsys.readouterr().out
    for rng in [(-1, 5, 0, 5), (3, 2, 0, 5), (0, 5, -1, 5), (0, 5, 4, 3)]:
        with pytest.raises(SystemExit) as e:
            fpa.pairwiseAlign(aln, DistMatrix(6), *rng)
        assert e.value.code == 1
        assert "The range for pairwise Alignment is incorrect." in capsys.readouterr().out
    # No sequences: returns without touching the device.
    fpa.pairwiseAlign(Alignment([]), DistMatrix(1), 0, 0, 0, 0)



def test_quick_mirror_error_behaviour(capsys):
    """FastPairwiseAlign's mirror rejects a wrong matrix size and bad ranges
    with the reference's messages and exit status 1 (FastPairwiseAlign.cpp:
    24-35), before any device work."""
    from clustalw_gb300.pairwise import Alignment, DistMatrix, FastPairwiseAlign

    g = load_golden("synth_uneven_40")
    aln = Alignment(g["seqs"][:5])
    fpa = FastPairwiseAlign()
    with pytest.raises(SystemExit) as e:
        fpa.pairwiseAlign(aln, DistMatrix(5), 0, 5, 0, 5)
    assert e.value.code == 1
    assert capsys.readouterr().out == "The distance matrix is not the right size!\nNeed to terminate program.\n"
    for rng in [(-1, 5, 0, 5), (3, 2, 0, 5), (0, 5, -1, 5), (0, 5, 4, 3)]:
        with pytest.raises(SystemExit) as e:
            fpa.pairwiseAlign(aln, DistMatrix(6), *rng)
        assert e.value.code == 1
        assert capsys.readouterr().out == "The range for pairwise Alignment is incorrect.\nNeed to terminate program.\n"


def test_encode_decode():
    from clustalw_gb300.pairwise import GAP_POS2, decode, encode

    c = encode("ACDEFGHIKLMNPQRSTVWYbzx-")
    assert c[-1] == GAP_POS2 and c[0] == 0 and c[1] == 2
    assert decode(c) == "ACDEFGHIKLMNPQRSTVWYBZX-"
    with pytest.raises(ValueError):
        encode("AJ")


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["fixture_100_97", "range_100_97_cols49", "range_100_97_block", "edge_protein"])
def test_pairwise_align_fills_distmatrix_like_reference(name):
    from clustalw_gb300.pairwise import Alignment, DistMatrix, FullPairwiseAlign, PairwiseSettings

    g = load_golden(name)
    aln = Alignment(g["seqs"])
    dm = DistMatrix(aln.getNumSeqs() + 1)
    FullPairwiseAlign(PairwiseSettings(g["matrix"], g["params"])).pairwiseAlign(aln, dm, *g["range"])
    assert np.array_equal(dm.getElements(), g["elements"])


@pytest.mark.gpu
def test_info_lines(capsys):
    from clustalw_gb300.pairwise import Alignment, DistMatrix, FullPairwiseAlign, PairwiseSettings

    g = load_golden("fixture_100_97")
    seqs = g["seqs"][:6]
    aln = Alignment(seqs)
    dm = DistMatrix(7)
    FullPairwiseAlign(PairwiseSettings(g["matrix"], g["params"], display_info=True)).pairwiseAlign(aln, dm, 0, 6, 0, 6)
    lines = [l for l in capsys.readouterr().out.splitlines() if l.startswith("Sequences (")]
    assert len(lines) == 15
    for line in lines:  # percent identity = (1 - d) * 100 truncated, from the same float arithmetic
        i, j = (int(x) for x in line.split("(")[1].split(")")[0].split(":"))
        score = int(line.rsplit(" ", 1)[1])
        d = dm.GetAt(i, j)
        assert abs((100.0 - 100.0 * d) - score) < 1.0 + 1e-4


INFO_LINE = r"Sequences \((\d+):(\d+)\) Aligned\. Score:  (-?\d+)"


@pytest.mark.parametrize("name,rng", [("fixture_100_97", None), ("edge_protein", None),
                                      ("fixture_100_97", (10, 30, 5, 60))])
def test_info_lines_match_the_reference(name, rng, tmp_path, capsys, oracle_mod):
    """The per-pair lines the mirror prints when display is on
    (FullPairwiseAlign.cpp:185-189, the "Score" known answers clustalw2 prints
    without -QUIET), built from the per-pair identity counts the GPU returns
    (here the oracle's, which the GPU tests equal), are the lines the
    unmodified reference prints (oracle/_ref/refharness with
    CWREF_DISPLAY_INFO=1), pair for pair. CPU only; needs the harness."""
    import os
    import re
    import subprocess

    from clustalw_gb300 import synth
    from clustalw_gb300.pairwise import Alignment, FullPairwiseAlign, PairwiseSettings
    from conftest import range_pairs

    if not os.path.exists(oracle_mod.REF_HARNESS):
        pytest.skip("reference harness not built")
    g = load_golden(name)
    n = len(g["seqs"])
    rng = rng or (0, n, 0, n)
    fa = tmp_path / "in.fa"
    fa.write_text(synth.to_fasta(g["seqs"]))
    out = subprocess.run([oracle_mod.REF_HARNESS, str(fa), str(tmp_path / "o.bin"), *map(str, rng)],
                         capture_output=True, text=True, check=True, env=dict(os.environ, CWREF_DISPLAY_INFO="1"))
    ref = oracle_mod.read_ref_output(str(tmp_path / "o.bin"))
    assert all(np.array_equal(a, b) for a, b in zip(ref["seqs"], g["seqs"]))  # the reader saw the same codes
    want = re.findall(INFO_LINE, out.stdout)
    pairs = range_pairs(n, *rng)
    stats = oracle_mod.align_pairs(g["seqs"], g["matrix"], g["params"], pairs)
    capsys.readouterr()
    FullPairwiseAlign(PairwiseSettings(g["matrix"], g["params"]))._print_info(Alignment(g["seqs"]), stats, *rng)
    got = re.findall(INFO_LINE, capsys.readouterr().out)
    assert len(want) > 0 and got == want


# the reference writes the newline before each line, so the last one runs into
# what follows: the score is matched as a %g number
QUICK_LINE = r"Sequences \((\d+):(\d+)\) (Aligned\. Score: \d+(?:\.\d+)?(?:e[-+]\d+)?|Not Aligned)"


@pytest.mark.parametrize("name,rng", [("fast_100_97", None), ("fast_edge_protein", None), ("fast_edge_dna", None),
                                      ("fast_100_97_block", None)])
def test_quick_info_lines_match_the_reference(name, rng, tmp_path, capsys, oracle_mod):
    """The quick path's per-pair lines (FastPairwiseAlign.cpp:110-120, "%lg"
    scores and "Not Aligned"), built by the mirror from per-pair best scores
    (the oracle's, which the GPU tests equal), are the lines the unmodified
    reference prints. CPU only; needs the harness."""
    import os
    import re
    import subprocess

    from clustalw_gb300 import synth
    from clustalw_gb300.native import FastParams
    from clustalw_gb300.pairwise import Alignment, FastPairwiseAlign
    from conftest import load_fast_golden, range_pairs

    if not os.path.exists(oracle_mod.REF_HARNESS):
        pytest.skip("reference harness not built")
    g = load_fast_golden(name)
    n = len(g["seqs"])
    rng = tuple(g["range"])
    fa = tmp_path / "in.fa"
    fa.write_text(synth.to_fasta(g["seqs"]))
    out = subprocess.run([oracle_mod.REF_HARNESS, "--fast", str(fa), str(tmp_path / "o.bin"), *map(str, rng)],
                         capture_output=True, text=True, check=True, env=dict(os.environ, CWREF_DISPLAY_INFO="1"))
    ref = oracle_mod.read_ref_output(str(tmp_path / "o.bin"))
    assert all(np.array_equal(a, b) for a, b in zip(ref["seqs"], g["seqs"]))
    want = re.findall(QUICK_LINE, out.stdout)
    stats = oracle_mod.fast_pairs(g["seqs"], g["fast_params"], range_pairs(n, *rng))
    capsys.readouterr()
    fp = FastParams.from_dict(g["fast_params"])
    FastPairwiseAlign(fp)._print_info(Alignment(g["seqs"]), fp, stats, *rng)
    got = re.findall(QUICK_LINE, capsys.readouterr().out)
    assert len(want) > 0 and got == want
