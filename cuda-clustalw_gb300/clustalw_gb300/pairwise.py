"""Host-side mirror of ClustalW 2.0.11's pairwise plugin interface over the
GB300 library.

The reference calls the distance stage through
``PairwiseAlignBase::pairwiseAlign(Alignment*, DistMatrix*, iStart, iEnd,
jStart, jEnd)`` (CPU/clustalw-2.0.11/src/pairwise/PairwiseAlignBase.h:19-20),
implemented by ``FullPairwiseAlign`` (pairwise/FullPairwiseAlign.cpp:34-211).
This module keeps those names, argument meanings and error behaviour:

* ``Alignment`` - the parts of clustalw::Alignment the stage reads: 1-based
  encoded sequences with a dummy element 0 (alignment/Alignment.h:96-117).
* ``SymMatrix`` (alias ``DistMatrix``) - the packed lower-triangular double
  store with the reference's index rule (general/SymMatrix.h:28-297).
* ``FullPairwiseAlign.pairwiseAlign`` - fills ``distMat`` exactly where and
  with what the reference writes; a wrong matrix size or a bad range prints the
  reference's message and exits with status 1 (FullPairwiseAlign.cpp:47-58).

All alignment work runs in the CUDA library; there is no CPU path here.
"""
import sys

import numpy as np

from . import native

GAP_POS1 = 30  # UserParameters.cpp defaults (gapPos1 = NUMRES - 2)
GAP_POS2 = 31  # gapPos2 = NUMRES - 1
AMINO_ACID_CODES = "ABCDEFGHIKLMNOPQRSTUVWXYZ-"  # UserParameters.cpp:132


def encode(text):
    """Residue letters -> codes like Sequence::encodeSequence
    (alignment/Sequence.cpp:63-83): '-' -> gapPos2, else the index in
    AMINO_ACID_CODES. Letters outside the alphabet raise ValueError (the
    reference's file parsers drop them before encoding)."""
    out = np.empty(len(text), dtype=np.int8)
    for i, ch in enumerate(text.upper()):
        if ch == "-":
            out[i] = GAP_POS2
        else:
            k = AMINO_ACID_CODES.find(ch)
            if k < 0:
                raise ValueError(f"residue {ch!r} not in {AMINO_ACID_CODES}")
            out[i] = k
    return out


def decode(codes):
    return "".join("-" if c in (GAP_POS1, GAP_POS2) else AMINO_ACID_CODES[c] for c in codes)


class Alignment:
    """Encoded sequences, 1-based like clustalw::Alignment's SeqArray."""

    def __init__(self, seqs=()):
        self._seqs = [np.ascontiguousarray(np.asarray(s, dtype=np.int8)) for s in seqs]

    def addSequence(self, codes):
        self._seqs.append(np.ascontiguousarray(np.asarray(codes, dtype=np.int8)))

    def getNumSeqs(self):
        return len(self._seqs)

    def getSeqLength(self, index):
        """Length of sequence `index` (1-based), Alignment.h:117."""
        return len(self._seqs[index - 1])

    def getSequence(self, index):
        """Codes of sequence `index` (1-based) with the dummy element 0."""
        return np.concatenate([[0], self._seqs[index - 1]]).astype(np.int32)

    def getMaxAlnLength(self):
        """2 * longest length (Alignment.cpp:747-780)."""
        longest = max((len(s) for s in self._seqs), default=0)
        return 2 * longest if self._seqs else 0

    def sequences(self):
        """0-based code arrays (no dummy element)."""
        return list(self._seqs)


class SymMatrix:
    """Packed lower-triangular double matrix (general/SymMatrix.h)."""

    def __init__(self, size=0):
        self.ResizeRect(size) if size > 0 else self._empty()

    def _empty(self):
        self.numSeqs = 0
        self.elements = np.zeros(1, dtype=np.float64)

    def ResizeRect(self, size, val=0.0):
        self.numSeqs = size - 1
        n = ((self.numSeqs + 1) * (self.numSeqs + 2)) >> 1
        self.elements = np.full(max(n, 1), val, dtype=np.float64)

    def getSize(self):
        return self.numSeqs + 1

    def getIndex(self, i, j):
        """SymMatrix::getIndex (:166-197): row or column 0 maps to slot 0."""
        if i == 0 or j == 0:
            return 0
        a, b = i - 1, j - 1
        if a == b:
            if a >= self.numSeqs or a < 0:
                raise IndexError("index out of range")
            return (a * (a + 3)) >> 1
        if a < b:
            a, b = b, a
        if a >= self.numSeqs or b < 0:
            raise IndexError("index out of range")
        return ((a * (a + 1)) >> 1) + b

    def SetAt(self, i, j, value):
        self.elements[self.getIndex(i, j)] = value

    def GetAt(self, i, j):
        return float(self.elements[self.getIndex(i, j)])

    def getElements(self):
        return self.elements


DistMatrix = SymMatrix


class PairwiseAlignBase:
    """PairwiseAlignBase.h:15-27."""

    def pairwiseAlign(self, alignPtr, distMat, iStart, iEnd, jStart, jEnd):
        raise NotImplementedError


class PairwiseSettings:
    """What FullPairwiseAlign reads from the userParameters and subMatrix
    singletons: the 32x32 pairwise matrix, PairScaleValues, matAvg, the DNA
    flag, the pairwise gap penalties and gapPos1/gapPos2."""

    def __init__(self, matrix, params, display_info=False):
        self.matrix = np.ascontiguousarray(np.asarray(matrix, dtype=np.int32).reshape(32, 32))
        self.params = dict(params)
        self.display_info = display_info


class FullPairwiseAlign(PairwiseAlignBase):
    """GB300 drop-in for clustalw::FullPairwiseAlign."""

    def __init__(self, settings, device=0, context=None):
        self.settings = settings
        self._ctx = context
        self._device = device
        self.last_stats = None

    def _context(self):
        if self._ctx is None:
            self._ctx = native.Context(self._device)
        return self._ctx

    def pairwiseAlign(self, alignPtr, distMat, iStart, iEnd, jStart, jEnd):
        numSeqs = alignPtr.getNumSeqs()
        if distMat.getSize() != numSeqs + 1:
            sys.stdout.write("The distance matrix is not the right size!\nNeed to terminate program.\n")
            raise SystemExit(1)
        if iStart < 0 or iEnd < iStart or jStart < 0 or jEnd < jStart:
            sys.stdout.write("The range for pairwise Alignment is incorrect.\nNeed to terminate program.\n")
            raise SystemExit(1)
        if numSeqs == 0:
            return
        ctx = self._context()
        ctx.set_matrix(self.settings.matrix)
        ctx.set_params(self.settings.params)
        ctx.upload_seqs(alignPtr.sequences())
        stats = ctx.pairwise_align(
            iStart, iEnd, jStart, jEnd, distMat.getElements(), distMat.getSize(), stats=True
        )
        self.last_stats = stats
        if self.settings.display_info:
            self._print_info(alignPtr, stats, iStart, iEnd, jStart, jEnd)

    def _print_info(self, aln, stats, iStart, iEnd, jStart, jEnd):
        """utilityObject->info lines of FullPairwiseAlign.cpp:185-189."""
        p = self.settings.params
        n = aln.getNumSeqs()
        seqs = aln.sequences()
        res = [int(np.count_nonzero((s != p["gap_pos1"]) & (s != p["gap_pos2"]))) for s in seqs]
        q = 0
        for si in range(max(0, iStart), min(n, iEnd)):
            for sj in range(max(si + 1, jStart + 1), min(n, jEnd)):
                if len(seqs[si]) == 0 or len(seqs[sj]) == 0:
                    q += 1
                    continue
                if res[si] == 0 or res[sj] == 0:
                    mm = np.float32(0.0)
                else:
                    mm = np.float32(100 * int(stats["n_ident"][q])) / np.float32(min(res[si], res[sj]))
                print(f"Sequences ({si + 1}:{sj + 1}) Aligned. Score:  {int(mm)}")
                q += 1


class FastPairwiseAlign(PairwiseAlignBase):
    """GB300 drop-in for clustalw::FastPairwiseAlign (quick k-tuple distances,
    pairwise/FastPairwiseAlign.cpp:20-139). `fast_params` are the userParameters
    values it reads (native.FastParams or a dict of its fields); by default the
    reference's protein or DNA defaults for the sequences' type."""

    def __init__(self, fast_params=None, dna=False, display_info=False, device=0, context=None):
        self.fast_params = fast_params
        self.dna = dna
        self.display_info = display_info
        self._ctx = context
        self._device = device
        self.last_stats = None

    def _context(self):
        if self._ctx is None:
            self._ctx = native.Context(self._device)
        return self._ctx

    def pairwiseAlign(self, alignPtr, distMat, iStart, iEnd, jStart, jEnd):
        numSeqs = alignPtr.getNumSeqs()
        if distMat.getSize() != numSeqs + 1:
            sys.stdout.write("The distance matrix is not the right size!\nNeed to terminate program.\n")
            raise SystemExit(1)
        if iStart < 0 or iEnd < iStart or jStart < 0 or jEnd < jStart:
            sys.stdout.write("The range for pairwise Alignment is incorrect.\nNeed to terminate program.\n")
            raise SystemExit(1)
        fp = self.fast_params
        if fp is None:
            fp = native.FastParams.defaults(self.dna, alignPtr.getMaxAlnLength())
        ctx = self._context()
        ctx.upload_seqs(alignPtr.sequences())
        stats = ctx.fast_pairwise_align(fp, iStart, iEnd, jStart, jEnd, distMat.getElements(), distMat.getSize(),
                                        stats=True)
        self.last_stats = stats
        if self.display_info:
            self._print_info(alignPtr, fp, stats, iStart, iEnd, jStart, jEnd)

    def _print_info(self, aln, fp, stats, iStart, iEnd, jStart, jEnd):
        """utilityObject->info lines of FastPairwiseAlign.cpp:107-118."""
        fp = fp if isinstance(fp, native.FastParams) else native.FastParams.from_dict(fp)
        n = aln.getNumSeqs()
        q = 0
        for si in range(max(0, iStart), min(n, iEnd)):
            for sj in range(max(si + 1, jStart + 1), min(n, jEnd)):
                score = int(stats["score"][q])
                calc = float(score)
                if score and fp.percent:
                    calc = (calc / float(min(aln.getSeqLength(si + 1), aln.getSeqLength(sj + 1)))) * 100.0
                if calc > 0.1:
                    print(f"Sequences ({si + 1}:{sj + 1}) Aligned. Score: {calc:g}")
                else:
                    print(f"Sequences ({si + 1}:{sj + 1}) Not Aligned")
                q += 1
