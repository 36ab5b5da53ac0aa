"""Guide tree: the reference's ClusterTreeAlgorithm plugin interface
(CPU/clustalw-2.0.11/src/tree/ClusterTreeAlgorithm.h:16-24) with its NJTree
implementation (tree/NJTree.cpp:161-748) running on the GPU through
include/cwgpu_nj.h.

NJTree.generateTree(phyTree, distMat, seqInfo) fills phyTree.leftBranch,
rightBranch and treeDesc and joins distMat in place, bit-identically to the
reference. There is no CPU path: without the CUDA library the call raises.
"""
import ctypes

import numpy as np

from . import native
from .native import CwgpuError


class PhyloTree:
    """general/clustalw.h:88-93."""

    def __init__(self):
        self.treeDesc = np.zeros((0, 0), dtype=np.int32)
        self.leftBranch = np.zeros(0, dtype=np.float64)
        self.rightBranch = np.zeros(0, dtype=np.float64)


class SeqInfo:
    """general/clustalw.h:94-99."""

    def __init__(self, firstSeq, lastSeq, numSeqs):
        self.firstSeq = firstSeq
        self.lastSeq = lastSeq
        self.numSeqs = numSeqs


class ClusterTreeAlgorithm:
    """ClusterTreeAlgorithm.h:16-24."""

    def generateTree(self, phyTree, distMat, seqInfo, tree=None):
        raise NotImplementedError

    def setVerbose(self, choice):
        raise NotImplementedError


class NJGpu:
    """Owner of a cwgpu_nj handle (device scratch grows to the largest n)."""

    def __init__(self, device=0):
        self._lib = native.load()
        h = ctypes.c_void_p()
        rc = self._lib.cwgpu_nj_create(int(device), ctypes.byref(h))
        if rc:
            raise CwgpuError(rc, "cwgpu_nj_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.cwgpu_nj_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _err(self, rc, what):
        msg = self._lib.cwgpu_nj_last_error(self._h)
        return CwgpuError(rc, f"{what}: {msg.decode() if msg else ''}")

    def tree(self, n, elements, want_joins=False):
        """Runs the join on host arrays. `elements` (float64, (n+1)(n+2)/2) is
        joined in place; returns (left, right, desc[(n+1),(n+1)], joins or None)."""
        assert elements.dtype == np.float64 and elements.flags.c_contiguous
        assert len(elements) >= (n + 1) * (n + 2) // 2
        left = np.zeros(n + 2, dtype=np.float64)
        right = np.zeros(n + 2, dtype=np.float64)
        desc = np.zeros((n + 1, n + 1), dtype=np.int32)
        joins = np.zeros((max(n - 3, 0), 2), dtype=np.int32) if want_joins else None
        rc = self._lib.cwgpu_nj_tree(self._h, int(n), elements.ctypes.data, left.ctypes.data, right.ctypes.data,
                                     desc.ctypes.data, None if joins is None else joins.ctypes.data)
        if rc:
            raise self._err(rc, "cwgpu_nj_tree")
        return left, right, desc, joins

    def tree_device(self, n, d_in, d_out, d_left, d_right, d_desc, d_joins=None, stream=None):
        """Device-pointer form (ints are raw device addresses)."""
        rc = self._lib.cwgpu_nj_tree_device(self._h, int(n), d_in, d_out, d_left, d_right, d_desc, d_joins, stream)
        if rc:
            raise self._err(rc, "cwgpu_nj_tree_device")

    def seq_sum(self, x, s0=0.0):
        """The device's replay of a sequentially rounded double sum."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = ctypes.c_double()
        rc = self._lib.cwgpu_nj_seq_sum(self._h, x.ctypes.data if len(x) else None, len(x), float(s0),
                                        ctypes.byref(out))
        if rc:
            raise self._err(rc, "cwgpu_nj_seq_sum")
        return out.value

    def wait_probe(self, timeout_ns):
        """The tree kernel's bounded wait on a counter nothing raises: True
        when it ended at its limit with the timeout status."""
        out = ctypes.c_int32()
        rc = self._lib.cwgpu_nj_wait_probe(self._h, int(timeout_ns), ctypes.byref(out))
        if rc:
            raise self._err(rc, "cwgpu_nj_wait_probe")
        return bool(out.value)

    def last_stats(self):
        p = ctypes.c_int64()
        s = ctypes.c_double()
        self._lib.cwgpu_nj_last_stats(self._h, ctypes.byref(p), ctypes.byref(s))
        return p.value, s.value


# The reference's verbose report (NJTree.cpp:209-236, 413-470, 694-740):
# C++ ostream with setprecision(5) (%g style) and setw(9) for branch lengths.
_REPORT_HEAD = ("\n\n\t\t\tNeighbor-joining Method\n"
                "\n Saitou, N. and Nei, M. (1987) The Neighbor-joining Method:"
                "\n A New Method for Reconstructing Phylogenetic Trees."
                "\n Mol. Biol. Evol., 4(4), 406-425\n\n\n This is an UNROOTED tree\n"
                "\n Numbers in parentheses are branch lengths\n\n")


def _br(v):
    return "%9s" % ("%.5g" % v)


def _side(node, index, branch):
    return ("Node:" if node else " SEQ:") + "%4d" % index + " (" + _br(branch) + ")"


def nj_report(n, joins, left, right):
    """The cycle report NJTree writes when verbose, rebuilt from the joins
    (mini, minj per cycle) and branch lengths of a tree of n > 2 sequences."""
    out = []
    joined = [False] * (n + 1)  # av[i] > 0 in the reference
    gone = [False] * (n + 1)
    for nc in range(1, n - 2):
        mini, minj = int(joins[nc - 1][0]), int(joins[nc - 1][1])
        out.append("\n Cycle" + "%4d" % nc + "     = " + _side(joined[mini], mini, left[nc]) + " joins "
                   + _side(joined[minj], minj, right[nc]) + "\n")
        joined[mini] = True
        gone[minj] = True
    out.append("\n Cycle" + "%4d" % (n - 2) + " (Last cycle, trichotomy):\n")
    rest = [i for i in range(1, n + 1) if not gone[i]]
    for k, i in enumerate(rest, start=1):
        out.append(("\n\t\t Node:" if joined[i] else "\n\t\t  SEQ:") + "%4d" % i + " (" + _br(left[n - 3 + k]) + ") "
                   + ("joins" if k < 3 else ""))
    out.append("\n")
    return "".join(out)


class NJTree(ClusterTreeAlgorithm):
    """NJTree (tree/NJTree.h) on the GPU. As UnRootedClusterTree::treeFromDistMatrix
    calls it (tree/UnRootedClusterTree.cpp:241-246), distMat holds seqInfo.numSeqs
    sequences at 1-based indices 1..numSeqs."""

    def __init__(self, device=0, gpu=None):
        self.verbose = False
        self._gpu = gpu
        self._device = device
        self.lastJoins = None

    def setVerbose(self, choice):
        self.verbose = bool(choice)

    def generateTree(self, phyTree, distMat, seqInfo, tree=None):
        """tree: a text stream for the verbose report (None: no report, as
        the reference resets verbose when given no stream)."""
        if tree is None:
            self.verbose = False
        n = seqInfo.lastSeq - seqInfo.firstSeq + 1
        if n < 2:
            raise ValueError("NJTree needs at least two sequences")
        if self.verbose:
            tree.write(_REPORT_HEAD)
        if n == 2:  # NJTree.cpp:218-229: returns before touching the tree
            if self.verbose:
                d = distMat.GetAt(seqInfo.firstSeq, seqInfo.firstSeq + 1)
                tree.write("Cycle   1     =  SEQ:   1 (" + _br(d) + ") joins  SEQ:   2 (" + _br(d) + ")")
            return
        if self._gpu is None:
            self._gpu = NJGpu(self._device)
        el = distMat.getElements()
        need = (n + 1) * (n + 2) // 2
        if len(el) < need:
            raise ValueError("distance matrix smaller than numSeqs")
        work = np.ascontiguousarray(el[:need], dtype=np.float64)
        left, right, desc, joins = self._gpu.tree(n, work, want_joins=True)
        el[:need] = work
        phyTree.leftBranch = left
        phyTree.rightBranch = right
        phyTree.treeDesc = desc
        self.lastJoins = joins
        if self.verbose:
            tree.write(nj_report(n, joins, left, right))
