/*
 * cwgpu_nj.h - C ABI of the GB300 (sm_103a) guide-tree step: neighbour joining
 * over the distance matrix the pairwise stage writes.
 *
 * Replaces the pure virtual
 *   ClusterTreeAlgorithm::generateTree(PhyloTree*, DistMatrix*, SeqInfo*,
 *                                      ofstream* tree = 0)
 * (CPU/clustalw-2.0.11/src/tree/ClusterTreeAlgorithm.h:19-20) as NJTree
 * implements it (CPU/clustalw-2.0.11/src/tree/NJTree.cpp:161-748), which
 * UnRootedClusterTree::treeFromDistMatrix calls for the guide tree
 * (tree/UnRootedClusterTree.cpp:228-246, with ofstream* = 0).
 *
 * Layouts are the reference's own:
 *   elements     the packed DistMatrix (SymMatrix, general/SymMatrix.h:166-197)
 *                of dimension n+1: (n+1)(n+2)/2 doubles, entry (i, j) for
 *                1-based i >= j at ((i-1)*i)/2 + (j-1). NJTree joins in place
 *                and so does this call: on return the array holds the matrix
 *                the reference leaves behind.
 *   left_branch, right_branch   PhyloTree::leftBranch / rightBranch
 *                (general/clustalw.h:88-93), n+2 doubles each.
 *   tree_desc    PhyloTree::treeDesc, (n+1) x (n+1) int32, row-major; row nc
 *                marks the members of the cluster formed at cycle nc, row n-2
 *                the final trichotomy (1, 2, 3).
 *   joins        optional, 2*(n-3) int32: (mini, minj) of every cycle, what the
 *                reference prints in its verbose cycle lines
 *                (NJTree.cpp:413-470); NULL to skip.
 * Results are bit-identical to the reference (same double rounding, same
 * first-minimum tie rule). n == 2 returns without touching the outputs, as
 * the reference does (NJTree.cpp:218-229).
 *
 * Every call returns a cwgpu_status (cwgpu.h). A handle owns one device and its
 * scratch, grows it to the largest n seen, and is not thread-safe.
 */
#ifndef CWGPU_NJ_H
#define CWGPU_NJ_H

#include <stdint.h>

#include "cwgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define CWGPU_NJ_MAX_N 16384 /* largest matrix the device kernel accepts */

typedef struct cwgpu_nj cwgpu_nj;

int cwgpu_nj_create(int device, cwgpu_nj** out);
void cwgpu_nj_destroy(cwgpu_nj* nj);
const char* cwgpu_nj_last_error(const cwgpu_nj* nj);

/* NJTree::generateTree(phyTree, distMat, seqInfo{1, n, n}) on HOST buffers:
 * copies the matrix in, builds the tree on the device, copies the matrix,
 * branches and treeDesc back. tree_desc is overwritten in full (the reference
 * receives it zero-filled from treeFromDistMatrix). */
int cwgpu_nj_tree(cwgpu_nj* nj, int32_t n, double* elements, double* left_branch, double* right_branch,
                  int32_t* tree_desc, int32_t* joins);

/* The same on DEVICE buffers of this handle's device. d_elements_in is not
 * modified (the join runs on a copy); d_elements_out (may equal NULL) receives
 * the matrix after the joins. stream is a cudaStream_t (NULL: the handle's own
 * stream); the call is asynchronous on it except for the final status check,
 * which waits. */
int cwgpu_nj_tree_device(cwgpu_nj* nj, int32_t n, const double* d_elements_in, double* d_elements_out,
                         double* d_left_branch, double* d_right_branch, int32_t* d_tree_desc, int32_t* d_joins,
                         void* stream);

/* Work counters of the last call: pair criteria evaluated (the NJ search's
 * unit of work) and wall time of the device kernel in seconds. */
int cwgpu_nj_last_stats(const cwgpu_nj* nj, int64_t* pairs_evaluated, double* kernel_seconds);

/* Diagnostic: the device's replay of the reference's sequential double sum,
 * s0 + x[0] + ... + x[count-1] with every addition rounded to nearest-even in
 * order (the loops of NJTree.cpp:267-293, 314-321, 590-616). The tree uses the
 * same routine; this entry point lets tests feed it adversarial terms. */
int cwgpu_nj_seq_sum(cwgpu_nj* nj, const double* x, int64_t count, double s0, double* out);

/* Diagnostic: runs the tree kernel's wait between CTAs on a counter that
 * nothing raises, limited to timeout_ns (1 .. 4e9). *timed_out is 1 when the
 * wait ended at its limit with the timeout status, as every such wait must;
 * the handle stays usable. No GPU fault or hang is involved. */
int cwgpu_nj_wait_probe(cwgpu_nj* nj, int64_t timeout_ns, int32_t* timed_out);

#ifdef __cplusplus
}
#endif
#endif /* CWGPU_NJ_H */
