// GpuNJTree: drop-in replacement for clustalw::NJTree
// (CPU/clustalw-2.0.11/src/tree/NJTree.h:15-27), the ClusterTreeAlgorithm
// (tree/ClusterTreeAlgorithm.h:16-24) that builds the neighbour-joining guide
// tree, running the joins on a GB300 through the C ABI of cwgpu_nj.h.
//
// It is compiled inside the ClustalW source tree and constructed wherever the
// reference constructs NJTree, e.g. UnRootedClusterTree::treeFromDistMatrix
// (tree/UnRootedClusterTree.cpp:223). Results (branch lengths, treeDesc, the
// joined DistMatrix and the verbose cycle report) are identical.
#ifndef GPUNJTREE_H
#define GPUNJTREE_H

#include "tree/ClusterTreeAlgorithm.h"

struct cwgpu_nj;

namespace clustalw
{

class GpuNJTree : public ClusterTreeAlgorithm
{
    public:
        explicit GpuNJTree(int device = 0);
        virtual ~GpuNJTree();
        // Same contract as NJTree::generateTree (NJTree.cpp:161-748): joins
        // distMat(1..n, 1..n) in place, n = seqInfo->lastSeq -
        // seqInfo->firstSeq + 1, fills phyTree->leftBranch / rightBranch
        // (resized to numSeqs + 2) and rows 1..n-2 of phyTree->treeDesc (sized
        // by the caller), and writes the cycle report to *tree when verbose.
        virtual void generateTree(PhyloTree* phyTree, DistMatrix* distMat, SeqInfo* seqInfo,
                                  ofstream* tree = 0);
        virtual void setVerbose(bool choice) { verbose = choice; }

    private:
        GpuNJTree(const GpuNJTree&);
        GpuNJTree& operator=(const GpuNJTree&);
        int device;
        bool verbose;
        cwgpu_nj* nj;  // the process-wide handle of this device (see GpuNJTree.cpp)
};

}
#endif
