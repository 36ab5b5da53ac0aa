// See GpuNJTree.h. The joins run on the GPU; this file keeps the reference's
// interface: it reads and writes the same PhyloTree and DistMatrix fields and
// prints the same verbose report, rebuilt from the joins the GPU returns
// (which node joined which in every cycle) and the branch lengths.
#include "GpuNJTree.h"

#include <cstdlib>
#include <iomanip>
#include <iostream>
#include <vector>

#include "cwgpu_nj.h"

namespace clustalw
{

// One join handle per device for the life of the process: the reference
// deletes its tree algorithm through ClusterTreeAlgorithm*
// (UnRootedClusterTree.cpp:248), whose destructor is not virtual, so this class
// must not own device resources. Released at exit. Not thread-safe, like the
// reference class.
static const int kMaxDevices = 64;
static cwgpu_nj* sharedHandles[kMaxDevices];
static bool cleanupRegistered = false;

static void releaseHandles()
{
    for (int d = 0; d < kMaxDevices; ++d)
    {
        if (sharedHandles[d])
        {
            cwgpu_nj_destroy(sharedHandles[d]);
            sharedHandles[d] = 0;
        }
    }
}

GpuNJTree::GpuNJTree(int dev)
: device(dev),
  verbose(false),
  nj(0)
{
}

GpuNJTree::~GpuNJTree()
{
}

static void njFailure(cwgpu_nj* nj, int status)
{
    std::cout << "ERROR: Error has occured in treeFromDistMatrix. "
              << "Need to terminate program.\n"
              << cwgpu_status_string(status) << ": " << (nj ? cwgpu_nj_last_error(nj) : "") << "\n";
    exit(1);
}

// " SEQ:   3 (  0.12345) " / "Node:   3 (  0.12345)": one side of a join in
// the reference's report (NJTree.cpp:429-453).
static void side(ofstream* tree, bool node, int index, double branch)
{
    (*tree) << (node ? "Node:" : " SEQ:") << std::setw(4) << index << " (" << std::setw(9)
            << std::setprecision(5) << branch << ")";
}

void GpuNJTree::generateTree(PhyloTree* phyTree, DistMatrix* distMat, SeqInfo* seqInfo, ofstream* tree)
{
    if (tree == NULL)
    {
        verbose = false;
    }
    const int firstSeq = seqInfo->firstSeq;
    const int lastSeq = seqInfo->lastSeq;
    const int numSeqs = seqInfo->numSeqs;
    const int n = lastSeq - firstSeq + 1;

    if (verbose)
    {
        (*tree) << "\n\n\t\t\tNeighbor-joining Method\n"
                << "\n Saitou, N. and Nei, M. (1987)" << " The Neighbor-joining Method:"
                << "\n A New Method for Reconstructing Phylogenetic Trees."
                << "\n Mol. Biol. Evol., 4(4), 406-425\n" << "\n\n This is an UNROOTED tree\n"
                << "\n Numbers in parentheses are branch lengths\n\n";
    }
    if (n == 2)
    {
        if (verbose)
        {
            (*tree) << "Cycle   1     =  SEQ:   1 (" << std::setw(9) << std::setprecision(5)
                    << (*distMat)(firstSeq, firstSeq + 1) << ") joins  SEQ:   2 (" << std::setw(9)
                    << std::setprecision(5) << (*distMat)(firstSeq, firstSeq + 1) << ")";
        }
        return;
    }
    if (n < 2 || n > CWGPU_NJ_MAX_N)
    {
        njFailure(nj, CWGPU_ERR_ARG);
    }
    if (device < 0 || device >= kMaxDevices)
    {
        njFailure(0, CWGPU_ERR_ARG);
    }
    nj = sharedHandles[device];
    if (!nj)
    {
        if (!cleanupRegistered)
        {
            atexit(releaseHandles);
            cleanupRegistered = true;
        }
        int rc = cwgpu_nj_create(device, &nj);
        if (rc != CWGPU_OK)
        {
            njFailure(nj, rc);
        }
        sharedHandles[device] = nj;
    }

    std::vector<double> left(n + 2, 0.0), right(n + 2, 0.0);
    std::vector<int32_t> desc((size_t)(n + 1) * (n + 1), 0);
    std::vector<int32_t> joins(2 * (n - 3) + 2, 0);
    int rc = cwgpu_nj_tree(nj, n, distMat->getElements(), &left[0], &right[0], &desc[0], &joins[0]);
    if (rc != CWGPU_OK)
    {
        njFailure(nj, rc);
    }

    phyTree->leftBranch.resize(numSeqs + 2, 0.0);
    phyTree->rightBranch.resize(numSeqs + 2, 0.0);
    std::vector<bool> joined(n + 1, false);  // av[i] > 0 in the reference: i already stands for a node
    for (int nc = 1; nc <= n - 3; ++nc)
    {
        const int mini = joins[2 * (nc - 1)], minj = joins[2 * (nc - 1) + 1];
        if (verbose)
        {
            (*tree) << "\n Cycle" << std::setw(4) << nc << "     = ";
            side(tree, joined[mini], mini, left[nc]);
            (*tree) << " joins ";
            side(tree, joined[minj], minj, right[nc]);
            (*tree) << "\n";
        }
        joined[mini] = true;
        joined[minj] = false;
        phyTree->leftBranch[nc] = left[nc];
        phyTree->rightBranch[nc] = right[nc];
    }
    for (int nc = 1; nc <= n - 2; ++nc)
    {
        for (int i = 1; i <= n; ++i)
        {
            phyTree->treeDesc[nc][i] = desc[(size_t)nc * (n + 1) + i];
        }
    }
    for (int i = n - 2; i <= n; ++i)
    {
        phyTree->leftBranch[i] = left[i];
    }
    if (verbose)
    {
        // The three nodes left, in ascending order, are those never joined
        // away as minj (NJTree.cpp:646-737).
        std::vector<bool> gone(n + 1, false);
        for (int nc = 1; nc <= n - 3; ++nc)
        {
            gone[joins[2 * (nc - 1) + 1]] = true;
        }
        (*tree) << "\n Cycle" << std::setw(4) << n - 2 << " (Last cycle, trichotomy):\n";
        int k = 1;
        for (int i = 1; i <= n; ++i)
        {
            if (gone[i])
            {
                continue;
            }
            (*tree) << (joined[i] ? "\n\t\t Node:" : "\n\t\t  SEQ:") << std::setw(4) << i << " (" << std::setw(9)
                    << std::setprecision(5) << left[n - 3 + k] << ") ";
            if (k < 3)
            {
                (*tree) << "joins";
            }
            ++k;
        }
        (*tree) << "\n";
    }
}

}
