// Test stand-in for the reference header of the same path (general/clustalw.h
// of ClustalW 2.0.11). TEST INFRASTRUCTURE ONLY: it declares just the names
// the C++ drop-ins (cuda-clustalw_gb300/host/Gpu*.cpp) use, so that they
// compile and run against the GB300 library on a host without the reference
// tree (tests/test_dropin_shim.py). Written for these tests, not taken from
// the reference.
#ifndef DROPIN_SHIM_CLUSTALW_H
#define DROPIN_SHIM_CLUSTALW_H

#include <fstream>
#include <vector>

namespace clustalw
{

using std::ofstream;

const int NUMRES = 32;  // residue codes 0..31, as the pairwise matrix is indexed

// Rows 1..numSeqs of residue codes; element 0 of each row is unused.
typedef std::vector<std::vector<int> > SeqArray;

// Integer scaling of the pairwise matrix and gap penalties.
struct PairScaleValues
{
    int intScale;
    float gapOpenScale;
    float gapExtendScale;
};

// What a guide-tree algorithm fills: branch lengths by cycle and, per cycle,
// which sequences sit on each side.
struct PhyloTree
{
    std::vector<std::vector<int> > treeDesc;
    std::vector<double> leftBranch;
    std::vector<double> rightBranch;
};

struct SeqInfo
{
    int firstSeq;
    int lastSeq;
    int numSeqs;
};

}
#endif
