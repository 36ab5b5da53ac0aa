// Link check for the C++ drop-ins: defines the reference's five process
// globals (as CPU/clustalw-2.0.11/src/main.cpp:23-30 does), constructs
// GpuFullPairwiseAlign and GpuFastPairwiseAlign behind a PairwiseAlignBase
// pointer and GpuNJTree behind
// a ClusterTreeAlgorithm pointer, and exits without calling them (this binary
// is built and linked on a host without a GPU).
#include "pairwise/PairwiseAlignBase.h"
#include "general/DebugLog.h"
#include "general/Stats.h"
#include "general/UserParameters.h"
#include "general/Utility.h"
#include "substitutionMatrix/SubMatrix.h"
#include "GpuFullPairwiseAlign.h"
#include "GpuNJTree.h"
#include "GpuFastPairwiseAlign.h"

namespace clustalw {
UserParameters* userParameters;
Utility* utilityObject;
SubMatrix* subMatrix;
DebugLog* logObject;
Stats* statsObject;
}

int main() {
    clustalw::PairwiseAlignBase* p = new clustalw::GpuFullPairwiseAlign(0);
    delete p;
    p = new clustalw::GpuFastPairwiseAlign(0);
    delete p;
    // Deleted through the base pointer, as UnRootedClusterTree.cpp:248 does;
    // the drop-ins own no per-object device resources.
    clustalw::ClusterTreeAlgorithm* t = new clustalw::GpuNJTree(0);
    t->setVerbose(false);
    delete t;
    return 0;
}
