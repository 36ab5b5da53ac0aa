// Link check for the C++ drop-in: defines the reference's five process
// globals (as CPU/clustalw-2.0.11/src/main.cpp:23-30 does), constructs
// GpuFullPairwiseAlign behind a PairwiseAlignBase pointer, and exits without
// calling it (this binary is built and linked on a host without a GPU).
#include "pairwise/PairwiseAlignBase.h"
#include "general/DebugLog.h"
#include "general/Stats.h"
#include "general/UserParameters.h"
#include "general/Utility.h"
#include "substitutionMatrix/SubMatrix.h"
#include "GpuFullPairwiseAlign.h"

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
    return 0;
}
