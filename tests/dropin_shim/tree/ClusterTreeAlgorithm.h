// Test stand-in for tree/ClusterTreeAlgorithm.h (see general/clustalw.h
// here): the interface the guide-tree drop-in implements.
#ifndef DROPIN_SHIM_CLUSTERTREEALGORITHM_H
#define DROPIN_SHIM_CLUSTERTREEALGORITHM_H

#include "general/SymMatrix.h"
#include "general/clustalw.h"

namespace clustalw
{

class ClusterTreeAlgorithm
{
    public:
        virtual ~ClusterTreeAlgorithm() {}
        virtual void generateTree(PhyloTree* phyTree, DistMatrix* distMat, SeqInfo* seqInfo,
                                  ofstream* tree = 0) = 0;
        virtual void setVerbose(bool choice) = 0;
};

}
#endif
