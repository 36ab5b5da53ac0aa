// Test stand-in for pairwise/PairwiseAlignBase.h (see general/clustalw.h
// here): the interface the pairwise drop-ins implement.
#ifndef DROPIN_SHIM_PAIRWISEALIGNBASE_H
#define DROPIN_SHIM_PAIRWISEALIGNBASE_H

#include "alignment/Alignment.h"
#include "general/SymMatrix.h"

namespace clustalw
{

class PairwiseAlignBase
{
    public:
        virtual ~PairwiseAlignBase() {}
        virtual void pairwiseAlign(Alignment* alignPtr, DistMatrix* distMat, int iStart, int iEnd, int jStart,
                                   int jEnd) = 0;
};

}
#endif
