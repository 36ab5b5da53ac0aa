// GpuFastPairwiseAlign: drop-in replacement for clustalw::FastPairwiseAlign
// (CPU/clustalw-2.0.11/src/pairwise/FastPairwiseAlign.h:15-50), the quick
// k-tuple distances, running on a GB300 through the C ABI of cwgpu.h.
//
// Constructed wherever the reference constructs FastPairwiseAlign, e.g.
// Clustal::align when userParameters->getQuickPairAlign() is set
// (Clustal.cpp:152-155). Same distances, messages and exit codes.
#ifndef GPUFASTPAIRWISEALIGN_H
#define GPUFASTPAIRWISEALIGN_H

#include "pairwise/PairwiseAlignBase.h"

struct cwgpu_context;

namespace clustalw
{

class GpuFastPairwiseAlign : public PairwiseAlignBase
{
    public:
        explicit GpuFastPairwiseAlign(int device = 0);
        virtual ~GpuFastPairwiseAlign();
        // Same contract as FastPairwiseAlign::pairwiseAlign
        // (FastPairwiseAlign.cpp:20-139): switches userParameters to the DNA
        // or protein k-tuple parameters, writes distMat->SetAt(i, j) for
        // i = iStart+1..iEnd, j = max(jStart+2, i+1)..jEnd, prints the same
        // info lines when display is on, and exits(1) on a wrong matrix size,
        // a bad range or a device failure.
        virtual void pairwiseAlign(Alignment *alignPtr, DistMatrix *distMat, int iStart,
                                   int iEnd, int jStart, int jEnd);

    private:
        GpuFastPairwiseAlign(const GpuFastPairwiseAlign&);
        GpuFastPairwiseAlign& operator=(const GpuFastPairwiseAlign&);
        int device;
};

}
#endif
