// GpuFullPairwiseAlign: drop-in replacement for clustalw::FullPairwiseAlign
// (CPU/clustalw-2.0.11/src/pairwise/FullPairwiseAlign.h:44-91) that runs the
// full-pairwise distance stage on a GB300 through the C ABI of cwgpu.h.
//
// It is compiled inside the ClustalW source tree (it includes the reference's
// own headers) and is constructed wherever the reference constructs
// FullPairwiseAlign, e.g. Clustal::align (Clustal.cpp:151-162).
#ifndef GPUFULLPAIRWISEALIGN_H
#define GPUFULLPAIRWISEALIGN_H

#include "pairwise/PairwiseAlignBase.h"

struct cwgpu_context;

namespace clustalw
{

class GpuFullPairwiseAlign : public PairwiseAlignBase
{
    public:
        explicit GpuFullPairwiseAlign(int device = 0);
        virtual ~GpuFullPairwiseAlign();
        // Same contract as FullPairwiseAlign::pairwiseAlign
        // (FullPairwiseAlign.cpp:34-211): writes distMat->SetAt(si+1, sj+1)
        // and SetAt(sj+1, si+1) for si in [max(0,iStart), min(N,iEnd)),
        // sj in [max(si+1,jStart+1), min(N,jEnd)); prints and exits(1) on a
        // wrong matrix size, a bad range or a device failure.
        virtual void pairwiseAlign(Alignment *alignPtr, DistMatrix *distMat, int iStart,
                                   int iEnd, int jStart, int jEnd);

    private:
        GpuFullPairwiseAlign(const GpuFullPairwiseAlign&);
        GpuFullPairwiseAlign& operator=(const GpuFullPairwiseAlign&);
        int device;
        cwgpu_context* ctx;  // the process-wide context of this device (see the .cpp)
};

}
#endif
