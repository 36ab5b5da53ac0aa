// See GpuFastPairwiseAlign.h. Reads what FastPairwiseAlign reads (the
// SeqArray, userParameters' k-tuple settings after setDNAParams /
// setProtParams, Alignment::getMaxAlnLength) and hands it to the library.
#include "GpuFastPairwiseAlign.h"

#include <cstdlib>
#include <iostream>
#include <vector>

#include "cwgpu.h"
#include "general/UserParameters.h"
#include "general/Utility.h"

namespace clustalw
{

// One context per device for the life of the process (the reference deletes
// the object through PairwiseAlignBase*, whose destructor is not virtual,
// Clustal.cpp:162). Released at exit. Not thread-safe, like the reference.
static const int kMaxDevices = 64;
static cwgpu_context* fastContexts[kMaxDevices];
static bool fastCleanupRegistered = false;

static void releaseFastContexts()
{
    for (int d = 0; d < kMaxDevices; ++d)
    {
        if (fastContexts[d])
        {
            cwgpu_destroy(fastContexts[d]);
            fastContexts[d] = 0;
        }
    }
}

GpuFastPairwiseAlign::GpuFastPairwiseAlign(int dev)
: device(dev)
{
}

GpuFastPairwiseAlign::~GpuFastPairwiseAlign()
{
}

static void fastFailure(cwgpu_context* ctx, int status)
{
    std::cerr << "An exception has occured in the FastPairwiseAlign class.\n"
              << cwgpu_status_string(status) << ": " << (ctx ? cwgpu_last_error(ctx) : "") << "\n";
    exit(1);
}

void GpuFastPairwiseAlign::pairwiseAlign(Alignment *alignPtr, DistMatrix *distMat, int iStart,
                                         int iEnd, int jStart, int jEnd)
{
    if (distMat->getSize() != alignPtr->getNumSeqs() + 1)
    {
        std::cout << "The distance matrix is not the right size!\n"
                  << "Need to terminate program.\n";
        exit(1);
    }
    if ((iStart < 0) || (iEnd < iStart) || (jStart < 0) || (jEnd < jStart))
    {
        std::cout << "The range for pairwise Alignment is incorrect.\n"
                  << "Need to terminate program.\n";
        exit(1);
    }
    const bool dna = userParameters->getDNAFlag();
    if (dna)
    {
        userParameters->setDNAParams();
    }
    else
    {
        userParameters->setProtParams();
    }
    std::cout << "\n\n";
    const int numSeqs = alignPtr->getNumSeqs();
    if (numSeqs == 0)
    {
        return;
    }
    if (device < 0 || device >= kMaxDevices)
    {
        fastFailure(0, CWGPU_ERR_ARG);
    }
    cwgpu_context* ctx = fastContexts[device];
    int status = CWGPU_OK;
    if (!ctx)
    {
        if (!fastCleanupRegistered)
        {
            atexit(releaseFastContexts);
            fastCleanupRegistered = true;
        }
        status = cwgpu_create(device, &ctx);
        if (status != CWGPU_OK)
        {
            fastFailure(ctx, status);
        }
        fastContexts[device] = ctx;
    }

    // SeqArray rows 1..numSeqs, elements 1..len (element 0 is the dummy).
    const SeqArray* seqs = alignPtr->getSeqArray();
    std::vector<int8_t> codes;
    std::vector<int64_t> offsets(numSeqs);
    std::vector<int32_t> lens(numSeqs);
    for (int s = 0; s < numSeqs; ++s)
    {
        lens[s] = alignPtr->getSeqLength(s + 1);
        offsets[s] = (int64_t)codes.size();
        for (int i = 1; i <= lens[s]; ++i)
        {
            codes.push_back((int8_t)(*seqs)[s + 1][i]);
        }
    }
    status = cwgpu_upload_seqs(ctx, numSeqs, codes.empty() ? 0 : &codes[0], &offsets[0], &lens[0]);
    if (status != CWGPU_OK)
    {
        fastFailure(ctx, status);
    }

    cwgpu_fast_params p;
    p.dna = dna ? 1 : 0;
    p.ktup = userParameters->getKtup();
    p.window = userParameters->getWindow();
    p.window_gap = userParameters->getWindowGap();
    p.signif = userParameters->getSignif();
    p.percent = userParameters->getPercent() ? 1 : 0;
    p.max_aa = userParameters->getMaxAA();
    p.max_aln_length = alignPtr->getMaxAlnLength();

    const int64_t npairs = cwgpu_range_pair_count(numSeqs, iStart, iEnd, jStart, jEnd);
    std::vector<cwgpu_fast_stats> stats(npairs > 0 ? npairs : 1);
    status = cwgpu_fast_pairwise_align(ctx, &p, iStart, iEnd, jStart, jEnd, distMat->getElements(),
                                       distMat->getSize(), &stats[0]);
    if (status != CWGPU_OK)
    {
        fastFailure(ctx, status);
    }

    // The reference's messages (FastPairwiseAlign.cpp:107-118, 273-278), in
    // its loop order.
    int64_t q = 0;
    for (int si = iStart; si < iEnd && si < numSeqs; ++si)
    {
        for (int sj = (jStart + 1 > si + 1 ? jStart + 1 : si + 1); sj < jEnd && sj < numSeqs; ++sj, ++q)
        {
            if (stats[q].partial)
            {
                utilityObject->info("(Partial alignment)");
            }
            if (!userParameters->getDisplayInfo())
            {
                continue;
            }
            double calcScore = 0.0;
            if (stats[q].score)
            {
                calcScore = (double)stats[q].score;
                if (p.percent)
                {
                    const int l1 = lens[si], l2 = lens[sj];
                    calcScore = (calcScore / (double)(l1 < l2 ? l1 : l2)) * 100.0;
                }
            }
            if (calcScore > 0.1)
            {
                utilityObject->info("Sequences (%d:%d) Aligned. Score: %lg", si + 1, sj + 1, calcScore);
            }
            else
            {
                utilityObject->info("Sequences (%d:%d) Not Aligned", si + 1, sj + 1);
            }
        }
    }
}

}
