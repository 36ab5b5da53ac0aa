// See GpuFullPairwiseAlign.h. Reads the same inputs FullPairwiseAlign reads
// (FullPairwiseAlign.cpp:60-95: the SeqArray, userParameters, and the matrix
// and scale values of subMatrix->getPairwiseMatrix), hands them to the GPU
// library, and keeps the reference's messages and exit codes.
#include "GpuFullPairwiseAlign.h"

#include <cstdlib>
#include <iostream>
#include <vector>

#include "cwgpu.h"
#include "general/UserParameters.h"
#include "general/Utility.h"
#include "substitutionMatrix/SubMatrix.h"

namespace clustalw
{

// One context per device for the life of the process. The reference news a
// FullPairwiseAlign per alignment and deletes it through PairwiseAlignBase*
// (Clustal.cpp:151-162), whose destructor is not virtual, so this class must
// not own device resources; the cached context also keeps the device set-up
// between calls. Released at exit. Not thread-safe, like the reference class.
static const int kMaxDevices = 64;
static cwgpu_context* sharedContexts[kMaxDevices];
static bool cleanupRegistered = false;

static void releaseContexts()
{
    for (int d = 0; d < kMaxDevices; ++d)
    {
        if (sharedContexts[d])
        {
            cwgpu_destroy(sharedContexts[d]);
            sharedContexts[d] = 0;
        }
    }
}

GpuFullPairwiseAlign::GpuFullPairwiseAlign(int dev)
: device(dev),
  ctx(0)
{
}

GpuFullPairwiseAlign::~GpuFullPairwiseAlign()
{
}

static void gpuFailure(cwgpu_context* ctx, int status)
{
    std::cerr << "An exception has occured in the FullPairwiseAlign class.\n"
              << cwgpu_status_string(status) << ": " << cwgpu_last_error(ctx) << "\n";
    exit(1);
}

void GpuFullPairwiseAlign::pairwiseAlign(Alignment *alignPtr, DistMatrix *distMat, int iStart,
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
    const int numSeqs = alignPtr->getNumSeqs();
    if (numSeqs == 0)
    {
        return;
    }

    int matrix[NUMRES][NUMRES];
    PairScaleValues scaleValues;
    int matAvgScore = 0;
    int maxRes = subMatrix->getPairwiseMatrix(matrix, scaleValues, matAvgScore);
    if (maxRes == 0)
    {
        std::cout << "Could not get the substitution matrix\n";
        return;
    }

    cwgpu_params params;
    params.dna = userParameters->getDNAFlag() ? 1 : 0;
    params.pw_gap_open = userParameters->getPWGapOpen();
    params.pw_gap_extend = userParameters->getPWGapExtend();
    params.int_scale = scaleValues.intScale;
    params.gap_open_scale = scaleValues.gapOpenScale;
    params.gap_extend_scale = scaleValues.gapExtendScale;
    params.mat_avg = matAvgScore;
    params.gap_pos1 = userParameters->getGapPos1();
    params.gap_pos2 = userParameters->getGapPos2();

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

    int32_t flat[NUMRES * NUMRES];
    for (int a = 0; a < NUMRES; ++a)
    {
        for (int b = 0; b < NUMRES; ++b)
        {
            flat[a * NUMRES + b] = matrix[a][b];
        }
    }

    int status = CWGPU_OK;
    if (device < 0 || device >= kMaxDevices)
    {
        gpuFailure(0, CWGPU_ERR_ARG);
    }
    ctx = sharedContexts[device];
    if (!ctx)
    {
        if (!cleanupRegistered)
        {
            atexit(releaseContexts);
            cleanupRegistered = true;
        }
        status = cwgpu_create(device, &ctx);
        sharedContexts[device] = ctx;
        if (status != CWGPU_OK)
        {
            gpuFailure(ctx, status);
        }
    }
    if (status == CWGPU_OK) status = cwgpu_set_matrix(ctx, flat);
    if (status == CWGPU_OK) status = cwgpu_set_params(ctx, &params);
    if (status == CWGPU_OK)
        status = cwgpu_upload_seqs(ctx, numSeqs, codes.empty() ? 0 : &codes[0], &offsets[0], &lens[0]);
    if (status != CWGPU_OK)
    {
        gpuFailure(ctx, status);
    }

    const bool display = userParameters->getDisplayInfo();
    std::vector<cwgpu_pair_stats> stats;
    if (display)
    {
        stats.resize((size_t)cwgpu_range_pair_count(numSeqs, iStart, iEnd, jStart, jEnd) + 1);
    }
    status = cwgpu_pairwise_align(ctx, iStart, iEnd, jStart, jEnd, distMat->getElements(),
                                  distMat->getSize(), display ? &stats[0] : 0);
    if (status != CWGPU_OK)
    {
        gpuFailure(ctx, status);
    }

    if (display)
    {
        // utilityObject->info lines of FullPairwiseAlign.cpp:185-189, with the
        // same float arithmetic for the printed percent identity.
        const int gp1 = params.gap_pos1, gp2 = params.gap_pos2;
        std::vector<int> residues(numSeqs);
        for (int s = 0; s < numSeqs; ++s)
        {
            int c = 0;
            for (int i = 0; i < lens[s]; ++i)
            {
                if (codes[offsets[s] + i] != gp1 && codes[offsets[s] + i] != gp2) ++c;
            }
            residues[s] = c;
        }
        size_t q = 0;
        for (int si = utilityObject->MAX(0, iStart); si < numSeqs && si < iEnd; si++)
        {
            for (int sj = utilityObject->MAX(si + 1, jStart + 1); sj < numSeqs && sj < jEnd; sj++, q++)
            {
                if (lens[si] == 0 || lens[sj] == 0) continue;
                float mmScore = 100.0 * (float)stats[q].n_ident;
                if (residues[si] == 0 || residues[sj] == 0)
                    mmScore = 0;
                else
                    mmScore /= (float)utilityObject->MIN(residues[si], residues[sj]);
                utilityObject->info("Sequences (%d:%d) Aligned. Score:  %d", si + 1, sj + 1, (int)mmScore);
            }
        }
        distMat->printArray();
    }
}

}
