// Test stand-in for alignment/Alignment.h (see general/clustalw.h here): the
// sequences as a 1-based SeqArray, filled by the test driver.
#ifndef DROPIN_SHIM_ALIGNMENT_H
#define DROPIN_SHIM_ALIGNMENT_H

#include "general/clustalw.h"

namespace clustalw
{

class Alignment
{
    public:
        Alignment() : seqArray(1), maxAlnLength(0) {}
        void addSequence(const std::vector<int>& codes)
        {
            std::vector<int> row(1, 0);
            row.insert(row.end(), codes.begin(), codes.end());
            seqArray.push_back(row);
        }
        int getNumSeqs() const { return (int)seqArray.size() - 1; }
        const SeqArray* getSeqArray() const { return &seqArray; }
        int getSeqLength(int seq) const { return (int)seqArray[seq].size() - 1; }
        int getMaxAlnLength() const { return maxAlnLength; }

        SeqArray seqArray;
        int maxAlnLength;
};

}
#endif
