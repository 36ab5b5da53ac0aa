// Test stand-in for substitutionMatrix/SubMatrix.h (see general/clustalw.h
// here): getPairwiseMatrix hands back the matrix, scale values and average
// score the test driver stored (taken from a reference-generated fixture).
#ifndef DROPIN_SHIM_SUBMATRIX_H
#define DROPIN_SHIM_SUBMATRIX_H

#include "general/clustalw.h"

namespace clustalw
{

class SubMatrix
{
    public:
        SubMatrix() : matAvg(0), maxRes(NUMRES)
        {
            scale.intScale = 0;
            scale.gapOpenScale = scale.gapExtendScale = 0.0f;
            for (int a = 0; a < NUMRES; ++a)
                for (int b = 0; b < NUMRES; ++b) matrix[a][b] = 0;
        }
        int getPairwiseMatrix(int out[NUMRES][NUMRES], PairScaleValues& sv, int& avg)
        {
            for (int a = 0; a < NUMRES; ++a)
                for (int b = 0; b < NUMRES; ++b) out[a][b] = matrix[a][b];
            sv = scale;
            avg = matAvg;
            return maxRes;
        }

        int matrix[NUMRES][NUMRES];
        PairScaleValues scale;
        int matAvg, maxRes;
};

extern SubMatrix* subMatrix;

}
#endif
