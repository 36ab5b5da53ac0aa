// Runs one C++ drop-in (cuda-clustalw_gb300/host/Gpu*.cpp) compiled against
// the stand-in headers of tests/dropin_shim, on the library it is linked with
// (lib/libcwgpu.so on a GPU host, or the oracle test double), for
// tests/test_dropin_shim.py. TEST INFRASTRUCTURE ONLY.
//
//   dropin_shim_run <input> <output> [<report>]
//
// input (whitespace-separated):
//   full <device> <iStart> <iEnd> <jStart> <jEnd> <display>
//        <dna> <int_scale> <mat_avg> <gap_pos1> <gap_pos2>
//        <pw_gap_open> <pw_gap_extend> <gap_open_scale> <gap_extend_scale>   (hex floats)
//        <32 x 32 matrix> <nseqs> then per sequence <len> <codes...>
//   fast <device> <iStart> <iEnd> <jStart> <jEnd> <display>
//        <dna> <ktup> <window> <window_gap> <signif> <percent> <max_aa> <max_aln_length>
//        <nseqs> then per sequence <len> <codes...>
//   nj   <device> <verbose> <n> <elements...>   ((n+1)(n+2)/2 hex floats)
// output: full/fast: the DistMatrix elements; nj: n + 2 left branches, n + 2
// right branches, (n+1) x (n+1) treeDesc, the joined DistMatrix elements; one
// value per line, doubles as hex floats. With <report>, nj writes the verbose
// cycle report there.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <vector>

#include "GpuFastPairwiseAlign.h"
#include "GpuFullPairwiseAlign.h"
#include "GpuNJTree.h"
#include "general/UserParameters.h"
#include "general/Utility.h"
#include "substitutionMatrix/SubMatrix.h"

namespace clustalw
{
UserParameters* userParameters = 0;
Utility* utilityObject = 0;
SubMatrix* subMatrix = 0;
}

using namespace clustalw;

static FILE* in = 0;

static int readInt()
{
    int v = 0;
    if (std::fscanf(in, "%d", &v) != 1)
    {
        std::fprintf(stderr, "bad input\n");
        std::exit(2);
    }
    return v;
}

static double readDouble()
{
    char buf[64];
    if (std::fscanf(in, "%63s", buf) != 1)
    {
        std::fprintf(stderr, "bad input\n");
        std::exit(2);
    }
    return std::strtod(buf, 0);
}

static void readSeqs(Alignment& aln)
{
    const int n = readInt();
    for (int s = 0; s < n; ++s)
    {
        const int len = readInt();
        std::vector<int> codes(len);
        for (int i = 0; i < len; ++i) codes[i] = readInt();
        aln.addSequence(codes);
    }
}

int main(int argc, char** argv)
{
    if (argc < 3) return 2;
    in = std::fopen(argv[1], "r");
    if (!in) return 2;
    FILE* out = std::fopen(argv[2], "w");
    if (!out) return 2;
    UserParameters params;
    Utility utility;
    SubMatrix matrix;
    userParameters = &params;
    utilityObject = &utility;
    subMatrix = &matrix;

    char mode[16];
    if (std::fscanf(in, "%15s", mode) != 1) return 2;
    const int device = readInt();
    if (!std::strcmp(mode, "full") || !std::strcmp(mode, "fast"))
    {
        const int i0 = readInt(), i1 = readInt(), j0 = readInt(), j1 = readInt();
        params.displayInfo = readInt() != 0;
        Alignment aln;
        PairwiseAlignBase* align = 0;
        if (!std::strcmp(mode, "full"))
        {
            params.dnaFlag = readInt() != 0;
            matrix.scale.intScale = readInt();
            matrix.matAvg = readInt();
            params.gapPos1 = readInt();
            params.gapPos2 = readInt();
            params.pwGapOpen = (float)readDouble();
            params.pwGapExtend = (float)readDouble();
            matrix.scale.gapOpenScale = (float)readDouble();
            matrix.scale.gapExtendScale = (float)readDouble();
            for (int a = 0; a < NUMRES; ++a)
                for (int b = 0; b < NUMRES; ++b) matrix.matrix[a][b] = readInt();
            align = new GpuFullPairwiseAlign(device);
        }
        else
        {
            params.dnaFlag = readInt() != 0;
            QuickParams q;
            q.ktup = readInt();
            q.window = readInt();
            q.windowGap = readInt();
            q.signif = readInt();
            params.percent = readInt() != 0;
            params.maxAA = readInt();
            aln.maxAlnLength = readInt();
            params.dnaQuick = q;
            params.protQuick = q;
            align = new GpuFastPairwiseAlign(device);
        }
        readSeqs(aln);
        DistMatrix dist(aln.getNumSeqs() + 1);
        align->pairwiseAlign(&aln, &dist, i0, i1, j0, j1);
        delete align;
        const double* el = dist.getElements();
        for (size_t k = 0; k < dist.numElements(); ++k) std::fprintf(out, "%a\n", el[k]);
    }
    else if (!std::strcmp(mode, "nj"))
    {
        const bool verbose = readInt() != 0;
        const int n = readInt();
        DistMatrix dist(n + 1);
        double* el = dist.getElements();
        for (size_t k = 0; k < dist.numElements(); ++k) el[k] = readDouble();
        PhyloTree tree;
        tree.treeDesc.assign(n + 1, std::vector<int>(n + 1, 0));
        SeqInfo info;
        info.firstSeq = 1;
        info.lastSeq = n;
        info.numSeqs = n;
        std::ofstream report;
        if (verbose && argc > 3) report.open(argv[3]);
        GpuNJTree nj(device);
        nj.setVerbose(verbose);
        nj.generateTree(&tree, &dist, &info, verbose ? &report : 0);
        tree.leftBranch.resize(n + 2, 0.0);
        tree.rightBranch.resize(n + 2, 0.0);
        for (int i = 0; i < n + 2; ++i) std::fprintf(out, "%a\n", tree.leftBranch[i]);
        for (int i = 0; i < n + 2; ++i) std::fprintf(out, "%a\n", tree.rightBranch[i]);
        for (int a = 0; a <= n; ++a)
            for (int b = 0; b <= n; ++b) std::fprintf(out, "%d\n", tree.treeDesc[a][b]);
        for (size_t k = 0; k < dist.numElements(); ++k) std::fprintf(out, "%a\n", el[k]);
    }
    else
    {
        return 2;
    }
    std::fclose(out);
    std::fclose(in);
    return 0;
}
