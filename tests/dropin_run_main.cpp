// Runs one pairwise or guide-tree plugin the way clustalw2 runs it, either the
// reference class (IMPL "ref": FullPairwiseAlign, FastPairwiseAlign, NJTree)
// or the drop-in (IMPL "dropin": GpuFullPairwiseAlign, GpuFastPairwiseAlign,
// GpuNJTree), and writes what it leaves behind. tests/test_dropin_run.py links
// the drop-ins against tests/dropin_stub_cwgpu.c (the oracle standing in for
// the GPU library) and compares the two runs byte for byte.
//
// Usage: dropin_run IMPL KIND IN.fa OUT.bin [iStart iEnd jStart jEnd]
//   KIND full | fast: the DistMatrix elements (display info on, so the
//   per-pair lines and the matrix print go to standard output);
//   KIND nj: the full DistMatrix from the reference FullPairwiseAlign, then the
//   tree plugin with its verbose report written to OUT.bin.report; OUT.bin
//   holds leftBranch, rightBranch, treeDesc and the joined matrix.
// The CWREF_* variables of oracle/ref_overrides.h set the pairwise matrix, gap
// penalties and quick-distance settings for both implementations alike.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

#include "alignment/Alignment.h"
#include "fileInput/FileReader.h"
#include "general/DebugLog.h"
#include "general/Stats.h"
#include "general/UserParameters.h"
#include "general/Utility.h"
#include "general/clustalw.h"
#include "pairwise/FastPairwiseAlign.h"
#include "pairwise/FullPairwiseAlign.h"
#include "substitutionMatrix/SubMatrix.h"
#include "tree/NJTree.h"
#include "GpuFastPairwiseAlign.h"
#include "GpuFullPairwiseAlign.h"
#include "GpuNJTree.h"

namespace clustalw {
UserParameters* userParameters;
Utility* utilityObject;
SubMatrix* subMatrix;
DebugLog* logObject;
Stats* statsObject;
}  // namespace clustalw

using namespace clustalw;

#include "ref_overrides.h"  // CWREF_* parameter settings from the environment

static void put(FILE* f, const void* p, size_t n) {
    if (n && fwrite(p, 1, n, f) != n) exit(2);
}

int main(int argc, char** argv) {
    if (argc != 5 && argc != 9) {
        fprintf(stderr, "usage: %s ref|dropin full|fast|nj IN.fa OUT.bin [iStart iEnd jStart jEnd]\n", argv[0]);
        return 2;
    }
    const std::string impl(argv[1]), kind(argv[2]);
    const bool dropin = impl == "dropin";
    userParameters = new UserParameters(false);
    utilityObject = new Utility();
    subMatrix = new SubMatrix();
    statsObject = new Stats();
    userParameters->setSeqName(std::string(argv[3]));
    Alignment aln;
    FileReader reader;
    if (reader.readSeqs(&aln, 1) != OK) return 3;
    apply_overrides(userParameters->getDNAFlag());
    apply_quick_overrides(userParameters->getDNAFlag());
    if (userParameters->getDNAFlag())
        userParameters->setDNAParams();
    else
        userParameters->setProtParams();
    const int n = aln.getNumSeqs();
    int range[4] = {0, n, 0, n};
    if (argc == 9)
        for (int k = 0; k < 4; ++k) range[k] = atoi(argv[5 + k]);
    SymMatrix dist;
    dist.ResizeRect(n + 1);
    FILE* f = fopen(argv[4], "wb");
    if (!f) return 4;
    if (kind == "full" || kind == "fast") {
        userParameters->setDisplayInfo(true);
        PairwiseAlignBase* p;
        if (kind == "full")
            p = dropin ? (PairwiseAlignBase*)new GpuFullPairwiseAlign(0) : (PairwiseAlignBase*)new FullPairwiseAlign();
        else
            p = dropin ? (PairwiseAlignBase*)new GpuFastPairwiseAlign(0) : (PairwiseAlignBase*)new FastPairwiseAlign();
        p->pairwiseAlign(&aln, &dist, range[0], range[1], range[2], range[3]);
        delete p;
        fflush(stdout);
        put(f, dist.getElements(), sizeof(double) * (size_t)(n + 1) * (n + 2) / 2);
    } else {
        userParameters->setDisplayInfo(false);
        FullPairwiseAlign fpa;
        fpa.pairwiseAlign(&aln, &dist, 0, n, 0, n);
        PhyloTree tree;
        tree.treeDesc.resize(n + 1, std::vector<int>(n + 1));
        SeqInfo info;
        info.firstSeq = 1;
        info.lastSeq = n;
        info.numSeqs = n;
        ClusterTreeAlgorithm* t = dropin ? (ClusterTreeAlgorithm*)new GpuNJTree(0) : (ClusterTreeAlgorithm*)new NJTree();
        std::ofstream rep((std::string(argv[4]) + ".report").c_str());
        t->setVerbose(true);
        t->generateTree(&tree, &dist, &info, &rep);
        delete t;
        rep.close();
        tree.leftBranch.resize(n + 2, 0.0);
        tree.rightBranch.resize(n + 2, 0.0);
        put(f, &tree.leftBranch[0], sizeof(double) * (n + 2));
        put(f, &tree.rightBranch[0], sizeof(double) * (n + 2));
        for (int i = 0; i <= n; ++i) put(f, &tree.treeDesc[i][0], sizeof(int) * (n + 1));
        put(f, dist.getElements(), sizeof(double) * (size_t)(n + 1) * (n + 2) / 2);
    }
    fclose(f);
    return 0;
}
