// Reference harness: links the UNMODIFIED ClustalW 2.0.11 CPU objects (built from
// the reference tree by oracle/build_ref.sh, outputs only under oracle/_ref/) and
// runs clustalw::FullPairwiseAlign::pairwiseAlign on one FASTA file.
//
// TEST INFRASTRUCTURE ONLY. This program is the reference itself, used to pin the
// oracle restatement (oracle/oracle.c) and to write the golden fixtures under
// tests/golden/. Nothing in the shipped library calls it.
//
// It mirrors what Clustal::align does before the pairwise stage
// (CPU/clustalw-2.0.11/src/Clustal.cpp:129-162): sequence input through
// FileReader::readSeqs (Clustal.cpp:1051-1059), setDNAParams/setProtParams,
// DistMatrix sized numSeqs+1, then one pairwiseAlign(iStart, iEnd, jStart, jEnd).
//
// Usage: refharness IN.fa OUT.bin [iStart iEnd jStart jEnd]
//        refharness --fast IN.fa OUT.bin [iStart iEnd jStart jEnd]
//        refharness --nj IN.dist OUT.tree [OUT.report]
//        refharness --dnd IN.fa IN.dist OUT.dnd
// (CWREF_PWMATRIX, CWREF_PWGAPOPEN, CWREF_PWGAPEXT in the environment change the
// pairwise matrix and gap penalties, see apply_overrides; CWREF_KTUP,
// CWREF_WINDOW, CWREF_WINDOWGAP, CWREF_SIGNIF, CWREF_PERCENT the quick-distance
// settings, see apply_quick_overrides.)
//
// --fast runs clustalw::FastPairwiseAlign::pairwiseAlign (the k-tuple quick
// distances, pairwise/FastPairwiseAlign.cpp:20-139) instead; its OUT.bin starts
// with "CWREF02\0" and adds, after the four floats, int32 ktup, window,
// windowGap, signif, percent, maxAA (the userParameters values the call used).
//
// --nj runs clustalw::NJTree::generateTree (tree/NJTree.cpp:161-748) the way
// UnRootedClusterTree::treeFromDistMatrix calls it (tree/UnRootedClusterTree.cpp:
// 236-245): IN.dist is int32 n followed by the packed SymMatrix elements
// (double[(n+1)(n+2)/2]); OUT.tree is int32 n, double leftBranch[n+2],
// double rightBranch[n+2], int32 treeDesc[(n+1)*(n+1)], and the SymMatrix
// elements as generateTree leaves them (it works in place). With OUT.report the
// tree is built verbose and the reference's cycle report is written there.
//
// OUT.bin layout (little endian):
//   char[8]  "CWREF01\0"
//   int32    nseqs, dna_flag, int_scale, mat_avg, gap_pos1, gap_pos2, max_aln_length
//   float    pw_gap_open, pw_gap_extend, gap_open_scale, gap_extend_scale
//   int32    matrix[32*32]          (SubMatrix::getPairwiseMatrix output)
//   int32    lens[nseqs]
//   int32    codes[sum(lens)]       (SeqArray rows 1..nseqs, elements 1..len)
//   int32    range[4]               (iStart, iEnd, jStart, jEnd)
//   double   elements[(N+1)(N+2)/2] (SymMatrix::getElements, packed lower triangle)
//   double   seconds                (wall time of pairwiseAlign)
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
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
#include "tree/UnRootedClusterTree.h"

namespace clustalw {
UserParameters* userParameters;
Utility* utilityObject;
SubMatrix* subMatrix;
DebugLog* logObject;
Stats* statsObject;
}  // namespace clustalw

using namespace clustalw;

#include "ref_overrides.h"

static void put(FILE* f, const void* p, size_t n) {
    if (n && fwrite(p, 1, n, f) != n) {
        fprintf(stderr, "refharness: short write\n");
        exit(2);
    }
}

static int run_nj(const char* in, const char* out, const char* report) {
    FILE* f = fopen(in, "rb");
    if (!f) return 4;
    int n = 0;
    if (fread(&n, sizeof(int), 1, f) != 1 || n < 2) return 5;
    SymMatrix dist;
    dist.ResizeRect(n + 1);
    size_t nel = (size_t)(n + 1) * (n + 2) / 2;
    if (fread(dist.getElements(), sizeof(double), nel, f) != nel) return 5;
    fclose(f);
    PhyloTree tree;
    tree.treeDesc.resize(n + 1, std::vector<int>(n + 1));
    SeqInfo info;
    info.firstSeq = 1;
    info.lastSeq = n;
    info.numSeqs = n;
    NJTree nj;
    std::ofstream rep;
    if (report) {
        rep.open(report);
        nj.setVerbose(true);
    }
    auto t0 = std::chrono::steady_clock::now();
    nj.generateTree(&tree, &dist, &info, report ? &rep : 0);
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    tree.leftBranch.resize(n + 2, 0.0);
    tree.rightBranch.resize(n + 2, 0.0);
    FILE* g = fopen(out, "wb");
    if (!g) return 4;
    put(g, &n, sizeof(int));
    put(g, tree.leftBranch.data(), sizeof(double) * (n + 2));
    put(g, tree.rightBranch.data(), sizeof(double) * (n + 2));
    for (int i = 0; i <= n; ++i) put(g, tree.treeDesc[i].data(), sizeof(int) * (n + 1));
    put(g, dist.getElements(), sizeof(double) * nel);
    put(g, &secs, sizeof(secs));
    fclose(g);
    printf("refharness: NJ on %d sequences, %.6f s\n", n, secs);
    return 0;
}

// --dnd: the guide-tree file Clustal::align writes after the pairwise stage
// (TreeInterface::generateTreeFromDistMatNJ -> UnRootedClusterTree::
// treeFromDistMatrix, tree/TreeInterface.cpp:418-430, tree/UnRootedClusterTree.cpp:
// 171-260), from a given DistMatrix (IN.dist: int32 n, then the packed
// elements) and the sequence names of IN.fa.
static int run_dnd(const char* fasta, const char* dist_in, const char* out) {
    userParameters->setDisplayInfo(false);
    userParameters->setSeqName(std::string(fasta));
    Alignment aln;
    FileReader reader;
    if (reader.readSeqs(&aln, 1) != OK) return 3;
    const int n = aln.getNumSeqs();
    FILE* f = fopen(dist_in, "rb");
    if (!f) return 4;
    int n2 = 0;
    if (fread(&n2, sizeof(int), 1, f) != 1 || n2 != n) return 5;
    SymMatrix dist;
    dist.ResizeRect(n + 1);
    const size_t nel = (size_t)(n + 1) * (n + 2) / 2;
    if (fread(dist.getElements(), sizeof(double), nel, f) != nel) return 5;
    fclose(f);
    std::string name(out);
    UnRootedClusterTree tree;
    tree.treeFromDistMatrix(&dist, &aln, 1, n, name);
    return 0;
}

int main(int argc, char** argv) {
    bool fast = false;
    if (argc > 1 && std::string(argv[1]) == "--fast") {
        fast = true;
        --argc;
        ++argv;
    }
    if ((argc == 4 || argc == 5) && std::string(argv[1]) == "--nj") {
        userParameters = new UserParameters(false);
        utilityObject = new Utility();
        return run_nj(argv[2], argv[3], argc == 5 ? argv[4] : 0);
    }
    if (argc == 5 && std::string(argv[1]) == "--dnd") {
        userParameters = new UserParameters(false);
        utilityObject = new Utility();
        subMatrix = new SubMatrix();
        statsObject = new Stats();
        return run_dnd(argv[2], argv[3], argv[4]);
    }
    if (argc != 3 && argc != 7) {
        fprintf(stderr, "usage: %s IN.fa OUT.bin [iStart iEnd jStart jEnd]\n", argv[0]);
        return 2;
    }
    userParameters = new UserParameters(false);
    utilityObject = new Utility();
    subMatrix = new SubMatrix();
    statsObject = new Stats();
    // CWREF_DISPLAY_INFO=1: the per-pair info lines of FullPairwiseAlign.cpp:185-189
    // (and FastPairwiseAlign's) go to standard output, as clustalw2 prints them
    // without -QUIET.
    const char* disp = getenv("CWREF_DISPLAY_INFO");
    userParameters->setDisplayInfo(disp && *disp == '1');
    userParameters->setSeqName(std::string(argv[1]));

    Alignment aln;
    FileReader reader;
    int code = reader.readSeqs(&aln, 1);
    if (code != OK) {
        fprintf(stderr, "refharness: readSeqs failed with code %d\n", code);
        return 3;
    }
    apply_overrides(userParameters->getDNAFlag());
    apply_quick_overrides(userParameters->getDNAFlag());
    if (userParameters->getDNAFlag())
        userParameters->setDNAParams();
    else
        userParameters->setProtParams();

    const int n = aln.getNumSeqs();
    int range[4] = {0, n, 0, n};
    if (argc == 7)
        for (int k = 0; k < 4; ++k) range[k] = atoi(argv[3 + k]);

    SymMatrix dist;
    dist.ResizeRect(n + 1);

    auto t0 = std::chrono::steady_clock::now();
    if (fast) {
        FastPairwiseAlign qpa;
        qpa.pairwiseAlign(&aln, &dist, range[0], range[1], range[2], range[3]);
    } else {
        FullPairwiseAlign fpa;
        fpa.pairwiseAlign(&aln, &dist, range[0], range[1], range[2], range[3]);
    }
    auto t1 = std::chrono::steady_clock::now();
    double secs = std::chrono::duration<double>(t1 - t0).count();

    int matrix[NUMRES][NUMRES];
    PairScaleValues scale;
    int mat_avg = 0;
    subMatrix->getPairwiseMatrix(matrix, scale, mat_avg);

    FILE* f = fopen(argv[2], "wb");
    if (!f) {
        fprintf(stderr, "refharness: cannot open %s\n", argv[2]);
        return 4;
    }
    put(f, fast ? "CWREF02\0" : "CWREF01\0", 8);
    int hdr[7] = {n,
                  userParameters->getDNAFlag() ? 1 : 0,
                  scale.intScale,
                  mat_avg,
                  userParameters->getGapPos1(),
                  userParameters->getGapPos2(),
                  aln.getMaxAlnLength()};
    put(f, hdr, sizeof(hdr));
    float fl[4] = {userParameters->getPWGapOpen(), userParameters->getPWGapExtend(),
                   scale.gapOpenScale, scale.gapExtendScale};
    put(f, fl, sizeof(fl));
    if (fast) {
        int kp[6] = {userParameters->getKtup(), userParameters->getWindow(), userParameters->getWindowGap(),
                     userParameters->getSignif(), userParameters->getPercent() ? 1 : 0, userParameters->getMaxAA()};
        put(f, kp, sizeof(kp));
    }
    put(f, matrix, sizeof(matrix));
    std::vector<int> lens(n);
    for (int s = 0; s < n; ++s) lens[s] = aln.getSeqLength(s + 1);
    put(f, lens.data(), sizeof(int) * n);
    const SeqArray* sa = aln.getSeqArray();
    for (int s = 0; s < n; ++s) put(f, (*sa)[s + 1].data() + 1, sizeof(int) * lens[s]);
    put(f, range, sizeof(range));
    size_t nel = (size_t)(n + 1) * (n + 2) / 2;
    put(f, dist.getElements(), sizeof(double) * nel);
    put(f, &secs, sizeof(secs));
    fclose(f);
    printf("refharness: %d seqs, dna=%d, %s pairwise %.6f s\n", n, hdr[1], fast ? "fast" : "full", secs);
    return 0;
}
