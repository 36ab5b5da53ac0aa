// Parameter overrides from the environment for programs that run the
// reference classes (oracle/ref_harness.cpp, tests/dropin_run_main.cpp).
// TEST INFRASTRUCTURE ONLY. Include after the reference's headers and
// `using namespace clustalw`.
#ifndef CW_REF_OVERRIDES_H
#define CW_REF_OVERRIDES_H

#include <cstdio>
#include <cstdlib>
#include <string>

// Optional parameter overrides from the environment, set the way clustalw2's
// -pwmatrix, -pwgapopen and -pwgapext options set them
// (interface/CommandLineParser.cpp:1811-1850, 2265-2300):
//   CWREF_PWMATRIX  blosum | pam | gonnet | id   (protein pairwise matrix)
//   CWREF_PWGAPOPEN, CWREF_PWGAPEXT                (real numbers >= 0)
// Called after the sequence type is known and before setDNAParams /
// setProtParams copy the per-type penalties into the pairwise ones.
static void apply_overrides(bool dna) {
    const char* m = getenv("CWREF_PWMATRIX");
    if (m && *m) {
        const std::string name(m);
        const int num = name == "blosum" ? 1 : name == "pam" ? 2 : name == "gonnet" ? 3 : name == "id" ? 4 : 0;
        if (!num) {
            fprintf(stderr, "refharness: unknown CWREF_PWMATRIX %s\n", m);
            exit(2);
        }
        subMatrix->setCurrentNameAndNum(name, num, Protein, Pairwise);
    }
    const char* go = getenv("CWREF_PWGAPOPEN");
    if (go && *go) {
        float v = 0.0f;  // sscanf %f like the option parser
        sscanf(go, "%f", &v);
        if (dna)
            userParameters->setDNAPWGapOpenPenalty(v);
        else
            userParameters->setProteinPWGapOpenPenalty(v);
    }
    const char* ge = getenv("CWREF_PWGAPEXT");
    if (ge && *ge) {
        float v = 0.0f;
        sscanf(ge, "%f", &v);
        if (dna)
            userParameters->setDNAPWGapExtendPenalty(v);
        else
            userParameters->setProteinPWGapExtendPenalty(v);
    }
}

// Quick-distance settings from the environment, stored as the per-type values
// (AA* or DNA*, like the option parser does) that FastPairwiseAlign's own
// setProtParams / setDNAParams call copies into the ones pairAlign reads
// (FastPairwiseAlign.cpp:56-63, 176-183); the output file records what was used:
//   CWREF_KTUP, CWREF_WINDOW, CWREF_WINDOWGAP, CWREF_SIGNIF (integers),
//   CWREF_PERCENT (0 or 1)
static void apply_quick_overrides(bool dna) {
    int v = 0;
    const char* e = getenv("CWREF_KTUP");
    if (e && *e && sscanf(e, "%d", &v) == 1) {
        if (dna) userParameters->setDNAKtup(v); else userParameters->setAAKtup(v);
    }
    e = getenv("CWREF_WINDOW");
    if (e && *e && sscanf(e, "%d", &v) == 1) {
        if (dna) userParameters->setDNAWindow(v); else userParameters->setAAWindow(v);
    }
    e = getenv("CWREF_WINDOWGAP");
    if (e && *e && sscanf(e, "%d", &v) == 1) {
        if (dna) userParameters->setDNAWindowGap(v); else userParameters->setAAWindowGap(v);
    }
    e = getenv("CWREF_SIGNIF");
    if (e && *e && sscanf(e, "%d", &v) == 1) {
        if (dna) userParameters->setDNASignif(v); else userParameters->setAASignif(v);
    }
    e = getenv("CWREF_PERCENT");
    if (e && *e && sscanf(e, "%d", &v) == 1) userParameters->setPercent(v != 0);
}

#endif  // CW_REF_OVERRIDES_H
