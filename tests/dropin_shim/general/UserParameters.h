// Test stand-in for general/UserParameters.h (see general/clustalw.h here):
// the settings the drop-ins read, set directly by the test driver. The quick
// k-tuple settings exist twice, for DNA and protein, and setDNAParams /
// setProtParams make one pair current, as the drop-in expects.
#ifndef DROPIN_SHIM_USERPARAMETERS_H
#define DROPIN_SHIM_USERPARAMETERS_H

#include "general/clustalw.h"

namespace clustalw
{

struct QuickParams
{
    int ktup, window, windowGap, signif;
};

class UserParameters
{
    public:
        UserParameters()
        : dnaFlag(false), displayInfo(false), percent(true), pwGapOpen(0), pwGapExtend(0),
          gapPos1(31), gapPos2(30), maxAA(24)
        {
            dnaQuick.ktup = dnaQuick.window = dnaQuick.windowGap = dnaQuick.signif = 0;
            protQuick = current = dnaQuick;
        }
        bool getDNAFlag() const { return dnaFlag; }
        bool getDisplayInfo() const { return displayInfo; }
        float getPWGapOpen() const { return pwGapOpen; }
        float getPWGapExtend() const { return pwGapExtend; }
        int getGapPos1() const { return gapPos1; }
        int getGapPos2() const { return gapPos2; }
        int getKtup() const { return current.ktup; }
        int getWindow() const { return current.window; }
        int getWindowGap() const { return current.windowGap; }
        int getSignif() const { return current.signif; }
        bool getPercent() const { return percent; }
        int getMaxAA() const { return maxAA; }
        void setDNAParams() { current = dnaQuick; }
        void setProtParams() { current = protQuick; }

        bool dnaFlag, displayInfo, percent;
        float pwGapOpen, pwGapExtend;
        int gapPos1, gapPos2, maxAA;
        QuickParams dnaQuick, protQuick, current;
};

extern UserParameters* userParameters;

}
#endif
