// Test stand-in for general/Utility.h (see general/clustalw.h here): info()
// prints one line to standard output.
#ifndef DROPIN_SHIM_UTILITY_H
#define DROPIN_SHIM_UTILITY_H

#include <cstdarg>
#include <cstdio>

namespace clustalw
{

class Utility
{
    public:
        int MAX(int a, int b) const { return a > b ? a : b; }
        int MIN(int a, int b) const { return a < b ? a : b; }
        void info(const char* fmt, ...) const
        {
            va_list ap;
            va_start(ap, fmt);
            std::vprintf(fmt, ap);
            va_end(ap);
            std::printf("\n");
        }
};

extern Utility* utilityObject;

}
#endif
