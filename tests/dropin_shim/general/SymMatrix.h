// Test stand-in for general/SymMatrix.h (see general/clustalw.h here): a
// symmetric matrix of doubles over 0..size-1 stored packed, element (i, j)
// with i <= j at j * (j + 1) / 2 + i, which is the layout the GB300 library
// writes distances into.
#ifndef DROPIN_SHIM_SYMMATRIX_H
#define DROPIN_SHIM_SYMMATRIX_H

#include <cstdio>
#include <vector>

namespace clustalw
{

class SymMatrix
{
    public:
        explicit SymMatrix(int size = 0) : n(size), el((size_t)size * (size + 1) / 2, 0.0) {}
        int getSize() const { return n; }
        double* getElements() { return el.empty() ? 0 : &el[0]; }
        double operator()(int i, int j) const { return el[index(i, j)]; }
        void SetAt(int i, int j, double v) { el[index(i, j)] = v; }
        void printArray() const
        {
            for (size_t k = 0; k < el.size(); ++k) std::printf("%g\n", el[k]);
        }
        size_t numElements() const { return el.size(); }

    private:
        static size_t index(int i, int j)
        {
            if (i > j) { const int t = i; i = j; j = t; }
            return (size_t)j * (j + 1) / 2 + i;
        }
        int n;
        std::vector<double> el;
};

typedef SymMatrix DistMatrix;

}
#endif
