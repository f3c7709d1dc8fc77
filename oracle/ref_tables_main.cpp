// Host program pinning the oracle's B-spline tables against the reference's own host code.
// Compiled by oracle/build_ref.sh against the reference headers (mesh/FunctionData.h,
// math/PPolynomial.h, math/Polynomial.h, mesh/BinaryNode.h); never shipped.
// Prints, for a given max depth, the piecewise polynomial of the normalised base function
// and every non-zero entry of the three dot-product tables, as text.
#include <cfloat>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include "mesh/FunctionData.h"

using namespace SparseSurfelFusion;

int main(int argc, char** argv) {
    int depth = argc > 1 ? atoi(argv[1]) : 6;
    PPolynomial<2> F = PPolynomial<2>::GaussianApproximation();
    FunctionData<2, double> fd;
    fd.set(depth, F, 0, 0);
    fd.setDotTables(fd.DOT_FLAG | fd.D_DOT_FLAG | fd.D2_DOT_FLAG);
    printf("res %d\n", fd.res);
    printf("pieces %d\n", (int)fd.baseFunction.polyCount);
    for (size_t i = 0; i < fd.baseFunction.polyCount; i++) {
        printf("piece %.9g %.9g %.9g %.9g\n", fd.baseFunction.polys[i].start,
               fd.baseFunction.polys[i].p.coefficients[0], fd.baseFunction.polys[i].p.coefficients[1],
               fd.baseFunction.polys[i].p.coefficients[2]);
    }
    for (int i = 0; i < fd.res; i++)
        for (int j = 0; j < fd.res; j++) {
            int k = i + fd.res * j;
            if (fd.dotTable[k] != 0 || fd.dDotTable[k] != 0 || fd.d2DotTable[k] != 0)
                printf("t %d %d %.17g %.17g %.17g\n", i, j, fd.dotTable[k], fd.dDotTable[k], fd.d2DotTable[k]);
        }
    return 0;
}
