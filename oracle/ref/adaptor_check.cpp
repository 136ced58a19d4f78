// Compile check of include/gsGpuPoissonAssembler.h against the reference headers (no run: the
// container has no GPU). Builds the 2D unit-square Poisson problem the way a G+Smo user would.
#include <gsCore/gsMultiPatch.h>
#include <gsCore/gsMultiBasis.h>
#include <gsCore/gsFunctionExpr.h>
#include <gsNurbs/gsKnotVector.h>
#include "gsGpuPoissonAssembler.h"
using namespace gismo;
int main(int argc, char**) {
    gsKnotVector<> kv(0, 1, 63, 3);
    gsTensorBSplineBasis<2> basis(kv, kv);
    gsTensorBSpline<2> geo(basis, basis.anchors().transpose());
    gsMultiPatch<> mp(geo);
    gsMultiBasis<> mb(mp);
    gsFunctionExpr<> f("2*pi^2*sin(pi*x)*sin(pi*y)", 2), g("0", 2);
    gsBoundaryConditions<> bc;
    for (boxSide s : {boundary::west, boundary::east, boundary::south, boundary::north})
        bc.addCondition(0, s, condition_type::dirichlet, &g);
    if (argc > 5) {  // never taken in the compile check
        gsGpuFields F;
        gsGpuPoissonAssembler<> A(mp, mb, bc, f, F, 0);
        A.assemble();
        gsMatrix<> x;
        A.solve(x);
        return int(A.matrix().nonZeros() + x.rows());
    }
    return 0;
}
