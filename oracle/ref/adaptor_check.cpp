// Compile check of include/gsGpuPoissonAssembler.h and include/gsGpuExprAssembler.h against the
// reference headers (no run: the container has no GPU). Builds the 2D unit-square Poisson problem
// the way a G+Smo user would, through gsPoissonAssembler and through gsExprAssembler
// (examples/poisson2_example.cpp:90-153 with the assembler type swapped).
#include <gsCore/gsMultiPatch.h>
#include <gsCore/gsMultiBasis.h>
#include <gsCore/gsFunctionExpr.h>
#include <gsNurbs/gsKnotVector.h>
#include <gsSolver/gsConjugateGradient.h>
#include "gsGpuPoissonAssembler.h"
#include "gsGpuExprAssembler.h"
#include <gsAssembler/gsExprEvaluator.h>
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
        gsOptionList opt;
        opt.addString("Preconditioner", "", "MultiGrid");
        opt.addInt("Levels", "", 3);
        A.solve(opt, x);
        // G+Smo's own CG on the device operator and V-cycle
        gsGpuMatrixOp<> K(A);
        gsGpuMultiGridOp<> M(A);
        M.setOptions(opt);
        gsMatrix<> y, z;
        K.apply(x, y);
        M.apply(y, z);
        // the reference's own CG driven by the device operator and the device V-cycle
        gsLinearOperator<>::Ptr Kp(new gsGpuMatrixOp<>(A)), Mp(new gsGpuMultiGridOp<>(A));
        gsConjugateGradient<> cg(Kp, Mp);
        cg.setTolerance(1e-8);
        gsMatrix<> xs;
        xs.setZero(A.numDofs(), 1);
        cg.solve(A.rhs(), xs);
        // gsExprAssembler route
        gsGpuExprAssembler<> E(1, 1);
        typedef gsGpuExprAssembler<>::geometryMap geometryMap;
        typedef gsGpuExprAssembler<>::space space;
        E.setIntegrationElements(mb);
        gsExprEvaluator<> ev(E);
        geometryMap G = E.getMap(mp);
        space u = E.getSpace(mb);
        auto ff = E.getCoeff(f, G);
        auto kk = E.getCoeff(g, G);
        u.setup(bc, dirichlet::l2Projection, 0);
        E.initSystem();
        static_assert(gsgpu_expr::same<decltype(igrad(u, G) * igrad(u, G).tr() * meas(G)),
                                       gsgpu_expr::poisson<real_t>::lhs>::value, "Poisson form");
        static_assert(gsgpu_expr::same<decltype(igrad(u, G) * kk * igrad(u, G).tr() * meas(G)),
                                       gsgpu_expr::poisson<real_t>::lhs_kappa>::value, "diffusion form");
        static_assert(gsgpu_expr::same<decltype(u * ff * meas(G)), gsgpu_expr::poisson<real_t>::rhs_coeff>::value,
                      "source form");
        static_assert(!gsgpu_expr::same<decltype(u * u.tr() * meas(G)), gsgpu_expr::poisson<real_t>::lhs>::value,
                      "a mass matrix is not the Poisson form");
        E.assemble(igrad(u, G) * igrad(u, G).tr() * meas(G), u * ff * meas(G));
        E.assemble(igrad(u, G) * kk * igrad(u, G).tr() * meas(G), u * ff * meas(G));
        auto g_N = E.getBdrFunction(G);
        E.assembleBdr(bc.get("Neumann"), u * g_N.tr() * nv(G));
        gsSparseSolver<>::CGDiagonal solver;
        solver.compute(E.matrix());
        gsMatrix<> sol = solver.solve(E.rhs());
        return int(A.matrix().nonZeros() + x.rows() + z.rows() + A.distanceL2() + A.distanceH1() + A.error() + cg.iterations() +
                   E.numDofs() + sol.rows());
    }
    return 0;
}
