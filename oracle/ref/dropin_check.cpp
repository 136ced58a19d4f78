// Host-side check of the C++ drop-in's function check (include/gsGpuPoissonAssembler.h) on
// host-only contexts (device -1, no GPU): the caller's rhs, Dirichlet and Neumann functions are
// compared with the closed forms the device evaluates, and a mismatch throws instead of silently
// assembling another problem (the reference evaluates exactly the caller's functions,
// gsVisitorPoisson.h:81, gsAssembler.hpp:314-390). Prints "ok" when every case behaves.
#include <gsCore/gsMultiPatch.h>
#include <gsCore/gsMultiBasis.h>
#include <gsCore/gsFunctionExpr.h>
#include <gsNurbs/gsKnotVector.h>
#include <cstdio>
#include <string>
#include "gsGpuPoissonAssembler.h"
using namespace gismo;

static int fails = 0;

template <class F>
static void expect(bool throws, const char* what, F&& make) {
    bool threw = false;
    std::string msg;
    try {
        make();
    } catch (const std::invalid_argument& e) {
        threw = true;
        msg = e.what();
    }
    if (threw != throws) {
        std::printf("FAIL %s: %s (%s)\n", what, throws ? "no exception" : "unexpected exception", msg.c_str());
        ++fails;
    }
}

int main() {
    gsKnotVector<> kv(0, 1, 7, 3);
    gsTensorBSplineBasis<2> basis(kv, kv);
    gsTensorBSpline<2> geo(basis, basis.anchors().transpose());
    gsMultiPatch<> mp(geo);
    mp.computeTopology();
    gsMultiBasis<> mb(mp);
    gsGpuFields F;  // kappa = 1, u = sin(pi x) sin(pi y)
    gsFunctionExpr<> f("2*pi^2*sin(pi*x)*sin(pi*y)", 2), wrongf("2*pi^2*sin(pi*x)*sin(pi*y) + 1e-3", 2);
    gsFunctionExpr<> u("sin(pi*x)*sin(pi*y)", 2), zero("0", 2), wrongu("x", 2);
    // flux kappa grad u . n on the east side (x = 1: +du/dx) and the north side (y = 1: +du/dy)
    gsFunctionExpr<> fluxE("pi*cos(pi*x)*sin(pi*y)", 2), fluxN("pi*sin(pi*x)*cos(pi*y)", 2);
    auto run = [&](gsFunctionExpr<>& rhs, gsFunctionExpr<>& dir, gsFunctionExpr<>* ne, gsFunctionExpr<>* nn) {
        gsBoundaryConditions<> bc;
        bc.addCondition(0, boundary::west, condition_type::dirichlet, &dir);
        bc.addCondition(0, boundary::south, condition_type::dirichlet, &dir);
        if (ne) bc.addCondition(0, boundary::east, condition_type::neumann, ne);
        else bc.addCondition(0, boundary::east, condition_type::dirichlet, &dir);
        if (nn) bc.addCondition(0, boundary::north, condition_type::neumann, nn);
        else bc.addCondition(0, boundary::north, condition_type::dirichlet, &dir);
        gsGpuPoissonAssembler<> A(mp, mb, bc, rhs, F, -1);
        if (A.numDofs() <= 0) throw std::logic_error("no dofs");
    };
    expect(false, "matching rhs and Dirichlet data", [&] { run(f, u, nullptr, nullptr); });
    expect(false, "zero Dirichlet data on the unit square's sides", [&] { run(f, zero, nullptr, nullptr); });
    expect(false, "matching Neumann fluxes", [&] { run(f, u, &fluxE, &fluxN); });
    expect(true, "a different rhs", [&] { run(wrongf, u, nullptr, nullptr); });
    expect(true, "different Dirichlet data", [&] { run(f, wrongu, nullptr, nullptr); });
    expect(true, "a different Neumann flux", [&] { run(f, u, &fluxN, &fluxN); });
    if (fails) return 1;
    std::printf("ok\n");
    return 0;
}
