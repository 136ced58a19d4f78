// Parity-fixture driver for the G+Smo reference (test infrastructure only; never shipped).
//
// Reads a problem specification (the text format written by gismo_gb300/problems.py,
// `write_spec`), builds the G+Smo objects, runs the reference's own FP64 assembler and
// solver and dumps raw results into an output directory:
//   dofmap.i32      gsDofMapper::asVector (src/gsCore/gsDofMapper.cpp:80-87), all patches
//   csc_ptr.i32     outerIndexPtr of the compressed ColMajor matrix (gsAssembler.h:614)
//   csc_idx.i32     innerIndexPtr
//   csc_val.f64     valuePtr
//   rhs.f64         gsAssembler::rhs() (gsAssembler.h:618)
//   ddof.f64        gsAssembler::fixedDofs() (gsAssembler.h:538)
//   x.f64           solution of gsConjugateGradient (+ gsJacobiOp or gsMultiGridOp)
//   info.txt        free dofs, nnz, iterations, relative residual, L2 error, timings
//
// Assembler: gsPoissonAssembler (src/gsAssembler/gsPoissonAssembler.h:93) when kappa is the
// constant 1, else gsCDRAssembler with A = kappa*I, b = 0, c = 0 (gsCDRAssembler.h:113).
#include <gsCore/gsMultiPatch.h>
#include <gsCore/gsMultiBasis.h>
#include <gsCore/gsField.h>
#include <gsNurbs/gsKnotVector.h>
#include <gsNurbs/gsTensorBSplineBasis.h>
#include <gsNurbs/gsTensorBSpline.h>
#include <gsPde/gsBoundaryConditions.h>
#include <gsAssembler/gsPoissonAssembler.h>
#include <gsAssembler/gsCDRAssembler.h>
#include <gsAssembler/gsGenericAssembler.h>
#include <gsSolver/gsConjugateGradient.h>
#include <gsSolver/gsSimplePreconditioners.h>
#include <gsSolver/gsMatrixOp.h>
#include <gsMultiGrid/gsMultiGrid.h>
#include <gsMultiGrid/gsGridHierarchy.h>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

using namespace gismo;

namespace {

struct Mode { double amp; int k[3]; double phase; };

struct Spec {
    int dim = 2;
    struct Patch {
        int deg[3] = {0, 0, 0};
        std::vector<double> knots[3];
        int gdeg[3] = {0, 0, 0};
        std::vector<double> gknots[3];
        std::vector<double> coefs;  // ncoef x dim, row-major
    };
    std::vector<Patch> patches;
    std::vector<std::array<int, 4>> ifaces;
    std::vector<std::array<int, 2>> dirichlet;
    std::vector<std::array<int, 2>> neumann;
    bool kappa_fourier = false;
    double kappa_const = 1.0, kappa_alpha = 0.0, kappa_scale = 0.0;
    std::vector<Mode> modes;
    int ufreq = 1;
    double quA = 1.0;
    int quB = 1;
    std::string solver = "cg";
    double tol = 1e-10;
    int maxit = 1000;
    int levels = 4, npre = 2, npost = 2;
    double damping = 0.6;
    int cycles = 1;
    double cgc = 1.0;
    int dirL2 = 0;  // Dirichlet values by L2 projection instead of interpolation
};

Spec readSpec(const std::string& path) {
    std::ifstream in(path);
    if (!in) { std::cerr << "cannot open " << path << "\n"; std::exit(2); }
    Spec s;
    std::string tok;
    in >> tok;  // magic
    int ver; in >> ver;
    while (in >> tok) {
        if (tok == "dim") in >> s.dim;
        else if (tok == "patch") {
            Spec::Patch p;
            for (int k = 0; k < s.dim; ++k) in >> p.deg[k];
            for (int k = 0; k < s.dim; ++k) { int n; in >> n; p.knots[k].resize(n); for (auto& v : p.knots[k]) in >> v; }
            for (int k = 0; k < s.dim; ++k) in >> p.gdeg[k];
            for (int k = 0; k < s.dim; ++k) { int n; in >> n; p.gknots[k].resize(n); for (auto& v : p.gknots[k]) in >> v; }
            int nc; in >> nc; p.coefs.resize(size_t(nc) * s.dim);
            for (auto& v : p.coefs) in >> v;
            s.patches.push_back(p);
        } else if (tok == "interface") {
            std::array<int, 4> a; in >> a[0] >> a[1] >> a[2] >> a[3]; s.ifaces.push_back(a);
        } else if (tok == "dirichlet") {
            std::array<int, 2> a; in >> a[0] >> a[1]; s.dirichlet.push_back(a);
        } else if (tok == "neumann") {
            std::array<int, 2> a; in >> a[0] >> a[1]; s.neumann.push_back(a);
        } else if (tok == "kappa_const") { in >> s.kappa_const; s.kappa_fourier = false; }
        else if (tok == "kappa_fourier") {
            int nm; in >> s.kappa_alpha >> s.kappa_scale >> nm; s.kappa_fourier = true;
            s.modes.resize(nm);
            for (auto& m : s.modes) in >> m.amp >> m.k[0] >> m.k[1] >> m.k[2] >> m.phase;
        } else if (tok == "ufreq") in >> s.ufreq;
        else if (tok == "quad") in >> s.quA >> s.quB;
        else if (tok == "dirichlet_values") { std::string v; in >> v; s.dirL2 = v == "l2" ? 1 : 0; }
        else if (tok == "solver") in >> s.solver >> s.tol >> s.maxit;
        else if (tok == "mg") in >> s.levels >> s.npre >> s.npost >> s.damping;
        else if (tok == "mgcycle") in >> s.cycles >> s.cgc;
        else if (tok == "end") break;
        else { std::cerr << "bad token " << tok << "\n"; std::exit(2); }
    }
    return s;
}

// Closed forms shared with the GPU path:
//   g(x)   = scale * sum_m amp_m cos(pi k_m.x + phase_m)
//   kappa  = exp(alpha g)            (or a constant)
//   u(x)   = prod_i sin(freq pi x_i)
//   f      = -div(kappa grad u) = kappa (d freq^2 pi^2 u - alpha grad g . grad u)
struct Fields {
    const Spec& s;
    void eval(const double* x, double& kappa, double& f, double& u) const {
        const int d = s.dim;
        const double w = s.ufreq * M_PI;
        double sn[3], cs[3];
        for (int i = 0; i < d; ++i) { sn[i] = std::sin(w * x[i]); cs[i] = std::cos(w * x[i]); }
        u = 1.0;
        for (int i = 0; i < d; ++i) u *= sn[i];
        double gu[3];
        for (int j = 0; j < d; ++j) {
            gu[j] = w * cs[j];
            for (int i = 0; i < d; ++i) if (i != j) gu[j] *= sn[i];
        }
        double g = 0, gg[3] = {0, 0, 0};
        if (s.kappa_fourier) {
            for (const Mode& m : s.modes) {
                double th = m.phase;
                for (int i = 0; i < d; ++i) th += M_PI * m.k[i] * x[i];
                g += m.amp * std::cos(th);
                const double sth = std::sin(th);
                for (int i = 0; i < d; ++i) gg[i] -= m.amp * sth * M_PI * m.k[i];
            }
            g *= s.kappa_scale;
            for (int i = 0; i < d; ++i) gg[i] *= s.kappa_scale;
            kappa = std::exp(s.kappa_alpha * g);
        } else {
            kappa = s.kappa_const;
        }
        double dot = 0;
        for (int i = 0; i < d; ++i) dot += gg[i] * gu[i];
        f = kappa * (d * w * w * u - s.kappa_alpha * dot);
    }
};

class KappaMatrix : public gsFunction<real_t> {
    Fields F;
public:
    explicit KappaMatrix(const Spec& s) : F{s} {}
    GISMO_CLONE_FUNCTION(KappaMatrix)
    short_t domainDim() const override { return F.s.dim; }
    short_t targetDim() const override { return F.s.dim * F.s.dim; }
    void eval_into(const gsMatrix<real_t>& u, gsMatrix<real_t>& r) const override {
        const int d = F.s.dim;
        r.setZero(d * d, u.cols());
        for (index_t c = 0; c < u.cols(); ++c) {
            double k, f, uu; F.eval(u.col(c).data(), k, f, uu);
            for (int i = 0; i < d; ++i) r(i * d + i, c) = k;
        }
    }
};
class RhsFunc : public gsFunction<real_t> {
    Fields F;
public:
    explicit RhsFunc(const Spec& s) : F{s} {}
    GISMO_CLONE_FUNCTION(RhsFunc)
    short_t domainDim() const override { return F.s.dim; }
    short_t targetDim() const override { return 1; }
    void eval_into(const gsMatrix<real_t>& u, gsMatrix<real_t>& r) const override {
        r.resize(1, u.cols());
        for (index_t c = 0; c < u.cols(); ++c) { double k, f, uu; F.eval(u.col(c).data(), k, f, uu); r(0, c) = f; }
    }
};
class SolFunc : public gsFunction<real_t> {
    Fields F;
public:
    explicit SolFunc(const Spec& s) : F{s} {}
    GISMO_CLONE_FUNCTION(SolFunc)
    const gsFunction& piece(const index_t) const override { return *this; }
    short_t domainDim() const override { return F.s.dim; }
    short_t targetDim() const override { return 1; }
    void eval_into(const gsMatrix<real_t>& u, gsMatrix<real_t>& r) const override {
        r.resize(1, u.cols());
        for (index_t c = 0; c < u.cols(); ++c) { double k, f, uu; F.eval(u.col(c).data(), k, f, uu); r(0, c) = uu; }
    }
    // the exact gradient (gsField::distanceH1 differentiates the exact function through this)
    void deriv_into(const gsMatrix<real_t>& u, gsMatrix<real_t>& r) const override {
        const int d = F.s.dim;
        const double w = F.s.ufreq * M_PI;
        r.resize(d, u.cols());
        for (index_t c = 0; c < u.cols(); ++c)
            for (int j = 0; j < d; ++j) {
                double g = w;
                for (int i = 0; i < d; ++i) g *= i == j ? std::cos(w * u(i, c)) : std::sin(w * u(i, c));
                r(j, c) = g;
            }
    }
};
// Neumann data of side s (direction k = (s-1)/2): sgn kappa du/dx_k, sgn = -1 on the lower side
class NeumannFunc : public gsFunction<real_t> {
    Fields F;
    int k;
    double sgn;
public:
    NeumannFunc(const Spec& s, int side) : F{s}, k((side - 1) / 2), sgn((side - 1) % 2 ? 1.0 : -1.0) {}
    GISMO_CLONE_FUNCTION(NeumannFunc)
    short_t domainDim() const override { return F.s.dim; }
    short_t targetDim() const override { return 1; }
    void eval_into(const gsMatrix<real_t>& u, gsMatrix<real_t>& r) const override {
        r.resize(1, u.cols());
        const double w = F.s.ufreq * M_PI;
        for (index_t c = 0; c < u.cols(); ++c) {
            double kap, f, uu;
            F.eval(u.col(c).data(), kap, f, uu);
            double du = w;
            for (int i = 0; i < F.s.dim; ++i) du *= i == k ? std::cos(w * u(i, c)) : std::sin(w * u(i, c));
            r(0, c) = sgn * kap * du;
        }
    }
};
class ConstFunc : public gsFunction<real_t> {
    int dd, td; double v;
public:
    ConstFunc(int d, int t, double val) : dd(d), td(t), v(val) {}
    GISMO_CLONE_FUNCTION(ConstFunc)
    short_t domainDim() const override { return dd; }
    short_t targetDim() const override { return td; }
    void eval_into(const gsMatrix<real_t>& u, gsMatrix<real_t>& r) const override { r.setConstant(td, u.cols(), v); }
};

template <class T>
void dump(const std::string& path, const T* p, size_t n) {
    FILE* f = std::fopen(path.c_str(), "wb");
    std::fwrite(p, sizeof(T), n, f);
    std::fclose(f);
}

template <short_t D>
gsGeometry<>::uPtr makePatch(const Spec::Patch& p, gsBasis<>::uPtr& basis) {
    std::vector<gsKnotVector<>> kv, gkv;
    for (int k = 0; k < D; ++k) {
        kv.emplace_back(p.knots[k], p.deg[k]);
        gkv.emplace_back(p.gknots[k], p.gdeg[k]);
    }
    gsMatrix<> coefs(p.coefs.size() / D, D);
    for (index_t i = 0; i < coefs.rows(); ++i)
        for (int k = 0; k < D; ++k) coefs(i, k) = p.coefs[size_t(i) * D + k];
    gsTensorBSplineBasis<D> gb(gkv);
    basis.reset(new gsTensorBSplineBasis<D>(kv));
    return gsGeometry<>::uPtr(new gsTensorBSpline<D>(gb, coefs));
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) { std::cerr << "usage: gsref spec.txt outdir [nosolve]\n"; return 2; }
    const Spec s = readSpec(argv[1]);
    const std::string out = argv[2];
    const bool solve = !(argc > 3 && std::string(argv[3]) == "nosolve");

    gsMultiPatch<> mp;
    std::vector<gsBasis<>*> bases;
    for (const auto& p : s.patches) {
        gsBasis<>::uPtr b;
        gsGeometry<>::uPtr g = (s.dim == 2) ? makePatch<2>(p, b) : makePatch<3>(p, b);
        mp.addPatch(give(g));
        bases.push_back(b.release());
    }
    for (const auto& f : s.ifaces)
        mp.addInterface(f[0], boxSide(f[1]), f[2], boxSide(f[3]));
    mp.addAutoBoundaries();
    gsMultiBasis<> mb(bases, mp.topology());
    for (auto* b : bases) delete b;

    KappaMatrix kappaA(s);
    RhsFunc rhsF(s);
    SolFunc solF(s);
    ConstFunc zeroB(s.dim, s.dim, 0.0), zeroC(s.dim, 1, 0.0);

    gsBoundaryConditions<> bc;
    for (const auto& d : s.dirichlet)
        bc.addCondition(d[0], boxSide(d[1]), condition_type::dirichlet, &solF);
    std::vector<std::unique_ptr<NeumannFunc>> neuF;
    for (const auto& d : s.neumann) {
        neuF.emplace_back(new NeumannFunc(s, d[1]));
        bc.addCondition(d[0], boxSide(d[1]), condition_type::neumann, neuF.back().get());
    }

    std::unique_ptr<gsAssembler<>> A;
    const bool poisson = !s.kappa_fourier && s.kappa_const == 1.0;
    if (poisson)
        A.reset(new gsPoissonAssembler<>(mp, mb, bc, rhsF, dirichlet::elimination, iFace::glue));
    else
        A.reset(new gsCDRAssembler<>(mp, mb, bc, rhsF, kappaA, zeroB, zeroC, dirichlet::elimination, iFace::glue));
    A->options().setReal("quA", s.quA);
    A->options().setInt("quB", s.quB);
    if (s.dirL2) A->options().setInt("DirichletValues", dirichlet::l2Projection);

    auto t0 = std::chrono::steady_clock::now();
    A->assemble();
    auto t1 = std::chrono::steady_clock::now();

    const gsDofMapper& map = A->system().colMapper(0);
    {
        gsVector<index_t> v = map.asVector(0);
        dump(out + "/dofmap.i32", v.data(), v.size());
    }
    const gsSparseMatrix<>& K = A->matrix();
    dump(out + "/csc_ptr.i32", K.outerIndexPtr(), size_t(K.cols()) + 1);
    dump(out + "/csc_idx.i32", K.innerIndexPtr(), size_t(K.nonZeros()));
    dump(out + "/csc_val.f64", K.valuePtr(), size_t(K.nonZeros()));
    dump(out + "/rhs.f64", A->rhs().data(), size_t(A->rhs().rows()));
    dump(out + "/ddof.f64", A->fixedDofs().data(), size_t(A->fixedDofs().rows()));
    {
        // gsGenericAssembler::assembleMass with the same boundary conditions (the same dof map)
        gsOptionList gopt = gsGenericAssembler<>::defaultOptions();
        gopt.setReal("quA", s.quA);
        gopt.setInt("quB", s.quB);
        gopt.setInt("DirichletStrategy", dirichlet::elimination);
        gopt.setInt("InterfaceStrategy", iFace::glue);
        gsGenericAssembler<> G(mp, mb, gopt, &bc);
        const gsSparseMatrix<>& M = G.assembleMass();
        dump(out + "/mass_ptr.i32", M.outerIndexPtr(), size_t(M.cols()) + 1);
        dump(out + "/mass_idx.i32", M.innerIndexPtr(), size_t(M.nonZeros()));
        dump(out + "/mass_val.f64", M.valuePtr(), size_t(M.nonZeros()));
    }

    int iters = 0;
    double err = 0, l2 = 0, h1 = 0;
    double tsolve = 0;
    if (solve) {
        gsMatrix<> x;
        auto t2 = std::chrono::steady_clock::now();
        if (s.solver == "mg") {
            gsOptionList opt = gsGridHierarchy<>::defaultOptions();
            opt.setInt("Levels", s.levels);
            std::vector<gsSparseMatrix<real_t, RowMajor>> transfer;
            gsGridHierarchy<>::buildByCoarsening(give(gsMultiBasis<>(mb)), bc, opt)
                .moveTransferMatricesTo(transfer);
            gsMultiGridOp<>::Ptr mg = gsMultiGridOp<>::make(K, transfer);
            gsOptionList mgopt;
            mgopt.addInt("NumPreSmooth", "", s.npre);
            mgopt.addInt("NumPostSmooth", "", s.npost);
            mgopt.addInt("NumCycles", "", s.cycles);
            mgopt.addReal("CoarseGridCorrectionDamping", "", s.cgc);
            mg->setOptions(mgopt);
            mg->setCoarseSolver(makeSparseCholeskySolver(mg->matrix(0)));
            for (index_t i = 1; i < mg->numLevels(); ++i) {
                gsPreconditionerOp<>::Ptr sm = makeJacobiOp(mg->matrix(i));
                gsOptionList smopt;
                smopt.addReal("Damping", "", s.damping);
                sm->setOptions(smopt);
                mg->setSmoother(i, sm);
            }
            gsConjugateGradient<> cg(K, mg);
            cg.setTolerance(s.tol);
            cg.setMaxIterations(s.maxit);
            cg.solve(A->rhs(), x);
            iters = cg.iterations(); err = cg.error();
        } else {
            gsConjugateGradient<> cg(K, makeJacobiOp(K));
            cg.setTolerance(s.tol);
            cg.setMaxIterations(s.maxit);
            cg.solve(A->rhs(), x);
            iters = cg.iterations(); err = cg.error();
        }
        auto t3 = std::chrono::steady_clock::now();
        tsolve = std::chrono::duration<double>(t3 - t2).count();
        dump(out + "/x.f64", x.data(), size_t(x.rows()));
        gsMultiPatch<> sol;
        A->constructSolution(x, sol);
        gsField<> uh(mp, sol);
        l2 = uh.distanceL2(solF, mb, false);
        h1 = uh.distanceH1(solF, mb, false);
    }
    std::ofstream info(out + "/info.txt");
    info.precision(17);
    info << "free " << A->numDofs() << "\nnnz " << K.nonZeros() << "\nboundary " << map.boundarySize()
         << "\niters " << iters << "\nerror " << err << "\nl2 " << l2 << "\nh1 " << h1
         << "\nt_assemble " << std::chrono::duration<double>(t1 - t0).count() << "\nt_solve " << tsolve << "\n";
    return 0;
}
