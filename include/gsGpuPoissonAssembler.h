/** gsGpuPoissonAssembler: drop-in for gismo::gsPoissonAssembler / gsCDRAssembler that assembles
 *  on a GB300 through libgsgpu (include/gsgpu.h).
 *
 *  Header-only; include it in a G+Smo build and link libgsgpu.so. It keeps the
 *  gsPoissonAssembler interface (src/gsAssembler/gsPoissonAssembler.h:35-142): construct from
 *  (gsMultiPatch, gsMultiBasis, gsBoundaryConditions, rhs), call assemble(), then matrix(),
 *  rhs(), fixedDofs(), numDofs(), constructSolution() as usual. refresh() builds the dof map and
 *  the sparsity pattern on the host and uploads the patch data; assemble() runs the device
 *  kernels and brings back the rhs and the eliminated-dof values; matrix() materialises the
 *  system matrix on first access after an assemble(), straight into the compressed ColMajor
 *  storage of m_system (one copy of the device CSR arrays, no per-entry insertion). Call matrix(),
 *  rhs() and fixedDofs() on the gsGpuPoissonAssembler itself: they hide the base class's
 *  (non-virtual) accessors; through a gsPoissonAssembler reference call matrix() on the derived
 *  object once first.
 *
 *  Functions: the device evaluates closed forms, so the coefficient, the source and the
 *  Dirichlet data are passed as gsGpuFields parameters (kappa = exp(alpha g) with a Fourier
 *  field g, or a constant; f = -div(kappa grad u) for u = prod sin(freq pi x_i)). refresh()
 *  checks the caller's own functions against them: the rhs function given to the constructor
 *  at points of every patch, each Dirichlet side's function (u) and each Neumann side's function
 *  (the flux kappa grad u . n of the closed forms on the box side) at points of the side; a
 *  mismatch beyond 1e-8 relative throws std::invalid_argument instead of silently computing
 *  another problem. The coefficient has no caller-side function in gsPoissonAssembler's
 *  constructor and comes from gsGpuFields alone.
 *  Supported inputs: gsTensorBSpline patches of dimension 2 or 3, tensor B-spline bases,
 *  conforming interfaces with identity orientation (iFace::glue), Dirichlet sides eliminated
 *  with values by interpolation or L2 projection ("DirichletValues"), Neumann sides with the
 *  closed-form flux of u as data. Anything else throws (no CPU fallback).
 */
#pragma once

#include <gsAssembler/gsPoissonAssembler.h>
#include <gsIO/gsOptionList.h>
#include <gsSolver/gsLinearOperator.h>
#include <gsNurbs/gsTensorBSpline.h>
#include <gsNurbs/gsTensorBSplineBasis.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "gsgpu.h"
#include "gsgpu.hpp"

namespace gismo {

struct gsGpuFields {
    bool kappaFourier = false;
    double kappaConst = 1.0, kappaAlpha = 0.0, kappaScale = 0.0;
    std::vector<double> amp, phase;
    std::vector<int> waves;  // 3 per mode
    int ufreq = 1;
};

/// A G+Smo problem packed into the C-ABI struct (include/gsgpu.h gsgpu_problem) together with the
/// arrays it points to: tensor B-spline patches and bases, conforming identity-oriented
/// interfaces, the Dirichlet and Neumann sides (patch, side index pairs) and the device fields
template <class T = real_t>
struct gsGpuProblemPack {
    std::vector<int> degree, nknots, gdegree, gnknots, ifaces, dsides, nsides;
    std::vector<double> knots, gknots, coefs;
    gsGpuFields fields;
    gsgpu_problem prob{};

    void pack(const gsMultiPatch<T>& mp, const gsMultiBasis<T>& mb, const std::vector<int>& dirichletSides,
              const gsGpuFields& f, double quA, int quB, int dirichletStrategy = GSGPU_DIRICHLET_INTERPOLATION,
              const std::vector<int>& neumannSides = std::vector<int>()) {
        const short_t d = mp.parDim();
        degree.clear(); nknots.clear(); knots.clear(); gdegree.clear(); gnknots.clear(); gknots.clear();
        coefs.clear(); ifaces.clear();
        for (size_t k = 0; k < mp.nPatches(); ++k) {
            if (d == 2) packPatch<2>(mp, mb, index_t(k));
            else if (d == 3) packPatch<3>(mp, mb, index_t(k));
            else throw std::invalid_argument("gsgpu: dimension 2 or 3 only");
        }
        for (typename gsMultiPatch<T>::const_iiterator it = mp.iBegin(); it != mp.iEnd(); ++it) {
            // the orientation of the side's own direction records whether the two sides sit at the
            // same parameter (gsBoundary.h:665-716); only the tangential directions must be kept
            const index_t nd = it->first().direction();
            for (index_t i = 0; i < it->dirMap().size(); ++i) {
                if (it->dirMap()(i) != i) throw std::invalid_argument("gsgpu: permuted interface");
                if (i != nd && !it->dirOrientation()(i)) throw std::invalid_argument("gsgpu: re-oriented interface");
            }
            ifaces.push_back(it->first().patch);
            ifaces.push_back(it->first().side().index());
            ifaces.push_back(it->second().patch);
            ifaces.push_back(it->second().side().index());
        }
        dsides = dirichletSides;
        nsides = neumannSides;
        fields = f;
        prob = gsgpu_problem{};
        prob.dim = d;
        prob.npatches = int(mp.nPatches());
        prob.degree = degree.data(); prob.nknots = nknots.data(); prob.knots = knots.data();
        prob.gdegree = gdegree.data(); prob.gnknots = gnknots.data(); prob.gknots = gknots.data();
        prob.coefs = coefs.data();
        prob.ninterfaces = int(ifaces.size() / 4); prob.interfaces = ifaces.data();
        prob.ndirichlet = int(dsides.size() / 2); prob.dirichlet = dsides.data();
        prob.kappa_fourier = fields.kappaFourier ? 1 : 0;
        prob.kappa_const = fields.kappaConst; prob.kappa_alpha = fields.kappaAlpha; prob.kappa_scale = fields.kappaScale;
        prob.kappa_nmodes = int(fields.amp.size());
        prob.kappa_amp = fields.amp.data(); prob.kappa_k = fields.waves.data(); prob.kappa_phase = fields.phase.data();
        prob.ufreq = fields.ufreq;
        prob.quA = quA;
        prob.quB = quB;
        prob.dirichlet_strategy = dirichletStrategy;
        prob.nneumann = int(nsides.size() / 2); prob.neumann = nsides.data();
    }

private:
    template <short_t D>
    void packPatch(const gsMultiPatch<T>& mp, const gsMultiBasis<T>& mb, index_t k) {
        const gsTensorBSplineBasis<D, T>* db = dynamic_cast<const gsTensorBSplineBasis<D, T>*>(&mb[k]);
        const gsTensorBSpline<D, T>* geo = dynamic_cast<const gsTensorBSpline<D, T>*>(&mp.patch(k));
        if (!db || !geo) throw std::invalid_argument("gsgpu: tensor B-spline patches and bases only");
        for (short_t i = 0; i < 3; ++i) {
            if (i < D) {
                const gsKnotVector<T>& kv = db->knots(i);
                degree.push_back(kv.degree());
                nknots.push_back(index_t(kv.size()));
                knots.insert(knots.end(), kv.begin(), kv.end());
                const gsKnotVector<T>& gk = geo->basis().knots(i);
                gdegree.push_back(gk.degree());
                gnknots.push_back(index_t(gk.size()));
                gknots.insert(gknots.end(), gk.begin(), gk.end());
            } else {
                degree.push_back(0); nknots.push_back(0); gdegree.push_back(0); gnknots.push_back(0);
            }
        }
        const gsMatrix<T>& c = geo->coefs();
        for (index_t r = 0; r < c.rows(); ++r)
            for (index_t m = 0; m < c.cols(); ++m) coefs.push_back(c(r, m));
    }
};

template <class T = real_t>
class gsGpuPoissonAssembler : public gsPoissonAssembler<T> {
public:
    typedef gsPoissonAssembler<T> Base;

    gsGpuPoissonAssembler(const gsMultiPatch<T>& patches, const gsMultiBasis<T>& basis,
                          const gsBoundaryConditions<T>& bconditions, const gsFunction<T>& rhs,
                          const gsGpuFields& fields, int device = 0)
        : Base(patches, basis, bconditions, rhs, dirichlet::elimination, iFace::glue), m_sys(device), m_fields(fields) {
        upload();
    }

    /// gsAssembler::refresh(): dof map, sparsity pattern and device buffers
    void refresh() override {
        Base::refresh();
        if (m_ready) upload();
    }

    /// gsPoissonAssembler::assemble() on the device: the rhs and the eliminated-dof values come back
    /// at once, the matrix on first access (matrix())
    void assemble() override {
        m_sys.assemble(GSGPU_PREC_FP64);
        const gsgpu::Sizes sz = m_sys.sizes();
        gsMatrix<T>& b = this->m_system.rhs();
        b.resize(sz.nfree, 1);
        readInto(b.data(), sz.nfree, [&](double* p) { m_sys.rhs(p); });
        this->m_ddof.resize(1);
        this->m_ddof[0].resize(sz.nfixed, 1);
        if (sz.nfixed) readInto(this->m_ddof[0].data(), sz.nfixed, [&](double* p) { m_sys.fixedDofs(p); });
        m_matrixStale = true;
    }

    /// gsAssembler::matrix(), materialised from the device on the first access after assemble()
    const gsSparseMatrix<T>& matrix() const {
        if (m_matrixStale) const_cast<gsGpuPoissonAssembler*>(this)->materializeMatrix();
        return Base::matrix();
    }
    const gsMatrix<T>& rhs() const { return Base::rhs(); }
    const gsMatrix<T>& fixedDofs(short_t unk = 0) const { return Base::fixedDofs(unk); }

    /// CG (+ Jacobi) on the device-resident system (gsConjugateGradient(matrix(), gsJacobiOp))
    int solve(gsMatrix<T>& x, double tol = 1e-10, int maxIter = 1000) {
        gsgpu_solver_opts o = {GSGPU_SOLVER_CG_JACOBI, GSGPU_PREC_FP64, tol, maxIter, 4, 2, 2, 0.6, 1e-4, 1, 1.0};
        return run(o, x);
    }

    /// gsConjugateGradient(matrix(), gsJacobiOp | gsMultiGridOp).setOptions(opt).solve(rhs(), x) on
    /// the device, with G+Smo's option names: "Tolerance", "MaxIterations" (gsIterativeSolver.h:92-99),
    /// "Preconditioner" ("Jacobi" or "MultiGrid"), the multigrid's "Levels" (gsGridHierarchy),
    /// "NumPreSmooth", "NumPostSmooth", "NumCycles", "CoarseGridCorrectionDamping"
    /// (gsMultiGrid.hpp:299-328) and the smoother's "Damping" (gsJacobiOp), plus "Precision" ("fp64" or "mixed": re-assembles the double-float operator on
    /// the device; matrix() keeps the FP64 system). Returns the iteration count; error() gives the
    /// final relative residual as gsIterativeSolver::error() does.
    int solve(const gsOptionList& opt, gsMatrix<T>& x) {
        gsgpu_solver_opts o = {};
        o.method = opt.askString("Preconditioner", "Jacobi") == "MultiGrid" ? GSGPU_SOLVER_CG_MG : GSGPU_SOLVER_CG_JACOBI;
        o.precision = opt.askString("Precision", "fp64") == "mixed" ? GSGPU_PREC_MIXED : GSGPU_PREC_FP64;
        o.tol = opt.askReal("Tolerance", 1e-10);
        o.max_iters = opt.askInt("MaxIterations", 1000);
        o.mg_levels = opt.askInt("Levels", 4);
        o.mg_npre = opt.askInt("NumPreSmooth", 2);
        o.mg_npost = opt.askInt("NumPostSmooth", 2);
        o.mg_damping = opt.askReal("Damping", 0.6);
        o.mg_cycles = opt.askInt("NumCycles", 1);
        o.mg_cgc_damping = opt.askReal("CoarseGridCorrectionDamping", 1.0);
        o.inner_tol = 1e-4;
        if (o.precision == GSGPU_PREC_MIXED) {
            if (m_matrixStale) materializeMatrix();  // matrix() keeps the FP64 system
            m_sys.assemble(GSGPU_PREC_MIXED);
        }
        const int its = run(o, x);
        if (o.precision == GSGPU_PREC_MIXED) m_sys.assemble(GSGPU_PREC_FP64);
        return its;
    }

    /// relative residual of the last solve (gsIterativeSolver::error())
    double error() const { return m_error; }

    /// gsField::distanceL2 of the last device solution against the manufactured solution
    double distanceL2() const { return m_sys.l2Error(); }

    /// gsField::distanceH1 (H1 seminorm of the error) of the last device solution
    double distanceH1() const { return m_sys.h1Error(); }

    gsgpu_context* context() const { return m_sys.context(); }

private:
    int run(const gsgpu_solver_opts& o, gsMatrix<T>& x) {
        gsgpu_solve_info info;
        x.resize(this->numDofs(), 1);
        readInto(x.data(), int(x.rows()), [&](double* p) { m_sys.solve(o, p, &info); });
        m_error = info.relres;
        return info.iterations;
    }

    // a device read into T storage (directly when T is double)
    template <class F>
    static void readInto(double* out, int, F&& read) { read(out); }
    template <class U, class F>
    static void readInto(U* out, int n, F&& read) {
        std::vector<double> tmp(size_t(n > 0 ? n : 0));
        read(tmp.data());
        for (int i = 0; i < n; ++i) out[i] = U(tmp[size_t(i)]);
    }

    // the compressed ColMajor storage of m_system's matrix filled with one copy of the device CSR
    // arrays (the system is symmetric: the CSR row arrays are the column arrays)
    void materializeMatrix() {
        const gsgpu::Sizes sz = m_sys.sizes();
        gsSparseMatrix<T>& K = this->m_system.matrix();
        K.resize(sz.nfree, sz.nfree);
        K.resizeNonZeros(index_t(sz.nnz));
        fillCompressed(K.outerIndexPtr(), K.innerIndexPtr(), K.valuePtr(), sz);
        m_matrixStale = false;
    }
    void fillCompressed(int* outer, int* inner, double* values, const gsgpu::Sizes&) { m_sys.csrInto(outer, inner, values); }
    template <class I, class U>
    void fillCompressed(I* outer, I* inner, U* values, const gsgpu::Sizes& sz) {
        std::vector<int> p(static_cast<size_t>(sz.nfree) + 1), c(static_cast<size_t>(sz.nnz));
        std::vector<double> v(static_cast<size_t>(sz.nnz));
        m_sys.csr(p.data(), c.data(), v.data());
        for (size_t i = 0; i < p.size(); ++i) outer[i] = I(p[i]);
        for (size_t i = 0; i < c.size(); ++i) inner[i] = I(c[i]), values[i] = U(v[i]);
    }

    // the caller's functions against the device closed forms, at points of every patch (rhs) and of
    // every Dirichlet / Neumann side (u / the flux kappa grad u . n)
    void checkFunctions(const std::vector<int>& dsides, const std::vector<int>& nsides) const {
        const gsMultiPatch<T>& mp = this->patches();
        const short_t d = mp.parDim();
        const T tcs[3] = {T(0.17), T(0.5), T(0.83)};
        auto params = [&](int fixdir, T fixval) {  // 3^(d-1) or 3^d parametric points
            std::vector<gsVector<T> > pts;
            const int m = fixdir < 0 ? d : d - 1;
            int count = 1;
            for (int i = 0; i < m; ++i) count *= 3;
            for (int c = 0; c < count; ++c) {
                gsVector<T> u(d);
                int r = c;
                for (int i = 0, j = 0; i < d; ++i) {
                    if (i == fixdir) { u[i] = fixval; continue; }
                    u[i] = tcs[r % 3];
                    r /= 3;
                    ++j;
                }
                pts.push_back(u);
            }
            return pts;
        };
        auto compare = [&](const gsFunctionSet<T>& fn, bool parametric, index_t patch, int fixdir, T fixval, int what,
                           int side) {
            const gsGeometry<T>& G = mp.patch(patch);
            const std::vector<gsVector<T> > us = params(fixdir, fixval);
            gsMatrix<T> u(d, index_t(us.size()));
            for (size_t i = 0; i < us.size(); ++i) u.col(index_t(i)) = us[i];
            gsMatrix<T> x, got;
            G.eval_into(u, x);
            fn.eval_into(parametric ? u : x, got);  // a parametric condition takes the parameters
            const int n = int(x.cols());
            std::vector<double> xs(static_cast<size_t>(n) * d), kap(static_cast<size_t>(n)), ff(static_cast<size_t>(n)),
                uu(static_cast<size_t>(n));
            for (int i = 0; i < n; ++i)
                for (int k = 0; k < d; ++k) xs[size_t(i) * d + k] = double(x(k, i));
            gsgpu::evalFields(m_pack.prob, n, xs.data(), kap.data(), ff.data(), uu.data());
            for (int i = 0; i < n; ++i) {
                double want = what == 0 ? ff[size_t(i)] : uu[size_t(i)];
                if (what == 2) {  // flux sgn kappa du/dx_k on side s of direction k = (s-1)/2
                    const int k = (side - 1) / 2;
                    const double w = m_fields.ufreq * 3.14159265358979323846;
                    double g = w * std::cos(w * xs[size_t(i) * d + k]);
                    for (int j = 0; j < d; ++j)
                        if (j != k) g *= std::sin(w * xs[size_t(i) * d + j]);
                    want = ((side - 1) % 2 ? 1.0 : -1.0) * kap[size_t(i)] * g;
                }
                const double have = double(got(0, i));
                if (std::abs(have - want) > 1e-8 * std::max(1.0, std::abs(want)))
                    throw std::invalid_argument(
                        std::string("gsGpuPoissonAssembler: the caller's ") +
                        (what == 0 ? "rhs function" : what == 1 ? "Dirichlet function" : "Neumann function") +
                        " differs from the device's closed form (gsGpuFields) on patch " + std::to_string(patch) +
                        ": " + std::to_string(have) + " vs " + std::to_string(want));
            }
        };
        if (const gsFunctionSet<T>* f = static_cast<const gsPoissonPde<T>&>(this->pde()).rhs())
            for (index_t k = 0; k < index_t(mp.nPatches()); ++k) compare(*f, false, k, -1, T(0), 0, 0);
        const gsBoundaryConditions<T>& bc = this->pde().bc();
        for (typename gsBoundaryConditions<T>::const_iterator it = bc.dirichletBegin(); it != bc.dirichletEnd(); ++it)
            if (it->function())
                compare(*it->function(), it->parametric(), it->patch(), it->side().direction(), T(it->side().parameter()),
                        1, it->side().index());
        for (typename gsBoundaryConditions<T>::const_iterator it = bc.neumannBegin(); it != bc.neumannEnd(); ++it)
            if (it->function())
                compare(*it->function(), it->parametric(), it->patch(), it->side().direction(), T(it->side().parameter()),
                        2, it->side().index());
        (void)dsides;
        (void)nsides;
    }

    void upload() {
        std::vector<int> dsides;
        const gsBoundaryConditions<T>& bc = this->pde().bc();
        for (typename gsBoundaryConditions<T>::const_iterator it = bc.dirichletBegin(); it != bc.dirichletEnd(); ++it) {
            dsides.push_back(it->patch());
            dsides.push_back(it->side().index());
        }
        // Neumann sides (gsPoissonAssembler.hpp:59): their data is the closed-form flux
        // sgn kappa du/dx_k of the device fields
        std::vector<int> nsides;
        for (typename gsBoundaryConditions<T>::const_iterator it = bc.neumannBegin(); it != bc.neumannEnd(); ++it) {
            nsides.push_back(it->patch());
            nsides.push_back(it->side().index());
        }
        // "DirichletValues": interpolation or L2 projection (gsAssembler.hpp:34, 231-534)
        const index_t dv = this->m_options.getInt("DirichletValues");
        if (dv != dirichlet::interpolation && dv != dirichlet::l2Projection)
            throw std::invalid_argument("gsGpuPoissonAssembler: DirichletValues must be interpolation or l2Projection");
        m_pack.pack(this->patches(), this->m_bases[0], dsides, m_fields, this->m_options.getReal("quA"),
                    this->m_options.getInt("quB"),
                    dv == dirichlet::l2Projection ? GSGPU_DIRICHLET_L2 : GSGPU_DIRICHLET_INTERPOLATION, nsides);
        checkFunctions(dsides, nsides);
        m_sys.setProblem(m_pack.prob);
        m_sys.refresh();
        m_ready = true;
        m_matrixStale = false;
    }

    gsgpu::System m_sys;
    double m_error = 0.0;
    gsGpuFields m_fields;
    gsGpuProblemPack<T> m_pack;
    bool m_ready = false;
    bool m_matrixStale = false;
};

/// The assembled device matrix as a gsLinearOperator (gsMatrixOp semantics: x = K input, column
/// by column), so G+Smo's own solvers can run on the GPU operator
template <class T = real_t>
class gsGpuMatrixOp : public gsLinearOperator<T> {
public:
    explicit gsGpuMatrixOp(const gsGpuPoissonAssembler<T>& A) : m_ctx(A.context()), m_n(A.numDofs()) {}
    void apply(const gsMatrix<T>& input, gsMatrix<T>& x) const override {
        x.resize(m_n, input.cols());
        for (index_t c = 0; c < input.cols(); ++c) {
            gsMatrix<T> in = input.col(c), out(m_n, 1);
            if (gsgpu_apply(m_ctx, in.data(), out.data()) != GSGPU_OK)
                throw std::runtime_error(std::string("gsgpu: ") + gsgpu_last_error(m_ctx));
            x.col(c) = out;
        }
    }
    index_t rows() const override { return m_n; }
    index_t cols() const override { return m_n; }

private:
    gsgpu_context* m_ctx;
    index_t m_n;
};

/// gsMultiGridOp as a preconditioner on the device (gsPreconditionerOp::apply: one cycle from a
/// zero start, gsMultiGrid.hpp:147-201); setOptions takes "Levels", "NumPreSmooth",
/// "NumPostSmooth", "NumCycles", "CoarseGridCorrectionDamping" and "Damping". "SymmSmooth" needs
/// no setting: the damped Jacobi step is its own transpose, so step and stepT coincide
template <class T = real_t>
class gsGpuMultiGridOp : public gsLinearOperator<T> {
public:
    explicit gsGpuMultiGridOp(const gsGpuPoissonAssembler<T>& A) : m_ctx(A.context()), m_n(A.numDofs()) {
        m_opts = {GSGPU_SOLVER_CG_MG, GSGPU_PREC_FP64, 0.0, 0, 4, 2, 2, 0.6, 0.0, 1, 1.0};
    }
    void setOptions(const gsOptionList& opt) override {
        m_opts.mg_levels = opt.askInt("Levels", m_opts.mg_levels);
        m_opts.mg_npre = opt.askInt("NumPreSmooth", m_opts.mg_npre);
        m_opts.mg_npost = opt.askInt("NumPostSmooth", m_opts.mg_npost);
        m_opts.mg_damping = opt.askReal("Damping", m_opts.mg_damping);
        m_opts.mg_cycles = opt.askInt("NumCycles", m_opts.mg_cycles);
        m_opts.mg_cgc_damping = opt.askReal("CoarseGridCorrectionDamping", m_opts.mg_cgc_damping);
    }
    void apply(const gsMatrix<T>& input, gsMatrix<T>& x) const override {
        x.resize(m_n, input.cols());
        for (index_t c = 0; c < input.cols(); ++c) {
            gsMatrix<T> in = input.col(c), out(m_n, 1);
            if (gsgpu_mg_apply(m_ctx, &m_opts, in.data(), out.data()) != GSGPU_OK)
                throw std::runtime_error(std::string("gsgpu: ") + gsgpu_last_error(m_ctx));
            x.col(c) = out;
        }
    }
    index_t rows() const override { return m_n; }
    index_t cols() const override { return m_n; }

private:
    gsgpu_context* m_ctx;
    index_t m_n;
    gsgpu_solver_opts m_opts;
};

}  // namespace gismo
