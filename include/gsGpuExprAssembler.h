/** gsGpuExprAssembler: drop-in for gismo::gsExprAssembler (src/gsAssembler/gsExprAssembler.h:85-381)
 *  that assembles the Poisson / diffusion expression pair on a GB300 through libgsgpu.
 *
 *  It is a gsExprAssembler (getMap, getSpace, getCoeff, getSolution, options, gsExprEvaluator all
 *  work as before) whose assemble(lhs, rhs) recognises, by expression type,
 *
 *      igrad(u, G) * igrad(u, G).tr() * meas(G)              (kappa = 1)
 *      igrad(u, G) * K * igrad(u, G).tr() * meas(G)          (K = getCoeff(kappa, G))
 *      u * ff * meas(G)                                      (ff = getCoeff(f, G) or getCoeff(f))
 *
 *  and runs them on the device (gsExprAssembler.h:754-833 and _eval::push :553-630 on the host in
 *  the reference). Any other expression, and every assembleBdr / assembleIfc with terms, throws:
 *  there is no CPU fallback.
 *
 *  The space must be set up by the caller as in G+Smo, u.setup(bc, dirichlet::interpolation or
 *  dirichlet::l2Projection, 0) (gsExpressions.h:1091-1212): the eliminated dofs and their values
 *  (u.fixedPart()) are taken from it, so both Dirichlet strategies give the reference's lift; the
 *  Dirichlet sides are the sides whose dofs the space eliminates, and its dof map must equal the
 *  device's (gsgpu_dof_map). As with gsGpuPoissonAssembler, the device evaluates closed forms: the
 *  coefficient kappa and the source f come from setFields (gsGpuFields); the gsFunctions given to
 *  getCoeff stay on the host. With the kappa-free left-hand side the device uses kappa = 1.
 *
 *  initSystem() builds the device problem (no host matrix reservation); matrix(), rhs() and
 *  numDofs() return the device-assembled system (full symmetric matrix, compressed ColMajor,
 *  explicit zeros kept where the reference's expression push skips exact-zero local entries).
 */
#pragma once

#include <gsAssembler/gsExprAssembler.h>

#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "gsGpuPoissonAssembler.h"
#include "gsgpu.h"

namespace gismo {

namespace gsgpu_expr {
// an expression type without the _expr<E, bool> base it may come wrapped in
template <class E> struct unwrap { typedef E type; };
template <class E, bool B> struct unwrap<expr::_expr<E, B> > { typedef E type; };
template <class A, class B>
struct same : std::is_same<typename unwrap<typename std::decay<A>::type>::type,
                           typename unwrap<typename std::decay<B>::type>::type> {};

// the expression types of the recognised pair, built on the handles a gsExprAssembler hands out
template <class T>
struct poisson {
    typedef const expr::gsFeSpace<T>& S;
    typedef const expr::gsGeometryMap<T>& G;
    typedef expr::gsComposition<T>& C;
    typedef const expr::gsFeVariable<T>& V;
    typedef decltype(igrad(std::declval<S>(), std::declval<G>()) * igrad(std::declval<S>(), std::declval<G>()).tr() *
                     meas(std::declval<G>())) lhs;
    typedef decltype(igrad(std::declval<S>(), std::declval<G>()) * std::declval<C>() *
                     igrad(std::declval<S>(), std::declval<G>()).tr() * meas(std::declval<G>())) lhs_kappa;
    typedef decltype(std::declval<S>() * std::declval<C>() * meas(std::declval<G>())) rhs_coeff;
    typedef decltype(std::declval<S>() * std::declval<V>() * meas(std::declval<G>())) rhs_var;
};
}  // namespace gsgpu_expr

template <class T = real_t>
class gsGpuExprAssembler : public gsExprAssembler<T> {
public:
    typedef gsExprAssembler<T> Base;
    typedef typename Base::geometryMap geometryMap;
    typedef typename Base::space space;
    typedef typename Base::variable variable;

    explicit gsGpuExprAssembler(index_t rBlocks = 1, index_t cBlocks = 1, int device = 0) : Base(rBlocks, cBlocks) {
        if (rBlocks != 1 || cBlocks != 1) throw std::invalid_argument("gsGpuExprAssembler: one scalar space only");
        check(gsgpu_create(&m_ctx, device));
    }
    ~gsGpuExprAssembler() {
        if (m_ctx) gsgpu_destroy(m_ctx);
    }
    gsGpuExprAssembler(const gsGpuExprAssembler&) = delete;
    gsGpuExprAssembler& operator=(const gsGpuExprAssembler&) = delete;

    /// closed-form coefficient and source for the device (see gsGpuFields)
    void setFields(const gsGpuFields& f) { m_fields = f; }

    /// gsExprAssembler::getMap, remembering the patches
    geometryMap getMap(const gsFunctionSet<T>& g) {
        m_patches = dynamic_cast<const gsMultiPatch<T>*>(&g);
        return Base::getMap(g);
    }

    /// gsExprAssembler::getSpace, remembering the basis and the space handle
    space getSpace(const gsFunctionSet<T>& mb, index_t dim = 1, index_t id = 0) {
        if (dim != 1 || id != 0) throw std::invalid_argument("gsGpuExprAssembler: one scalar space only");
        m_basis = dynamic_cast<const gsMultiBasis<T>*>(&mb);
        space s = Base::getSpace(mb, dim, id);
        m_space.assign(1, s);
        return s;
    }

    /// gsExprAssembler::initSystem: the device problem, its dof map checked against the space's,
    /// and the space's eliminated-dof values
    void initSystem(const index_t numRhs = 1) {
        if (numRhs != 1) throw std::invalid_argument("gsGpuExprAssembler: one right-hand side");
        if (!m_patches || !m_basis || m_space.empty())
            throw std::logic_error("gsGpuExprAssembler: getMap(gsMultiPatch) and getSpace(gsMultiBasis) first");
        const gsDofMapper& map = m_space[0].mapper();
        if (!map.isFinalized()) throw std::logic_error("gsGpuExprAssembler: set up the space (u.setup) first");
        // Dirichlet sides: the sides whose dofs the space eliminates
        std::vector<int> dsides;
        const short_t d = m_patches->parDim();
        for (size_t k = 0; k < m_basis->nBases(); ++k)
            for (int s = 1; s <= 2 * d; ++s) {
                const gsMatrix<index_t> bnd = (*m_basis)[k].boundary(boxSide(s));
                bool all = bnd.size() > 0;
                for (index_t i = 0; i < bnd.size() && all; ++i) all = map.is_boundary(bnd(i), index_t(k));
                if (all) {
                    dsides.push_back(int(k));
                    dsides.push_back(s);
                }
            }
        m_pack.pack(*m_patches, *m_basis, dsides, m_fields, this->options().askReal("quA", 1.0),
                    this->options().askInt("quB", 1));
        check(gsgpu_set_problem(m_ctx, &m_pack.prob));
        check(gsgpu_refresh(m_ctx));
        int n = 0, nb = 0, nl = 0;
        long long nnz = 0;
        check(gsgpu_sizes(m_ctx, &n, &nnz, &nb, &nl));
        std::vector<int> dev(nl);
        check(gsgpu_dof_map(m_ctx, dev.data()));
        const gsVector<index_t> ref = map.asVector();
        if (index_t(dev.size()) != ref.size() || n != map.freeSize() || nb != map.boundarySize())
            throw std::runtime_error("gsGpuExprAssembler: the space's dof map is not the device's");
        for (size_t i = 0; i < dev.size(); ++i)
            if (dev[i] != ref[index_t(i)]) throw std::runtime_error("gsGpuExprAssembler: the space's dof map is not the device's");
        const gsMatrix<T>& fixed = m_space[0].fixedPart();
        std::vector<double> g(nb);
        for (int i = 0; i < nb; ++i) g[i] = i < fixed.rows() ? double(fixed(i, 0)) : 0.0;
        check(gsgpu_set_fixed_dofs(m_ctx, g.data(), nb));
        m_n = n;
        m_ready = true;
    }

    /// the recognised Poisson / diffusion pair on the device
    template <class E1, class E2>
    void assemble(const E1& lhs, const E2& rhs) {
        typedef gsgpu_expr::poisson<T> P;
        const bool plain = gsgpu_expr::same<E1, typename P::lhs>::value;
        const bool kappa = gsgpu_expr::same<E1, typename P::lhs_kappa>::value;
        const bool source = gsgpu_expr::same<E2, typename P::rhs_coeff>::value || gsgpu_expr::same<E2, typename P::rhs_var>::value;
        (void)lhs;
        (void)rhs;
        if (!(plain || kappa) || !source)
            throw std::runtime_error("gsGpuExprAssembler: only igrad(u,G)*[K*]igrad(u,G).tr()*meas(G) with u*ff*meas(G) runs on the GPU");
        if (!m_ready) throw std::logic_error("gsGpuExprAssembler: initSystem() first");
        if (plain && (m_fields.kappaFourier || m_fields.kappaConst != 1.0)) {
            // the kappa-free form integrates with kappa = 1
            gsGpuFields f = m_fields;
            f.kappaFourier = false;
            f.kappaConst = 1.0;
            f.amp.clear(); f.phase.clear(); f.waves.clear();
            std::swap(f, m_fields);
            initSystem();
            std::swap(f, m_fields);
        }
        check(gsgpu_assemble(m_ctx, GSGPU_PREC_FP64));
        download();
    }

    /// any other expression list: not on the GPU
    template <class... E>
    void assemble(const E&...) {
        throw std::runtime_error("gsGpuExprAssembler: only the Poisson / diffusion pair runs on the GPU");
    }

    /// boundary and interface integrals: none are supported (Neumann terms throw)
    template <class... E>
    void assembleBdr(const typename Base::bcRefList& BCs, E&...) {
        if (!BCs.empty()) throw std::runtime_error("gsGpuExprAssembler: boundary integrals are not on the GPU");
    }
    template <class... E>
    void assembleIfc(const typename Base::ifContainer& ifc, E...) {
        if (!ifc.empty()) throw std::runtime_error("gsGpuExprAssembler: interface integrals are not on the GPU");
    }

    const gsSparseMatrix<T>& matrix() const { return m_matrix; }
    const gsMatrix<T>& rhs() const { return m_rhs; }
    index_t numDofs() const { return m_n; }
    gsgpu_context* context() const { return m_ctx; }

private:
    void check(int rc) const {
        if (rc != GSGPU_OK)
            throw std::runtime_error(std::string("gsgpu: ") + (m_ctx ? gsgpu_last_error(m_ctx) : "no context"));
    }

    void download() {
        int n = 0, nb = 0, nl = 0;
        long long nnz = 0;
        check(gsgpu_sizes(m_ctx, &n, &nnz, &nb, &nl));
        // symmetric: the CSR arrays are the compressed ColMajor arrays, copied straight into the
        // matrix's storage (no per-entry insertion)
        m_matrix.resize(n, n);
        m_matrix.resizeNonZeros(index_t(nnz));
        fillCompressed(m_matrix.outerIndexPtr(), m_matrix.innerIndexPtr(), m_matrix.valuePtr(), n, nnz);
        std::vector<double> b(n);
        check(gsgpu_rhs(m_ctx, b.data()));
        m_rhs.resize(n, 1);
        for (int i = 0; i < n; ++i) m_rhs(i, 0) = b[i];
    }
    void fillCompressed(int* outer, int* inner, double* values, int, long long) {
        check(gsgpu_matrix_csr(m_ctx, outer, inner, values));
    }
    template <class I, class U>
    void fillCompressed(I* outer, I* inner, U* values, int n, long long nnz) {
        std::vector<int> p(static_cast<size_t>(n) + 1), c(static_cast<size_t>(nnz));
        std::vector<double> v(static_cast<size_t>(nnz));
        check(gsgpu_matrix_csr(m_ctx, p.data(), c.data(), v.data()));
        for (size_t i = 0; i < p.size(); ++i) outer[i] = I(p[i]);
        for (size_t i = 0; i < c.size(); ++i) inner[i] = I(c[i]), values[i] = U(v[i]);
    }

    gsgpu_context* m_ctx = nullptr;
    gsGpuFields m_fields;
    gsGpuProblemPack<T> m_pack;
    const gsMultiPatch<T>* m_patches = nullptr;
    const gsMultiBasis<T>* m_basis = nullptr;
    std::vector<expr::gsFeSpace<T> > m_space;
    gsSparseMatrix<T> m_matrix;
    gsMatrix<T> m_rhs;
    index_t m_n = 0;
    bool m_ready = false;
};

}  // namespace gismo
