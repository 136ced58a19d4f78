/* gsgpu.hpp: header-only C++ layer over the C ABI of libgsgpu (include/gsgpu.h), with no G+Smo
 * dependency. gsgpu::System owns one context (device memory, stream) and turns status codes into
 * exceptions; the G+Smo drop-ins (gsGpuPoissonAssembler.h, gsGpuExprAssembler.h) are built on it,
 * and code that is not a G+Smo build can use it directly.
 *
 *   gsgpu::System S(0);                 // a context on CUDA device 0
 *   S.setProblem(prob);                 // gsgpu_problem, copied
 *   S.refresh(); S.assemble();
 *   S.csr(ptr, col, val);               // caller-sized arrays (sizes() first), or
 *   S.csrInto(outer, inner, values);    // straight into compressed-matrix storage
 *   S.solve(opts, x, &info);
 */
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

#include "gsgpu.h"

namespace gsgpu {

/* a failed libgsgpu call: the status code (GSGPU_ERR_*) and the context's message */
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error("gsgpu error " + std::to_string(c) + ": " + m), code(c) {}
};

struct Sizes {
    int nfree = 0, nfixed = 0, nlocal = 0;
    long long nnz = 0;
};

class System {
public:
    explicit System(int device = 0) {
        const int rc = gsgpu_create(&m_ctx, device);
        if (rc != GSGPU_OK) throw Error(rc, "could not create a context on CUDA device " + std::to_string(device));
    }
    ~System() {
        if (m_ctx) gsgpu_destroy(m_ctx);
    }
    System(const System&) = delete;
    System& operator=(const System&) = delete;

    gsgpu_context* context() const { return m_ctx; }

    void setProblem(const gsgpu_problem& p) { check(gsgpu_set_problem(m_ctx, &p)); }
    void refresh() { check(gsgpu_refresh(m_ctx)); }
    void assemble(int precision = GSGPU_PREC_FP64) { check(gsgpu_assemble(m_ctx, precision)); }
    void setCoefs(const double* coefs) { check(gsgpu_set_coefs(m_ctx, coefs)); }

    Sizes sizes() const {
        Sizes s;
        check(gsgpu_sizes(m_ctx, &s.nfree, &s.nnz, &s.nfixed, &s.nlocal));
        return s;
    }
    /* the CSR arrays (nfree + 1, nnz, nnz entries; any may be NULL) */
    void csr(int* ptr, int* col, double* val) const { check(gsgpu_matrix_csr(m_ctx, ptr, col, val)); }
    /* the same arrays, read straight into the storage of a compressed ColMajor matrix of the
     * symmetric system (outer = column pointers, inner = row indices): no per-entry insertion */
    void csrInto(int* outer, int* inner, double* values) const { csr(outer, inner, values); }
    void rhs(double* b) const { check(gsgpu_rhs(m_ctx, b)); }
    void fixedDofs(double* d) const { check(gsgpu_fixed_dofs(m_ctx, d)); }
    void dofMap(int* index) const { check(gsgpu_dof_map(m_ctx, index)); }

    /* CG + Jacobi / multigrid on the device; x receives the solution (NULL: it stays on the device).
     * Returns the status: GSGPU_OK or GSGPU_ERR_NOT_CONVERGED (other codes throw) */
    int solve(const gsgpu_solver_opts& o, double* x, gsgpu_solve_info* info = nullptr) {
        gsgpu_solve_info local;
        const int rc = gsgpu_solve(m_ctx, &o, x, info ? info : &local);
        if (rc != GSGPU_OK && rc != GSGPU_ERR_NOT_CONVERGED) check(rc);
        return rc;
    }
    void apply(const double* x, double* y) const { check(gsgpu_apply(m_ctx, x, y)); }
    void mgApply(const gsgpu_solver_opts& o, const double* r, double* z) const { check(gsgpu_mg_apply(m_ctx, &o, r, z)); }
    double l2Error() const {
        double e = 0.0;
        check(gsgpu_l2_error(m_ctx, &e));
        return e;
    }
    double h1Error() const {
        double e = 0.0;
        check(gsgpu_h1_error(m_ctx, &e));
        return e;
    }
    void setFixedDofs(const double* d, int n) { check(gsgpu_set_fixed_dofs(m_ctx, d, n)); }

    void check(int rc) const {
        if (rc != GSGPU_OK) throw Error(rc, m_ctx ? gsgpu_last_error(m_ctx) : "no context");
    }

private:
    gsgpu_context* m_ctx = nullptr;
};

/* The closed-form fields of a problem (coefficient kappa, source f, exact solution u, and the
 * outward flux kappa grad u . n on box sides) at physical points x (npts x dim, row-major): what
 * the device evaluates. Used to check that a caller's own functions are the ones the device
 * computes with. */
inline void evalFields(const gsgpu_problem& p, int npts, const double* x, double* kappa, double* f, double* u) {
    const int rc = gsgpu_eval_fields(&p, npts, x, kappa, f, u);
    if (rc != GSGPU_OK) throw Error(rc, "invalid problem fields");
}

}  // namespace gsgpu
