/* CPU oracle for the isogeometric Poisson / diffusion Galerkin path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain restatement of G+Smo's FP64 algorithm (element loop
 * with full local matrices, gsDofMapper numbering, Dirichlet elimination by interpolation,
 * gsConjugateGradient + gsJacobiOp, geometric multigrid) used as the parity checker by the tests,
 * by __graft_entry__.smoke() and by the CPU-baseline leg of bench.py. The GPU product never calls
 * it. Parity of this oracle with the reference itself is pinned by fixtures generated from the
 * reference's own sources (tests/golden/make_golden.py).
 */
#ifndef GSORACLE_H
#define GSORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int dim;                    /* 2 or 3 */
    int npatches;
    const int* degree;          /* npatches*3: discretisation degree per direction */
    const int* nknots;          /* npatches*3 */
    const double* knots;        /* all knot vectors, patch-major then direction */
    const int* gdegree;         /* geometry basis, same layout */
    const int* gnknots;
    const double* gknots;
    const double* coefs;        /* control points, patch-major, (ncoef x dim) row-major */
    int ninterfaces;
    const int* interfaces;      /* 4 per interface: patch1 side1 patch2 side2 */
    int ndirichlet;
    const int* dirichlet;       /* 2 per side: patch side */
    int kappa_fourier;
    double kappa_const, kappa_alpha, kappa_scale;
    int kappa_nmodes;
    const double* kappa_amp;
    const int* kappa_k;         /* 3 per mode */
    const double* kappa_phase;
    int ufreq;
    double quA;
    int quB;
    int dirichlet_l2;           /* 1: Dirichlet values by L2 projection, 0: by interpolation */
    int nneumann;
    const int* neumann;         /* 2 per side: patch side (condition_type::neumann) */
} orc_problem;

void* orc_create(const orc_problem* prob);
void orc_destroy(void* h);
/* Dof map + Dirichlet values + matrix/rhs, OpenMP over elements with a serialised scatter
 * (the reference's apply(): src/gsAssembler/gsAssembler.h:666-722). max_elements < 0 = all;
 * otherwise only the first max_elements elements (lexicographic over patches) are assembled,
 * which is how the bounded CPU baseline sample is taken. Returns elapsed seconds. */
double orc_assemble(void* h, int nthreads, long long max_elements);
void orc_sizes(void* h, int* nfree, long long* nnz, int* nbound, int* nlocal);
void orc_dofmap(void* h, int* out);             /* gsDofMapper::asVector, all patches */
void orc_csr(void* h, int* ptr, int* idx, double* val);
void orc_rhs(void* h, double* out);
void orc_ddof(void* h, double* out);
/* gsConjugateGradient + gsJacobiOp (damping 1): returns elapsed seconds */
double orc_solve_cg(void* h, double tol, int maxit, double* x, int* iters, double* relres);
/* CG preconditioned by gsMultiGridOp with damped Jacobi smoothing; cycles = NumCycles (1 = V, 2 = W),
 * cgc = CoarseGridCorrectionDamping */
double orc_solve_mg(void* h, double tol, int maxit, int levels, int npre, int npost, double damping,
                    int cycles, double cgc, double* x, int* iters, double* relres);
// gsGenericAssembler::assembleMass on the free dofs, in the CSR pattern of orc_csr (nnz values)
void orc_mass(void* h, double* val);
double orc_l2_error(void* h, const double* x);
/* gsField::distanceH1: H1 seminorm of u_h - u */
double orc_h1_error(void* h, const double* x);
/* the same norms (h1 = 0: L2, 1: H1 seminorm) with p + 1 Gauss points per direction, the rule
 * gsField::distanceL2/H1 integrate with whatever the assembler's quA/quB (gsExprEvaluator
 * defaults); orc_l2_error / orc_h1_error use the assembly rule, as the device does */
double orc_error_evaluator_rule(void* h, const double* x, int h1);
/* Gauss-Legendre rule on [-1,1] (ascending nodes) */
void orc_gauss(int n, double* nodes, double* weights);

#ifdef __cplusplus
}
#endif
#endif
