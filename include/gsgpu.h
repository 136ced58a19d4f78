/* gsgpu: GB300 (sm_103a) isogeometric Poisson / diffusion assembly and solve.
 *
 * C ABI of libgsgpu.so. Plain pointers and sizes only; every entry point returns a status code
 * (GSGPU_OK on success) and the message of the last failure is available from
 * gsgpu_last_error(). Each entry point names the G+Smo interface it replaces (paths relative to
 * the G+Smo source tree). A context owns all device memory of one problem; contexts are
 * independent and may be used from different host threads, one thread per context at a time
 * (G+Smo: one assembler object is not safe for concurrent assemble() calls either).
 */
#ifndef GSGPU_H
#define GSGPU_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (G+Smo reports failures as exceptions from GISMO_ENSURE / GISMO_ERROR,
 * src/gsCore/gsDebug.h:88-120; non-convergence is not an exception there either) */
#define GSGPU_OK 0
#define GSGPU_ERR_INVALID 1       /* invalid argument / unsupported input */
#define GSGPU_ERR_CUDA 2          /* CUDA runtime error */
#define GSGPU_ERR_BUDGET 3        /* device-memory budget exceeded */
#define GSGPU_ERR_NOT_CONVERGED 4 /* solver reached MaxIterations (solution still returned) */
#define GSGPU_ERR_JACOBIAN 5      /* geometry map has det J <= 0 at a quadrature point */
#define GSGPU_ERR_STATE 6         /* call out of order (e.g. matrix() before assemble()) */
#define GSGPU_ERR_TIMEOUT 7       /* a bounded device wait gave up */

typedef struct gsgpu_context gsgpu_context;

/* Problem description: what G+Smo receives as gsMultiPatch + gsMultiBasis +
 * gsBoundaryConditions + the PDE functions in the gsPoissonAssembler / gsCDRAssembler
 * constructors (src/gsAssembler/gsPoissonAssembler.h:93-106, gsCDRAssembler.h:113-125).
 * Patches are tensor-product B-spline maps (gsTensorBSpline, dim 2 or 3); the discretisation
 * basis of patch k is given by degree/knots, the geometry basis by gdegree/gknots.
 * Interfaces are conforming with identity orientation (the gsBoxTopology interfaces of
 * gsNurbsCreator::BSplineSquareGrid / BSplineCubeGrid), eliminated by gluing (iFace::glue).
 * Dirichlet sides are eliminated (dirichlet::elimination) with values by interpolation
 * (dirichlet::interpolation, gsAssembler.hpp:314-390) or L2 projection (dirichlet::l2Projection,
 * gsAssembler.hpp:392-534) of the exact solution u.
 * Neumann sides add the boundary integral of gsVisitorNeumann (gsPoissonAssembler.hpp:59,
 * gsCDRAssembler.hpp:58) to the load vector; the sides that are neither Dirichlet, Neumann nor
 * interface sides are natural (zero-flux) boundaries, as in the reference.
 * Coefficient, source, exact solution and Neumann data are closed forms evaluated on the device:
 *   g(x) = kappa_scale * sum_m kappa_amp[m] cos(pi kappa_k[m].x + kappa_phase[m])
 *   kappa = exp(kappa_alpha * g) if kappa_fourier else kappa_const
 *   u = prod_i sin(ufreq pi x_i),  f = -div(kappa grad u)
 *   Neumann data on side s of direction k = (s-1)/2: h(x) = sgn(s) kappa(x) du/dx_k(x),
 *   sgn = -1 on the lower side (s odd), +1 on the upper side: the flux kappa grad u . n of the
 *   manufactured solution wherever the side lies in a plane x_k = const. */
typedef struct {
    int dim;
    int npatches;
    const int* degree;     /* npatches*3 (unused directions: 0) */
    const int* nknots;     /* npatches*3 */
    const double* knots;   /* all knot vectors, patch-major then direction */
    const int* gdegree;
    const int* gnknots;
    const double* gknots;
    const double* coefs;   /* control points, patch-major, (ncoef x dim) row-major,
                              first parametric direction fastest (gsTensorBasis numbering) */
    int ninterfaces;
    const int* interfaces; /* 4 ints per interface: patch1 side1 patch2 side2 (boxSide numbers) */
    int ndirichlet;
    const int* dirichlet;  /* 2 ints per side: patch side */
    int kappa_fourier;
    double kappa_const, kappa_alpha, kappa_scale;
    int kappa_nmodes;
    const double* kappa_amp;
    const int* kappa_k;    /* 3 ints per mode, each in [0, 8] */
    const double* kappa_phase;
    int ufreq;
    double quA;            /* Gauss points per direction: quA * degree + quB (gsQuadrature.h:151-171) */
    int quB;
    int dirichlet_strategy; /* GSGPU_DIRICHLET_INTERPOLATION (0) or GSGPU_DIRICHLET_L2 (1): the
                               "DirichletValues" option, dirichlet::interpolation or
                               dirichlet::l2Projection (gsAssembler.hpp:231-534) */
    int nneumann;
    const int* neumann;    /* 2 ints per side: patch side (condition_type::neumann) */
} gsgpu_problem;
#define GSGPU_DIRICHLET_INTERPOLATION 0
#define GSGPU_DIRICHLET_L2 1

/* solver options (gsIterativeSolver::defaultOptions gsIterativeSolver.h:92-99,
 * gsMultiGridOp options gsMultiGrid.hpp:299-328, gsJacobiOp "Damping") */
#define GSGPU_SOLVER_CG_JACOBI 0
#define GSGPU_SOLVER_CG_MG 1
#define GSGPU_PREC_FP64 0   /* plain FP64 */
#define GSGPU_PREC_MIXED 1  /* FP32 inner iteration, FP64 residual / refinement */
typedef struct {
    int method;
    int precision;
    double tol;            /* relative residual ||r||/||b|| ("Tolerance", default 1e-10) */
    int max_iters;         /* "MaxIterations", default 1000 */
    int mg_levels;         /* "Levels" of gsGridHierarchy::buildByCoarsening */
    int mg_npre, mg_npost; /* "NumPreSmooth", "NumPostSmooth" */
    double mg_damping;     /* damping of the Jacobi smoother */
    double inner_tol;      /* unused (the mixed solves replace residuals instead of restarting) */
    int mg_cycles;         /* "NumCycles": 1 = V-cycle, 2 = W-cycle (0: 1) */
    double mg_cgc_damping; /* "CoarseGridCorrectionDamping" (0: 1) */
} gsgpu_solver_opts;

typedef struct {
    int iterations;        /* gsIterativeSolver::iterations() */
    double relres;         /* gsIterativeSolver::error(): final ||b - A x|| / ||b|| */
    int refinements;       /* mixed precision: outer FP64 residual evaluations */
    double t_solve_ms;     /* device time of the solve */
} gsgpu_solve_info;

/* lifetime. device >= 0: a CUDA device. device == -1: a host-only context that computes the
 * dof map, the sparsity pattern and the eliminated-dof values (set_problem, refresh, sizes,
 * dof_map, matrix_csr with val == NULL, fixed_dofs) and refuses every device call with
 * GSGPU_ERR_STATE. */
int gsgpu_create(gsgpu_context** ctx, int device);
int gsgpu_destroy(gsgpu_context* ctx);
const char* gsgpu_last_error(const gsgpu_context* ctx);

/* gsPoissonAssembler(patches, bases, bc, rhs) / gsCDRAssembler(..., coeff_A = kappa I, b = 0,
 * c = 0) constructors: copy the problem into the context (nothing is retained) */
int gsgpu_set_problem(gsgpu_context* ctx, const gsgpu_problem* prob);
/* gsAssembler::refresh() (gsPoissonAssembler.hpp:33-38, gsAssembler.hpp:101-122): dof mapper,
 * symbolic sparsity pattern, gather maps, device buffers */
int gsgpu_refresh(gsgpu_context* ctx);
/* replace the control points of all patches (same count and layout as in the problem) without
 * redoing refresh(); the next assemble() uses them (G+Smo: mutating gsMultiPatch::patch(k).coefs()) */
int gsgpu_set_coefs(gsgpu_context* ctx, const double* coefs);
/* gsPoissonAssembler::assemble() (gsPoissonAssembler.hpp:41-78): Dirichlet values, element
 * integrals, scatter into the CSR system. precision: GSGPU_PREC_FP64 assembles the FP64 system;
 * GSGPU_PREC_MIXED additionally keeps the FP32 inner operator used by the mixed solver. */
int gsgpu_assemble(gsgpu_context* ctx, int precision);

/* sizes: gsAssembler::numDofs() (gsAssembler.h:633-639), matrix().nonZeros(),
 * gsDofMapper::boundarySize(), total patch-local dofs */
int gsgpu_sizes(gsgpu_context* ctx, int* nfree, long long* nnz, int* nfixed, int* nlocal);
/* gsAssembler::matrix() (gsAssembler.h:614) as CSR (the matrix is symmetric, so these are also
 * the compressed ColMajor arrays outerIndexPtr / innerIndexPtr / valuePtr). Any of the three
 * pointers may be NULL; ptr/col are available after refresh(), val after assemble(). */
int gsgpu_matrix_csr(gsgpu_context* ctx, int* ptr, int* col, double* val);
/* gsGenericAssembler::assembleMass() (src/gsAssembler/gsGenericAssembler.h:103) with the
 * context's boundary conditions (gsGenericAssembler(patches, bases, opt, &bc)): the mass matrix
 * M_ij = int phi_i phi_j |det J| over all patches on the free dofs of the same dof map, in the
 * CSR pattern of gsgpu_matrix_csr (val: nnz values). Runs on the device in FP64; it reuses the
 * assembly's intermediate buffers, so it invalidates the last assemble() (assemble again before
 * matrix values, rhs or a solve are needed). */
int gsgpu_mass_csr(gsgpu_context* ctx, double* val);
/* gsAssembler::rhs() (gsAssembler.h:618) */
int gsgpu_rhs(gsgpu_context* ctx, double* rhs);
/* gsAssembler::fixedDofs() (gsAssembler.h:538); on a host-only context (device -1) computed on
 * the host after refresh() */
int gsgpu_fixed_dofs(gsgpu_context* ctx, double* ddof);
/* the eliminated-dof values (m_ddof, eliminated-dof order of gsgpu_fixed_dofs) computed by the
 * caller, e.g. gsFeSpace::setup's interpolation or L2 projection (gsExpressions.h:1091-1212,
 * gsAssembler::computeDirichletDofs gsAssembler.hpp:231-534), used by the following assembles
 * instead of the built-in interpolation; n = the eliminated-dof count. ddof == NULL restores the
 * built-in values. Cleared by set_problem. */
int gsgpu_set_fixed_dofs(gsgpu_context* ctx, const double* ddof, int n);
/* gsDofMapper::asVector() (gsDofMapper.cpp:80-87) over all patches */
int gsgpu_dof_map(gsgpu_context* ctx, int* index);

/* gsConjugateGradient(matrix, gsJacobiOp | gsMultiGridOp).solve(rhs, x)
 * (gsIterativeSolver.h:114-125, gsConjugateGradient.hpp:19-84). x: host array of nfree values
 * (may be NULL to keep the solution on the device only). */
int gsgpu_solve(gsgpu_context* ctx, const gsgpu_solver_opts* opts, double* x, gsgpu_solve_info* info);
/* gsMatrixOp::apply (gsMatrixOp.h:74-75) on the device: y = K x with the assembled FP64 matrix
 * (host arrays of nfree values), so that G+Smo's own solvers can run on the GPU operator */
int gsgpu_apply(gsgpu_context* ctx, const double* x, double* y);
/* gsMultiGridOp as a preconditioner (gsPreconditionerOp::apply, gsPreconditioner.h:79-84, and
 * multiGridStep, gsMultiGrid.hpp:147-201): z = one FP64 cycle on r from a zero start, with the
 * hierarchy, smoother and cycle options of opts (mg_levels, mg_npre, mg_npost, mg_damping,
 * mg_cycles, mg_cgc_damping) */
int gsgpu_mg_apply(gsgpu_context* ctx, const gsgpu_solver_opts* opts, const double* r, double* z);
/* gsField::distanceL2 of the last solution against u (gsField.hpp:23-41), integrated with the
 * assembly's quadrature rule; the reference integrates with its evaluator's default, p + 1 Gauss
 * points per direction, so the two agree when quA = 1 and quB = 1 (the default) */
int gsgpu_l2_error(gsgpu_context* ctx, double* err);
/* gsField::distanceH1 of the last solution against u (gsField.hpp:44-60): the H1 seminorm
 * sqrt(int |grad u_h - grad u|^2), with the same rule as gsgpu_l2_error */
int gsgpu_h1_error(gsgpu_context* ctx, double* err);

/* Batches of independent problems. No counterpart in the reference, where each problem is its own
 * gsPoissonAssembler + gsConjugateGradient run. `count` single-patch problems (each with its own
 * geometry, degree, knots and closed-form fields; quA/quB shared) form one block-diagonal system
 * that the same launches assemble as a multipatch problem; gsgpu_solve then runs a segmented
 * Jacobi-PCG whose scalars, stopping test and iteration count are per problem, i.e. one
 * gsConjugateGradient per problem. The free dofs of problem j are rows [offsets[j], offsets[j+1])
 * of the batch system, in problem order; refresh / assemble / solve / matrix_csr / rhs / dof_map
 * act on the whole batch. GSGPU_PREC_MIXED solves each problem by an FP32 segmented PCG inside an
 * iterative refinement whose residual b - A x (FP64 operator, FP64 x) and norms stay FP64. */
int gsgpu_set_batch(gsgpu_context* ctx, int count, const gsgpu_problem* problems);
/* per problem: free-dof offsets (count + 1 values), iterations (inner FP32 iterations summed over
 * the refinements in mixed precision) and relative residual of the last solve; any pointer may be NULL */
int gsgpu_batch_info(gsgpu_context* ctx, int* offsets, int* iterations, double* relres);
/* per problem: gsField::distanceL2 of the last solution (count values) */
int gsgpu_batch_l2_error(gsgpu_context* ctx, double* err);
/* per problem: gsField::distanceH1 of the last solution (count values) */
int gsgpu_batch_h1_error(gsgpu_context* ctx, double* err);

/* Request server (continuous batching). No counterpart in the reference, which has no serving
 * layer: a caller there runs one gsPoissonAssembler + gsConjugateGradient per request. Requests
 * (single-patch problems, each copied at submission) are queued in arrival order. Each of `slots`
 * worker threads owns a context and a CUDA stream; when it is free it takes the queue head and every
 * later queued request of the same dimension and tolerance, in arrival order, up to `max_batch`
 * requests and while their estimated device memory fits in what is left of `budget_bytes`, and
 * assembles and solves them as one batch (gsgpu_set_batch) in `precision`. Requests that arrive
 * while batches run join the next batch a slot forms; batches of different slots overlap on the
 * device. A request's result does not depend on the other requests of its batch (every problem of a
 * batch keeps its own CG scalars and stopping test). A request whose estimate exceeds the whole
 * budget fails with GSGPU_ERR_BUDGET. Times are seconds since the server was created. */
typedef struct gsgpu_server gsgpu_server;
typedef struct {
    int status;       /* GSGPU_OK or the request's error code */
    int nfree;        /* free dofs (length of the solution) */
    int iterations;   /* CG iterations (mixed: inner FP32 iterations summed over the refinements) */
    double relres;    /* ||b - A x|| / ||b|| of the returned solution (FP64) */
    double t_submit, t_start, t_done;
    int batch_size;   /* requests solved by the same launches */
    long long batch_id;
    double est_bytes; /* device-memory estimate the admission used */
    double ms_setup, ms_assemble, ms_solve;  /* wall time of the batch's refresh, assemble and solve */
    int resident;     /* 1: the batch ran on a resident context of the same structure (no refresh) */
} gsgpu_request_info;
int gsgpu_server_create(gsgpu_server** srv, int device, int slots, double budget_bytes, int max_batch,
                        int precision);
/* queue a copy of a single-patch problem; *id identifies it in gsgpu_server_wait */
int gsgpu_server_submit(gsgpu_server* srv, const gsgpu_problem* prob, double tol, long long* id);
/* block until request `id` is done; x (capacity doubles, may be NULL) receives the solution. The
 * request is forgotten afterwards. Returns the request's status (GSGPU_ERR_INVALID for an unknown
 * id or a too small x). */
int gsgpu_server_wait(gsgpu_server* srv, long long id, double* x, int capacity, gsgpu_request_info* info);
/* Residency: each slot keeps the contexts of its recent batches (plan, sparsity pattern, gather
 * maps, device buffers) in a least-recently-used list keyed by the batch's structure (per problem:
 * dimension, quadrature rule, Dirichlet strategy, degrees and knots, control-point count, boundary
 * sides). A later batch of the same structure reuses one without refresh(): only its control points
 * and field constants are uploaded (gsgpu_request_info.resident = 1, ms_setup the upload time).
 * Resident contexts hold at most `bytes` of device memory in total (default: a quarter of the
 * budget; 0 keeps none) and count against the budget: when a queued request does not fit beside
 * them, resident contexts are released first. */
int gsgpu_server_set_resident(gsgpu_server* srv, double bytes);
/* message of the last failed request taken by gsgpu_server_wait */
const char* gsgpu_server_last_error(const gsgpu_server* srv);
/* finishes the queued requests, then stops the workers and frees everything */
int gsgpu_server_destroy(gsgpu_server* srv);

/* The closed-form fields of the problem's description (kappa, f = -div(kappa grad u) and u; the
 * formulas in the gsgpu_problem comment) at npts physical points x (npts x dim, row-major), as the
 * device evaluates them. No counterpart in the reference, where these are the caller's gsFunction
 * objects: the C++ drop-in compares the caller's functions with these values. Outputs may be NULL. */
int gsgpu_eval_fields(const gsgpu_problem* prob, int npts, const double* x, double* kappa, double* f, double* u);

/* Utilities with no counterpart in the reference. */
/* the CUDA stream (cudaStream_t) all device work of the context is issued on */
int gsgpu_stream(gsgpu_context* ctx, void** stream);
/* profiling: when on, solve() launches its iterations one by one (no CUDA graph) and brackets
 * every SpMV with CUDA events; gsgpu_spmv_stats returns the launches and their summed device
 * time since profiling was switched on. */
int gsgpu_set_profiling(gsgpu_context* ctx, int on);
int gsgpu_spmv_stats(gsgpu_context* ctx, long long* launches, double* total_ms, double* bytes_per_launch);
/* Jacobi-preconditioned CG on a CSR system already in device memory, allocating no device
 * memory. No counterpart in the reference.
 * For callers that cannot call cudaMalloc: processes whose device memory is already handed to a
 * pool allocator sized to the GPU (a further cudaMalloc fails or evicts the pool's blocks), and
 * latency-bound loops that cannot afford the implicit device synchronisation of an allocation.
 * The caller passes the matrix (n rows, ptr/col/val with sorted columns and a non-zero diagonal in
 * every row), the right-hand side b and the output x, all device pointers on the current device,
 * and the stream to run on; x is overwritten with the solution (the start vector is 0), and the
 * stopping rule, iteration count and relative residual are those of gsgpu_solve with
 * GSGPU_SOLVER_CG_JACOBI. Each call reads the row-pointer end and the solver state back to the
 * host and synchronises `stream`, so it must not be called while that stream (or, in global
 * capture mode, any stream) is being captured into a CUDA graph. A row without a non-zero
 * diagonal returns GSGPU_ERR_INVALID before any iteration; an error already pending on entry
 * returns GSGPU_ERR_CUDA and stays pending. The working vectors live in one fixed 8 MiB device
 * array built into the library, which limits n to 204,276 unknowns; a larger n returns
 * GSGPU_ERR_INVALID before any device work. Every call shares that array, so calls whose work
 * overlaps on the GPU (other streams, other host threads) race and must be serialised by the
 * caller. The first call on a device looks up the array's device address (cudaGetSymbolAddress)
 * with that device current. */
int gsgpu_cg_jacobi_noalloc(int n, const int* ptr, const int* col, const double* val, const double* b, double* x,
                            double tol, int max_iters, void* stream, int* iterations, double* relres);
/* Autotuner of the kernel variants. No counterpart in the reference, whose element loop has no
 * variants. The tuned choices are the 3D stiffness stage 1 (interior rows in shared-memory tiles, or
 * rows with 4 or 2 output fields per launch), the 3D stage 2 (4 or 2 output fields) and the inner
 * FP32 product of single-patch mixed solves on the half-diagonal operator (load-based with one row
 * per thread, TMA-fed, or load-based with four rows per thread); every variant forms the same sums
 * in the same order, so results do not depend on the choice.
 * gsgpu_autotune times each variant on the context's problem with CUDA events (six stiffness
 * combinations and three inner products: ms9[0..5], ms9[6..8], -1 where not applicable; ms9 may be
 * NULL), records the fastest per (kernel group, dimension, degree, Gauss points) in a process-wide
 * table, applies it and leaves the context assembled in mixed precision. Contexts refreshed later
 * take their variants from the table. gsgpu_tuned_variants returns a context's variants for the
 * degrees of its first patch: stage 1, stage 2, inner product (-1 when the problem has no
 * half-diagonal operator). The table is saved to and loaded from a text file (lines "kind dim
 * degree gauss_points variant ms"); loading adds to or replaces the entries in memory. */
int gsgpu_autotune(gsgpu_context* ctx, double* ms9);
int gsgpu_tuned_variants(gsgpu_context* ctx, int* v3);
int gsgpu_tune_save(const char* path);
int gsgpu_tune_load(const char* path);
int gsgpu_tune_clear(void);
/* smallest det J over all quadrature points of the last assemble() */
int gsgpu_min_jacobian(gsgpu_context* ctx, double* detmin);
/* device-time breakdown of the last assemble() in milliseconds:
 * [0] Dirichlet values, [1] basis tables, [2] geometry + coefficient fields,
 * [3] stiffness contraction, [4] load contraction, [5] CSR + rhs scatter, [6] total */
int gsgpu_assemble_times(gsgpu_context* ctx, double* ms7);

#ifdef __cplusplus
}
#endif
#endif
