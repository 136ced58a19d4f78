// Launch wrappers of the h-multigrid kernels (kernels_mg.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "kernels_solve.h"

namespace gsgpu {

// one level of the device hierarchy in working precision T (level 0 = the assembled matrix)
template <typename T>
struct MgLevelDev {
    int n = 0;
    int lpr = 8;  // lanes per CSR row
    const int* ptr = nullptr;
    const int* col = nullptr;
    const int16_t* coff = nullptr;  // column = row + coff[k] when set
    const T* val = nullptr;
    const int* diag = nullptr;
    T* dinv = nullptr;
    T *b = nullptr, *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *t = nullptr;
    // transfer between this level (coarse) and the next finer one: P rows = finer free dofs
    const int *Pptr = nullptr, *Pcol = nullptr, *Rptr = nullptr, *Rcol = nullptr;
    const T *Pval = nullptr, *Rval = nullptr;
    // coarsest level: Jacobi-PCG reductions and state
    double *part0 = nullptr, *part1 = nullptr, *part2 = nullptr;
    CgState* st = nullptr;
};

struct MgParams {
    int npre = 2, npost = 2;
    double damping = 0.6;  // damped Jacobi smoother
    int cycles = 1;        // coarse-correction cycles on every level but the coarsest (1 = V, 2 = W)
    double cgc = 1.0;      // damping of the coarse-grid correction
    int coarse_iters = 100;  // cap of the coarsest-level Jacobi-PCG
    double coarse_tol = 1e-10;
};

// outer flexible PCG in FP64; the operator is val (FP64) or hi + lo (two FP32 halves)
struct MgOuter {
    int n = 0;
    int lpr = 8;
    const int* ptr = nullptr;
    const int* col = nullptr;
    const int16_t* coff = nullptr;
    const double* val = nullptr;
    const float* hi = nullptr;
    const float* lo = nullptr;
    const double* b = nullptr;
    double *x = nullptr, *r = nullptr, *rold = nullptr, *p = nullptr, *t = nullptr;
    float *phi = nullptr, *plo = nullptr;  // hi + lo operator: p as double-float, for the SpMV on the FP32 pipe
    double *part0 = nullptr, *part1 = nullptr, *part2 = nullptr;
    CgState* st = nullptr;
};

namespace launch {
int mgPartials();
template <typename T>
void mgDinv(const MgLevelDev<T>& L, cudaStream_t s);
// cast a vector between precisions (FP64 <-> FP32)
template <typename Ti, typename To>
void castVec(int n, const Ti* in, To* out, cudaStream_t s);
// coarsest level: Jacobi-PCG start (x = 0, from L.b) and k iterations (no-ops once converged)
template <typename T>
void coarseStart(const MgLevelDev<T>& L, double tol, const CgState* outer, cudaStream_t s);
template <typename T>
void coarseIters(const MgLevelDev<T>& L, int k, const CgState* outer, cudaStream_t s);
// one cycle on levels[l].b: from a zero start (zero) or from levels[l].x, result in levels[l].x;
// kernels skip once outer->done is set
template <typename T>
void vcycle(const std::vector<MgLevelDev<T>>& levels, int l, const MgParams& prm, const CgState* outer, cudaStream_t s,
            bool zero = true);
void mgPcgStart(const MgOuter& O, double tol, int maxit, cudaStream_t s);
// preconditioned direction: z is the V-cycle result of level 0 (precision T)
template <typename T>
void mgPcgPrecond(const MgOuter& O, const std::vector<MgLevelDev<T>>& levels, const MgParams& prm, cudaStream_t s);
void mgPcgStep(const MgOuter& O, cudaStream_t s);
}  // namespace launch
}  // namespace gsgpu
