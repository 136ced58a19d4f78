// Segmented Jacobi-PCG over a block-diagonal batch of independent systems (kernels_batch.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "gsgpu_internal.h"

namespace gsgpu {

// CG scalars and stopping state of one system of the batch
struct SegState {
    double rho, alpha, beta, bnorm, relres, tol;
    int iters, maxit, done, total;  // done: 0 running, 1 converged, 2 reached maxit; total: iterations summed
};

// The batch matrix is one CSR matrix (block diagonal, rows of segment s in [segRow[s], segRow[s+1]))
// swept by row-parallel kernels; rowSeg maps a row to its segment. Dot products go through
// per-row contributions (rc0, rc1) that one warp per segment sums in a fixed order.
template <typename T>
struct SegCg {
    int n = 0, nseg = 0;
    const int* segRow = nullptr;  // nseg + 1
    const int* rowSeg = nullptr;  // n
    const int* ptr = nullptr;
    const int* col = nullptr;
    const int16_t* coff = nullptr;
    const T* val = nullptr;
    const T* dinv = nullptr;
    const T* b = nullptr;
    T *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *t = nullptr;
    double *rc0 = nullptr, *rc1 = nullptr;  // n each
    SegState* st = nullptr;
    const SegState* outer = nullptr;  // segments whose outer state is done take no part (refinement)
    int* ndone = nullptr;
};

// iterative refinement: FP64 residual with the split operator hi + lo and FP64 x
struct SegRefine {
    const float* hi = nullptr;
    const float* lo = nullptr;
    const double* b = nullptr;
    double* x = nullptr;         // FP64 solution
    double* r = nullptr;         // FP64 residual
    float* r32 = nullptr;        // inner right-hand side
    const float* d32 = nullptr;  // inner solution (correction)
    SegState* st = nullptr;      // outer state: relres of b - A x, refinements in iters
    int* ndone = nullptr;
};

namespace launch {
template <typename T>
void segDinv(const SegCg<T>& B, const int* diag, cudaStream_t s);
// x = 0, r = b, z = D^-1 r, p = z; per-segment bnorm / rho; ndone counts the segments that start done
template <typename T>
void segInit(const SegCg<T>& B, double tol, int maxit, cudaStream_t s);
template <typename T>
void segIteration(const SegCg<T>& B, cudaStream_t s);
// refinement: x = 0 (first) then r = b - (hi + lo) x and the outer stopping test per segment
void refineResidual(const SegCg<float>& B, const SegRefine& R, double tol, int maxref, int first, cudaStream_t s);
// r32 = r (active segments), before an inner solve; x += d32 after it
void refineRhs(const SegCg<float>& B, const SegRefine& R, cudaStream_t s);
void refineCorrect(const SegCg<float>& B, const SegRefine& R, cudaStream_t s);
// per segment: add the inner iterations of the last inner solve to the outer state's total
void refineCount(const SegCg<float>& B, const SegRefine& R, cudaStream_t s);
}  // namespace launch
}  // namespace gsgpu
