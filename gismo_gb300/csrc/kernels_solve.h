// Solver kernels (kernels_solve.cu): device-resident PCG state and launch wrappers.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace gsgpu {

// scalars of one preconditioned CG run, kept in device memory
struct CgState {
    double rho, alpha, beta, bnorm, relres, tol;
    double last_true;  // mixed: true relative residual at the last replacement
    double delta;      // mixed: replace once the recursive residual dropped by this factor
    int iters, maxit;
    int done;          // 0 running, 1 converged, 2 reached max_iters
    int pause;         // mixed: waiting for a true-residual replacement
    int pupd_skip;     // the direction update of this iteration is skipped (its beta did not run)
    int replacements;  // mixed: number of true-residual evaluations
    int replaced;      // mixed: a replacement ran in this chunk (restart the FP32 recursion)
    int restart;       // mixed: the replacement moved the residual a lot; restart p = z
    unsigned arrive;   // blocks of the running kernel that have stored their partial sums
};

struct CgBuffers {
    int n = 0;
    int lanes_per_row = 32;
    double delta = 1e-2;  // mixed: residual replacement once the recursive residual dropped by this factor
    const int* ptr = nullptr;
    const int* col = nullptr;
    const int16_t* coff = nullptr;  // if set: column = row + coff[k] (banded patterns), col unused
    // box rows: rows with box[row] = 1 have columns row + box_off[0..nbox) (the full neighbour box of
    // an interior basis function); their column offsets come from a shared table in the SpMV
    const uint8_t* box = nullptr;
    const int* box_off = nullptr;
    int nbox = 0;
    const double* val = nullptr;
    const double* b = nullptr;
    const double* dinv = nullptr;
    double *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *t = nullptr;
    double *part0 = nullptr, *part1 = nullptr, *part2 = nullptr;
    CgState* st = nullptr;
    // mixed precision: FP32 inner operator (hi) and FP64-accurate outer operator (hi + lo)
    const float* val_hi = nullptr;
    const float* val_lo = nullptr;
    const float* dinv32 = nullptr;
    float *r32 = nullptr, *z32 = nullptr, *p32 = nullptr, *t32 = nullptr, *dx32 = nullptr, *xhi = nullptr,
          *xlo = nullptr;
};

namespace launch {
int cgPartials(int n);
int spmvPartials(int n, int lanes_per_row);
void jacobiDiag(int n, const int* diag, const double* val, double damping, double* dinv, cudaStream_t s);
void cgInit(const CgBuffers& B, double tol, int maxit, cudaStream_t s);
void cgIteration(const CgBuffers& B, cudaStream_t s);
void cgSpmv(const CgBuffers& B, cudaStream_t s);
void cgRest(const CgBuffers& B, cudaStream_t s);
// SpMV grids are capped (grid-stride over rows): partials <= this; 8 resident 256-thread blocks on
// each of GB300's 152 SMs, so every SM holds the same number of blocks
constexpr int kMaxSpmvBlocks = 152 * 8;
constexpr int kMaxBox = 1024;  // largest box-row offset table (the (2p+1)^3 box of p <= 4)
// box[row] = 1 iff row has exactly nbox slots with columns row + off[j]; *count = number of such rows
void boxFlags(int n, const int* ptr, const int* col, const int* off, int nbox, uint8_t* box,
              unsigned long long* count, cudaStream_t s);
// mixed precision (FP32 inner iteration, FP64-accurate residual replacement)
void jacobiDiag32(int n, const int* diag, const float* val_hi, float* dinv32, cudaStream_t s);
void mixedInit(const CgBuffers& B, double tol, int maxit, cudaStream_t s);
void mixedSpmv(const CgBuffers& B, cudaStream_t s);
void mixedRest(const CgBuffers& B, cudaStream_t s);
void mixedIteration(const CgBuffers& B, cudaStream_t s);
void mixedReplace(const CgBuffers& B, cudaStream_t s);  // x += dx, r = b - A x (df32), restart r32/z/rho
}  // namespace launch
}  // namespace gsgpu
