// Solver kernels (kernels_solve.cu): device-resident PCG state and launch wrappers.
#pragma once

#include <cuda_runtime.h>

namespace gsgpu {

// scalars of one preconditioned CG run, kept in device memory
struct CgState {
    double rho, alpha, beta, bnorm, relres, tol;
    int iters, maxit;
    int done;  // 0 running, 1 converged, 2 reached max_iters
    int pad;
};

struct CgBuffers {
    int n = 0;
    int lanes_per_row = 32;
    const int* ptr = nullptr;
    const int* col = nullptr;
    const double* val = nullptr;
    const double* b = nullptr;
    const double* dinv = nullptr;
    double *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *t = nullptr;
    double *part0 = nullptr, *part1 = nullptr, *part2 = nullptr;
    CgState* st = nullptr;
};

namespace launch {
int cgPartials(int n);
int spmvPartials(int n, int lanes_per_row);
void jacobiDiag(int n, const int* diag, const double* val, double damping, double* dinv, cudaStream_t s);
void cgInit(const CgBuffers& B, double tol, int maxit, cudaStream_t s);
void cgIteration(const CgBuffers& B, cudaStream_t s);
void cgSpmv(const CgBuffers& B, cudaStream_t s);
void cgRest(const CgBuffers& B, cudaStream_t s);
}  // namespace launch
}  // namespace gsgpu
