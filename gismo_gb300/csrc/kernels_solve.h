// Solver kernels (kernels_solve.cu): device-resident PCG state and launch wrappers.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

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

// half-diagonal storage of the FP32 inner operator of a single patch whose free dofs are one box of
// m0 x m1 x m2 functions numbered lexicographically (sdia.cu): d[h * ns + i] = A(i, i + o_h) for the
// nh offsets o_h of the half neighbour box (lexicographically >= 0), 0 where i + o_h leaves the box;
// the diagonal stride ns is n rounded up to a multiple of 256
struct SdiaOp {
    const float* d = nullptr;
    int n = 0, nh = 0, ns = 0;
    int m[3] = {1, 1, 1};
    int p[3] = {0, 0, 0};
    int xpad = 0;  // zeros the vector x of the product carries before and after its n entries
    int group = 1;  // rows per thread of the load-based product: 1 (scalar loads) or 4 (16-byte loads)
    bool pdl = false;  // launch the four-row product with programmatic dependent launch (pdl.cuh)
    // if set: host copies of the two tensor maps (the diagonals, the vector x) of the TMA-fed product,
    // and the device word its bounded waits set when they expire
    const void* tmaps = nullptr;
    int* err = nullptr;
};
// where the free box sits in the patch's band: patch-local dof counts n, band widths W = 2p + 1,
// the box's lower corner lo and the patch's band offset
struct SdiaBand {
    int n[3] = {1, 1, 1};
    int W[3] = {1, 1, 1};
    int lo[3] = {0, 0, 0};
    long long band_off = 0;
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
    // if sdia.d is set, the inner FP32 products use the half-diagonal form instead of the CSR hi values
    SdiaOp sdia;
    bool vec4 = false;  // the FP32 vectors are 16-byte aligned: the half-diagonal path's vector kernels take four entries a thread
    bool pdl = false;   // the half-diagonal path's iteration kernels use programmatic dependent launch
};

struct df32;

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
// half-diagonal inner operator (sdia.cu): offsets stored, the builder from the df32 band (the hi
// parts, as the CSR gather takes them) and the product t = A x with block partials of x.t
int sdiaHalf(const int* p);
// the largest linear offset |L| of the neighbour box: the zero padding the product needs around x
int sdiaReach(const SdiaOp& A);
void sdiaBuild(const SdiaOp& A, const SdiaBand& B, const df32* band, float* d, cudaStream_t s);
int sdiaPartials(const SdiaOp& A);
// encode the TMA tensor maps of A's diagonals and of the vector x into out2 (two CUtensorMap, 64-byte
// aligned); false (and the reason in *why) if the driver or the shape does not allow them
bool sdiaTensorMaps(const SdiaOp& A, const float* x, void* out2, std::string* why);
// t = A x and the block partials of x.t
void sdiaSpmv(const SdiaOp& A, const float* x, float* t, double* part, const CgState* st, cudaStream_t s);
}  // namespace launch
}  // namespace gsgpu
