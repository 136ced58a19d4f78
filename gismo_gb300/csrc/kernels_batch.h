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
    // mixed recursion: waiting for a true-residual replacement (1: set in this iteration, whose
    // direction update still runs; 2: idle), and the true relative residual of the last replacement
    int pause;
    double last_true;
};

// Half-diagonal storage of the FP32 inner operator of one batch problem whose free dofs are one box
// of m0 x m1 x m2 patch-local functions numbered lexicographically (the single-patch form of
// SdiaOp, sdia.cu, without padding): d[doff + h n + r] = A(r, r + o_h) for the nh offsets o_h of the
// half neighbour box, 0 where r + o_h leaves the box; r = row - row0 is the problem-local row.
// nh = 0: the problem does not have that shape, its rows use the CSR values
struct SegSdiaDesc {
    long long doff = 0;      // the problem's first stored value
    long long band_off = 0;  // the patch's band offset
    int row0 = 0, n = 0, nh = 0;
    int m[3] = {1, 1, 1}, p[3] = {0, 0, 0};
    int bn[3] = {1, 1, 1}, W[3] = {1, 1, 1}, lo[3] = {0, 0, 0};  // patch dof counts, band widths, box corner
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
    // FP32 recursion of the mixed solve: if set, the products use the problems' half diagonals sd
    // (described by sdia[segment]) instead of the CSR values
    const SegSdiaDesc* sdia = nullptr;
    const float* sd = nullptr;
    const T* dinv = nullptr;
    const T* b = nullptr;
    T *x = nullptr, *r = nullptr, *z = nullptr, *p = nullptr, *t = nullptr;
    double *rc0 = nullptr, *rc1 = nullptr;  // n each (start and residual replacements)
    // pieces: every segment split into runs of at most kSegPiece rows (piece j: rows pieceRow[j] ..
    // pieceRow[j + 1] - 1 of segment pieceSeg[j]; segment s owns pieces segPiece[s] .. segPiece[s + 1]
    // - 1). The iterations' dot products go through one fixed-order partial per piece (pp0, pp1)
    int npiece = 0;
    const int* pieceRow = nullptr;  // npiece + 1
    const int* pieceSeg = nullptr;  // npiece
    const int* segPiece = nullptr;  // nseg + 1
    double *pp0 = nullptr, *pp1 = nullptr;  // npiece each
    SegState* st = nullptr;
    const SegState* outer = nullptr;  // segments whose outer state is done take no part (refinement)
    int* ndone = nullptr;
};

// rows per piece: the lanes of one warp of the piece kernels
constexpr int kSegPiece = 32;

// iterative refinement: FP64 residual with the split operator hi + lo and FP64 x
struct df32;

struct SegRefine {
    const float* hi = nullptr;
    const float* lo = nullptr;
    const double* b = nullptr;
    double* x = nullptr;         // FP64 solution
    df32* xdf = nullptr;         // its double-float split, kept with x (the residual's right factor)
    double* r = nullptr;         // FP64 residual
    float* r32 = nullptr;        // FP32 copy of the first residual (the recursion's right-hand side)
    SegState* st = nullptr;      // outer state: relres of b - A x, residual replacements in iters
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
// mixed precision: FP32 segmented CG on hi (x = the correction d) with FP64-accurate residual
// replacement. refineResidual: x = 0 (first) then r = b - (hi + lo) x and the stopping test per
// segment on that true residual
void refineResidual(const SegCg<float>& B, const SegRefine& R, double tol, int maxref, int first, cudaStream_t s);
// r32 = r (running segments): the recursion's start
void refineRhs(const SegCg<float>& B, const SegRefine& R, cudaStream_t s);
// x += d, d = 0, the true residual and its test, then the recursion continues from it with its
// search direction kept (finished segments leave it)
void refineReplace(const SegCg<float>& B, const SegRefine& R, double tol, int maxref, cudaStream_t s);
// per segment: the recursion's iteration count into the outer state's total
void refineCount(const SegCg<float>& B, const SegRefine& R, cudaStream_t s);
// the half diagonals of every problem of an n-row batch from the df32 band (hi parts)
void segSdiaBuild(int n, const int* rowSeg, const SegSdiaDesc* desc, const df32* band, float* d, cudaStream_t s);
}  // namespace launch
}  // namespace gsgpu
