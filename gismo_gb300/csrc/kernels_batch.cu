// sm_103a kernels of the segmented Jacobi-PCG over a batch of independent systems: one
// gsConjugateGradient (src/gsSolver/gsConjugateGradient.hpp:19-84) per segment, with the
// segment's scalars (rho, alpha, beta), ||b|| and stopping test kept apart, and all segments
// advanced by the same launches. The batch matrix is swept as one CSR matrix by row-parallel
// grid-stride kernels (rows of converged segments are skipped after one rowSeg / done lookup);
// dot products are per-row contributions summed per segment by one warp in a fixed order, so
// the results do not depend on the launch shape.
#include <algorithm>
#include <type_traits>

#include "context.h"
#include "df32.cuh"
#include "kernels_batch.h"
#include "spmv_row.cuh"

namespace gsgpu {
namespace {

constexpr int kB = 256;
constexpr int kGridCap = 8 * 152;  // 8 resident CTAs of 256 threads on each of the 152 SMs
constexpr int kLanes = 8;          // lanes per CSR row in the SpMV kernels
constexpr int kUnroll = 4;

inline int gridFor(long long items, int perBlock) {
    const long long g = (items + perBlock - 1) / perBlock;
    return int(g < 1 ? 1 : (g < kGridCap ? g : kGridCap));
}
inline int segGrid(int nseg) { return (nseg * 32 + kB - 1) / kB > 0 ? (nseg * 32 + kB - 1) / kB : 1; }

__device__ __forceinline__ double warpSum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// one warp sums part[a..b) (lane-strided, then a fixed shuffle tree)
__device__ __forceinline__ double warpRange(const double* __restrict__ part, int a, int b, int lane) {
    double v = 0.0;
    for (int i = a + lane; i < b; i += 32) v += part[i];
    return warpSum(v);
}

// the same sum by the kSegB threads of one block (fixed order: thread-strided partials, then the
// warps' sums in warp order); every thread returns it. One block per segment: the largest segments
// of a batch (tens of thousands of rows) no longer serialise hundreds of dependent loads on one warp
constexpr int kSegB = 128;
__device__ __forceinline__ double blockRange(const double* __restrict__ part, int a, int b) {
    __shared__ double ws[kSegB / 32];
    double v = 0.0;
    for (int i = a + int(threadIdx.x); i < b; i += kSegB) v += part[i];
    v = warpSum(v);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    double sum = 0.0;
    for (int w = 0; w < kSegB / 32; ++w) sum += ws[w];
    __syncthreads();
    return sum;
}

__device__ __forceinline__ bool rowActive(const int* __restrict__ rowSeg, const SegState* __restrict__ st, int row) {
    const SegState& S = st[rowSeg[row]];
    return !S.done && !S.pause;
}

constexpr double kReplaceDrop = 1e-2;  // mixed: replace once the recursive residual dropped by this factor

template <typename T>
__global__ void __launch_bounds__(kB) k_seg_dinv(int n, const int* __restrict__ diag, const T* __restrict__ val,
                                                 T* __restrict__ dinv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dinv[i] = T(1) / val[diag[i]];
}

template <typename T>
__global__ void __launch_bounds__(kB) k_seg_init(SegCg<T> B) {
    for (int i = blockIdx.x * kB + threadIdx.x; i < B.n; i += gridDim.x * kB) {
        if (B.outer && B.outer[B.rowSeg[i]].done) continue;
        const T bi = B.b[i];
        B.x[i] = T(0);
        B.r[i] = bi;
        const T zi = B.dinv[i] * bi;
        B.z[i] = zi;
        B.p[i] = zi;
        B.rc0[i] = double(bi) * double(bi);
        B.rc1[i] = double(bi) * double(zi);
    }
}

template <typename T>
__global__ void __launch_bounds__(kB) k_seg_init_seg(SegCg<T> B, double tol, int maxit) {
    const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= B.nseg) return;
    const bool skip = B.outer && B.outer[s].done;
    double bb = 0.0, rz = 0.0;
    if (!skip) {
        bb = warpRange(B.rc0, B.segRow[s], B.segRow[s + 1], lane);
        rz = warpRange(B.rc1, B.segRow[s], B.segRow[s + 1], lane);
    }
    if (lane == 0) {
        SegState& S = B.st[s];
        S.bnorm = sqrt(bb);
        S.rho = rz;
        S.alpha = 0.0;
        S.beta = 0.0;
        S.tol = tol;
        S.maxit = maxit;
        S.iters = 0;
        S.relres = bb > 0.0 ? 1.0 : 0.0;
        S.pause = 0;
        S.last_true = 1.0;
        S.done = (skip || bb == 0.0) ? 1 : 0;
        if (S.done) atomicAdd(B.ndone, 1);
    }
}

// a piece's segment is running (the test is uniform over the warp that owns the piece)
template <typename T>
__device__ __forceinline__ bool pieceRunning(const SegCg<T>& B, int j) {
    const SegState& S = B.st[B.pieceSeg[j]];
    return !S.done && !S.pause;
}

// the piece kernels: one warp per piece of kSegPiece = 32 rows, grid-stride over the pieces; the
// piece's partial sums are the warp's shuffle trees (fixed order, no block barrier)
__device__ __forceinline__ int warpId() { return int((blockIdx.x * blockDim.x + threadIdx.x) >> 5); }
__device__ __forceinline__ int warpCount() { return int((gridDim.x * blockDim.x) >> 5); }

// t = A p on the pieces of running segments (kLanes lanes per CSR row); pp0[piece] = its part of p.t
template <typename T, bool REL>
__global__ void __launch_bounds__(kB) k_seg_spmv(SegCg<T> B) {
    constexpr int rpw = 32 / kLanes;  // rows per warp pass
    const int lane = threadIdx.x % kLanes;
    for (int j = warpId(); j < B.npiece; j += warpCount()) {
        if (!pieceRunning(B, j)) continue;
        const int r1 = B.pieceRow[j + 1];
        double c = 0.0;
        for (int base = B.pieceRow[j]; base < r1; base += rpw) {
            const int row = base + int(threadIdx.x & 31) / kLanes;
            const bool act = row < r1;
            T acc = T(0);
            if (act)
                dev::rowMac<kLanes, kUnroll, REL>(
                    row, B.ptr[row], B.ptr[row + 1], lane, B.col, B.coff, [&](int k) { return B.val[k]; },
                    [&](int c) { return B.p[c]; }, [&](T v, T x) { acc += v * x; });
            for (int o = kLanes / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (act && lane == 0) {
                B.t[row] = acc;
                c += double(acc) * double(B.p[row]);
            }
        }
        c = warpSum(c);  // one tree per piece (the rows' terms were summed per lane first)
        if ((threadIdx.x & 31) == 0) B.pp0[j] = c;
    }
}

// one warp per segment: alpha = rho / p.Ap from the segment's piece partials
template <typename T>
__global__ void __launch_bounds__(kB) k_seg_alpha(SegCg<T> B) {
    const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= B.nseg) return;
    const int done = B.st[s].done, pause = B.st[s].pause;
    __syncwarp();  // every lane has read the flags before lane 0 may change them
    if (done) return;
    if (pause) {  // idle until the replacement; the pausing iteration's p update has run
        if (lane == 0) B.st[s].pause = 2;
        return;
    }
    const double pAp = warpRange(B.pp0, B.segPiece[s], B.segPiece[s + 1], lane);
    if (lane == 0) B.st[s].alpha = B.st[s].rho / pAp;
}

// the warp's sum of the lanes' products a b as a double on lane 0. FP32 factors: each product is
// exact as a double-float (TwoProd) and the shuffle tree adds double-floats on the FP32 pipe; a tree
// of doubles (10 FP64 additions per warp and 32 rows for two sums) made the piece kernels FP64 bound
// (GB300's FP64 pipe does 2 FMAs per clock per SM: 133-150 us per update of 8M rows against 56 us
// for the row-parallel form). FP64 factors: the product and the tree in FP64.
__device__ __forceinline__ double warpDot(float a, float b) {
    float p, e;
    twoProd(a, b, p, e);
    df32 v(p, e);
    for (int o = 16; o > 0; o >>= 1)
        v = v + df32(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o));
    return double(v.hi) + double(v.lo);
}
__device__ __forceinline__ double warpDot(double a, double b) { return warpSum(a * b); }

// x += alpha p; r -= alpha t; z = D^-1 r on the pieces of running segments; pp0, pp1[piece] = its
// parts of r.r and r.z
template <typename T>
__global__ void __launch_bounds__(kB) k_seg_update(SegCg<T> B) {
    for (int j = warpId(); j < B.npiece; j += warpCount()) {
        if (!pieceRunning(B, j)) continue;
        const int i = B.pieceRow[j] + int(threadIdx.x & 31);
        T ri = T(0), zi = T(0);
        if (i < B.pieceRow[j + 1]) {
            const T alpha = T(B.st[B.pieceSeg[j]].alpha);
            B.x[i] += alpha * B.p[i];
            ri = B.r[i] - alpha * B.t[i];
            B.r[i] = ri;
            zi = B.dinv[i] * ri;
            B.z[i] = zi;
        }
        const double rr = warpDot(ri, ri), rz = warpDot(ri, zi);
        if ((threadIdx.x & 31) == 0) {
            B.pp0[j] = rr;
            B.pp1[j] = rz;
        }
    }
}

// one warp per segment: r.r and r.z from the piece partials, the stopping test, beta
template <typename T>
__global__ void __launch_bounds__(kB) k_seg_scalars(SegCg<T> B) {
    const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= B.nseg) return;
    const bool skip = B.st[s].done || B.st[s].pause;
    __syncwarp();  // lane 0 changes them only after every lane has read them
    if (skip) return;
    const double rr = warpRange(B.pp0, B.segPiece[s], B.segPiece[s + 1], lane);
    const double rz = warpRange(B.pp1, B.segPiece[s], B.segPiece[s + 1], lane);
    if (lane == 0) {
        SegState& S = B.st[s];
        S.iters += 1;
        S.relres = sqrt(rr) / S.bnorm;
        if (B.outer) {
            // mixed: the FP32 recursion stops for a true-residual replacement at the tolerance,
            // once it has gained kReplaceDrop over the last true residual, or at the limit
            if (S.relres < S.tol || S.relres < kReplaceDrop * S.last_true || S.iters >= S.maxit) S.pause = 1;
        } else {
            if (S.relres < S.tol) S.done = 1;
            else if (S.iters >= S.maxit) S.done = 2;
            if (S.done) atomicAdd(B.ndone, 1);
        }
        S.beta = rz / S.rho;
        S.rho = rz;
    }
}

template <typename T>
__global__ void __launch_bounds__(kB) k_seg_pupd(SegCg<T> B) {
    for (int i = blockIdx.x * kB + threadIdx.x; i < B.n; i += gridDim.x * kB) {
        const SegState& S = B.st[B.rowSeg[i]];
        if (S.done || S.pause > 1) continue;
        B.p[i] = B.z[i] + T(S.beta) * B.p[i];
    }
}

// ---- iterative refinement (outer FP64) ----

// r = b - (hi + lo) x on the rows of segments not yet converged; rc0 = r .* r
template <bool REL>
__global__ void __launch_bounds__(kB) k_ref_resid(SegCg<float> B, SegRefine R, int first) {
    constexpr int rpb = kB / kLanes;
    const int lane = threadIdx.x % kLanes;
    for (int base = blockIdx.x * rpb; base < B.n; base += gridDim.x * rpb) {
        const int row = base + threadIdx.x / kLanes;
        // the first residual on every running segment, later ones on the segments whose FP32
        // recursion is waiting for its replacement
        const bool act = row < B.n && rowActive(B.rowSeg, R.st, row) && (first || B.st[B.rowSeg[row]].pause);
        // (hi + lo) x in double-float arithmetic on the FP32 pipe (x as its df32 split, compensated
        // accumulation per lane, the lanes' sums added in df32), as the single-system residual
        // replacement does: FP64 products here ran on GB300's FP64 pipe at a fraction of the rate
        Dot2 acc;
        if (act)
            dev::rowMac<kLanes, kUnroll, REL>(
                row, B.ptr[row], B.ptr[row + 1], lane, B.col, B.coff,
                [&](int k) { return df32(R.hi[k], R.lo[k]); }, [&](int c) { return R.xdf[c]; },
                [&](df32 v, df32 x) { acc.mac(v, x); });
        df32 y = acc.result();
        for (int o = kLanes / 2; o > 0; o >>= 1) {
            const df32 oth(__shfl_xor_sync(0xffffffffu, y.hi, o), __shfl_xor_sync(0xffffffffu, y.lo, o));
            y = y + oth;
        }
        if (act && lane == 0) {
            const double ri = R.b[row] - y.toDouble();
            R.r[row] = ri;
            B.rc0[row] = ri * ri;
        }
    }
}

// one block per segment
__global__ void __launch_bounds__(kSegB) k_ref_seg(SegCg<float> B, SegRefine R, double tol, int maxref, int first) {
    const int s = blockIdx.x;
    if (R.st[s].done || (!first && !B.st[s].pause)) return;  // changed by thread 0 only after the sum
    const double rr = blockRange(B.rc0, B.segRow[s], B.segRow[s + 1]);
    if (threadIdx.x == 0) {
        SegState& S = R.st[s];
        if (first) {
            S.bnorm = sqrt(rr);
            S.iters = 0;
            S.total = 0;
            S.tol = tol;
            S.maxit = maxref;
        } else {
            S.iters += 1;  // replacements done
        }
        S.relres = S.bnorm > 0.0 ? sqrt(rr) / S.bnorm : 0.0;
        if (S.relres < tol) S.done = 1;
        else if (S.iters >= maxref) S.done = 2;
        if (S.done) atomicAdd(R.ndone, 1);
    }
}

__global__ void __launch_bounds__(kB) k_ref_rhs(SegCg<float> B, SegRefine R) {
    for (int i = blockIdx.x * kB + threadIdx.x; i < B.n; i += gridDim.x * kB)
        if (rowActive(B.rowSeg, R.st, i)) R.r32[i] = float(R.r[i]);
}

// x += d (FP64) and d = 0 on the rows of running segments: the FP32 recursion's progress moves into x
__global__ void __launch_bounds__(kB) k_ref_absorb(SegCg<float> B, SegRefine R) {
    for (int i = blockIdx.x * kB + threadIdx.x; i < B.n; i += gridDim.x * kB)
        if (rowActive(B.rowSeg, R.st, i)) {
            const double xi = R.x[i] + double(B.x[i]);
            R.x[i] = xi;
            R.xdf[i] = df32(xi);
            B.x[i] = 0.f;
        }
}

// a paused segment's recursion continues from the true residual: r32 = fl32(r), z = D^-1 r32,
// rc1 = r32 . z; the search direction is kept unless the true residual is more than 4x the
// recursive one (then p = z)
__global__ void __launch_bounds__(kB) k_ref_replace(SegCg<float> B, SegRefine R) {
    for (int i = blockIdx.x * kB + threadIdx.x; i < B.n; i += gridDim.x * kB) {
        const int sg = B.rowSeg[i];
        if (R.st[sg].done || B.st[sg].done || !B.st[sg].pause) continue;
        const float ri = float(R.r[i]);
        B.r[i] = ri;
        const float zi = B.dinv[i] * ri;
        B.z[i] = zi;
        if (R.st[sg].relres > 4.0 * B.st[sg].relres) B.p[i] = zi;
        B.rc1[i] = double(ri) * double(zi);
    }
}

// per segment: a segment the true residual has finished leaves the recursion; a paused one
// resumes with rho of the replaced residual (or ends at its iteration limit)
// one block per segment
__global__ void __launch_bounds__(kSegB) k_ref_replace_seg(SegCg<float> B, SegRefine R) {
    const int s = blockIdx.x;
    const int innerDone = B.st[s].done, outerDone = R.st[s].done, pause = B.st[s].pause;
    __syncthreads();  // every thread has read the flags before thread 0 may change them
    if (innerDone) return;
    if (outerDone) {
        if (threadIdx.x == 0) {
            B.st[s].done = outerDone;
            atomicAdd(B.ndone, 1);
        }
        return;
    }
    if (!pause) return;
    const double rz = blockRange(B.rc1, B.segRow[s], B.segRow[s + 1]);
    if (threadIdx.x == 0) {
        SegState& S = B.st[s];
        if (S.iters >= S.maxit) {
            S.done = 2;
            atomicAdd(B.ndone, 1);
            R.st[s].done = 2;
            atomicAdd(R.ndone, 1);
            return;
        }
        S.rho = rz;
        S.last_true = R.st[s].relres;
        S.pause = 0;
    }
}

__global__ void __launch_bounds__(kB) k_ref_count(SegCg<float> B, SegRefine R) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < B.nseg) R.st[s].total += B.st[s].iters;
}

// ---- half-diagonal FP32 inner operator of the problems (mixed solve) ----

// d of every problem from the df32 band: one thread per batch row. The band entry of the problem's
// row with box coordinates b and offset o is band_off + (c0 W0 + o0 + p0) + (c1 W1 + o1 + p1) n0 W0
// + (c2 W2 + o2 + p2) n0 W0 n1 W1 with c = b + lo; offsets in the storage order of sdia.cu (the
// centre line o0 = 0..p0 first, then the lines (o2, o1) >= (0, 1) lexicographically, o0 ascending).
__global__ void __launch_bounds__(kB) k_seg_sdia_build(int n, const int* __restrict__ rowSeg,
                                                      const SegSdiaDesc* __restrict__ desc,
                                                      const df32* __restrict__ band, float* __restrict__ d) {
    const int row = blockIdx.x * kB + threadIdx.x;
    if (row >= n) return;
    const SegSdiaDesc D = desc[rowSeg[row]];
    if (D.nh == 0) return;
    const int r = row - D.row0;
    int b[3];
    b[0] = r % D.m[0];
    b[1] = (r / D.m[0]) % D.m[1];
    b[2] = r / (D.m[0] * D.m[1]);
    const long long n0W = (long long)D.bn[0] * D.W[0], n1W = (long long)D.bn[1] * D.W[1];
    const long long rowBase = D.band_off + (long long)(b[0] + D.lo[0]) * D.W[0] +
                              (long long)(b[1] + D.lo[1]) * D.W[1] * n0W +
                              (long long)(b[2] + D.lo[2]) * D.W[2] * n0W * n1W;
    auto value = [&](int o0, int o1, int o2) -> float {
        const int c0 = b[0] + o0, c1 = b[1] + o1, c2 = b[2] + o2;
        if (c0 < 0 || c0 >= D.m[0] || c1 < 0 || c1 >= D.m[1] || c2 < 0 || c2 >= D.m[2]) return 0.f;
        return band[rowBase + (o0 + D.p[0]) + (long long)(o1 + D.p[1]) * n0W + (long long)(o2 + D.p[2]) * n0W * n1W].hi;
    };
    float* dr = d + D.doff + r;
    const long long ns = D.n;
    long long h = 0;
    for (int o0 = 0; o0 <= D.p[0]; ++o0, ++h) dr[h * ns] = value(o0, 0, 0);
    for (int o2 = 0; o2 <= D.p[2]; ++o2)
        for (int o1 = o2 ? -D.p[1] : 1; o1 <= D.p[1]; ++o1)
            for (int o0 = -D.p[0]; o0 <= D.p[0]; ++o0, ++h) dr[h * ns] = value(o0, o1, o2);
}

// row r (problem-local) of A x from the half diagonals dq = d + doff, x = xq[0..n): the row's own
// values d[h n + r] times x[r + L_h] and the mirrored ones d[h n + r - L_h] times x[r - L_h]
// (A(r, r - o) = A(r - o, r)). Every non-centre offset of the half box has L_h > 0 (the box is at
// least 2p + 1 wide), so a term is taken when r + L_h < n (upper) or r - L_h >= 0 (mirrored); the
// terms left out have a tensor point outside the box, whose stored value is 0. Terms in the order of
// k_sdia32_dot (sdia.cu): the centre line, then per line its 2 (2 P0 + 1) products summed first.
template <int P0>
__device__ __forceinline__ float segSdiaRow(const SegSdiaDesc& D, int r, const float* __restrict__ dq,
                                            const float* __restrict__ xq) {
    constexpr int W0 = 2 * P0 + 1;
    const int n = D.n;
    const float* dh = dq + r;
    float acc = 0.f;
#pragma unroll
    for (int o0 = 0; o0 <= P0; ++o0) {
        if (r + o0 < n) acc = fmaf(__ldcg(dh), __ldg(xq + r + o0), acc);
        if (o0 > 0 && r - o0 >= 0) acc = fmaf(__ldcg(dh - o0), __ldg(xq + r - o0), acc);
        dh += n;
    }
    const int p1 = D.p[1], p2 = D.p[2], m0 = D.m[0], m1 = D.m[1];
    for (int o2 = 0; o2 <= p2; ++o2)
        for (int o1 = o2 ? -p1 : 1; o1 <= p1; ++o1) {
            const int L21 = (o2 * m1 + o1) * m0;
            float vu[W0], xu[W0], vd[W0], xd[W0];
#pragma unroll
            for (int k = 0; k < W0; ++k) {
                const int L = L21 + k - P0;
                const bool up = r + L < n, down = r - L >= 0;
                vu[k] = up ? __ldcg(dh + (long long)k * n) : 0.f;
                xu[k] = up ? __ldg(xq + r + L) : 0.f;
                vd[k] = down ? __ldcg(dh + (long long)k * n - L) : 0.f;
                xd[k] = down ? __ldg(xq + r - L) : 0.f;
            }
            float lsum = 0.f;
#pragma unroll
            for (int k = 0; k < W0; ++k) {
                lsum = fmaf(vu[k], xu[k], lsum);
                lsum = fmaf(vd[k], xd[k], lsum);
            }
            acc += lsum;
            dh += (long long)W0 * n;
        }
    return acc;
}

// t = A p on the pieces of running segments from the half diagonals, one row per lane (a problem
// without them: its CSR row, one lane); pp0[piece] = its part of p.t. Blocks of kBS threads: at
// its 54 registers an SM holds 36 warps in blocks of 4 warps, 32 in blocks of 8
constexpr int kBS = 128;
__global__ void __launch_bounds__(kBS) k_seg_sdia(SegCg<float> B) {
    for (int j = warpId(); j < B.npiece; j += warpCount()) {
        if (!pieceRunning(B, j)) continue;
        const int row = B.pieceRow[j] + int(threadIdx.x & 31);
        float acc = 0.f, pr = 0.f;
        if (row < B.pieceRow[j + 1]) {
            const SegSdiaDesc& D = B.sdia[B.pieceSeg[j]];
            const int r = row - D.row0;
            const float* dq = B.sd + D.doff;
            const float* xq = B.p + D.row0;
            if (D.nh == 0) {
                for (int k = B.ptr[row]; k < B.ptr[row + 1]; ++k)
                    acc = fmaf(B.val[k], B.p[B.coff ? row + int(B.coff[k]) : B.col[k]], acc);
            } else switch (D.p[0]) {
                case 1: acc = segSdiaRow<1>(D, r, dq, xq); break;
                case 2: acc = segSdiaRow<2>(D, r, dq, xq); break;
                case 3: acc = segSdiaRow<3>(D, r, dq, xq); break;
                default: acc = segSdiaRow<4>(D, r, dq, xq); break;
            }
            B.t[row] = acc;
            pr = B.p[row];
        }
        const double c = warpDot(acc, pr);
        if ((threadIdx.x & 31) == 0) B.pp0[j] = c;
    }
}

}  // namespace

namespace launch {

template <typename T>
void segDinv(const SegCg<T>& B, const int* diag, cudaStream_t s) {
    if (B.n > 0) k_seg_dinv<T><<<(B.n + kB - 1) / kB, kB, 0, s>>>(B.n, diag, B.val, const_cast<T*>(B.dinv));
}

template <typename T>
void segInit(const SegCg<T>& B, double tol, int maxit, cudaStream_t s) {
    GSGPU_CUDA_TRY(cudaMemsetAsync(B.ndone, 0, sizeof(int), s));
    k_seg_init<T><<<gridFor(B.n, kB), kB, 0, s>>>(B);
    k_seg_init_seg<T><<<segGrid(B.nseg), kB, 0, s>>>(B, tol, maxit);
}

// blocks of kB threads that are resident together for kernel k (grid-stride over the pieces with
// every block resident: no SM runs a second wave that others do not)
template <typename K>
int residentBlocks(K k, int threads = kB) {
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, threads, 0);
    return std::max(1, sms * per);
}

template <typename T>
void segIteration(const SegCg<T>& B, cudaStream_t s) {
    const unsigned np = unsigned(std::max(1, (B.npiece + kB / 32 - 1) / (kB / 32)));  // blocks of kB / 32 pieces
    bool halfDiag = false;
    if constexpr (std::is_same<T, float>::value) {
        if (B.sdia) {
            static const int resident = residentBlocks(k_seg_sdia, kBS);
            const unsigned nps = unsigned(std::max(1, (B.npiece + kBS / 32 - 1) / (kBS / 32)));
            k_seg_sdia<<<std::min<unsigned>(nps, resident), kBS, 0, s>>>(B);
            halfDiag = true;
        }
    }
    if (!halfDiag) {
        if (B.coff) {
            static const int resident = residentBlocks(k_seg_spmv<T, true>);
            k_seg_spmv<T, true><<<std::min<unsigned>(np, resident), kB, 0, s>>>(B);
        } else {
            static const int resident = residentBlocks(k_seg_spmv<T, false>);
            k_seg_spmv<T, false><<<std::min<unsigned>(np, resident), kB, 0, s>>>(B);
        }
    }
    const unsigned ns = unsigned(segGrid(B.nseg));
    k_seg_alpha<T><<<ns, kB, 0, s>>>(B);
    static const int resident = residentBlocks(k_seg_update<T>);
    k_seg_update<T><<<std::min<unsigned>(np, resident), kB, 0, s>>>(B);
    k_seg_scalars<T><<<ns, kB, 0, s>>>(B);
    k_seg_pupd<T><<<gridFor(B.n, kB), kB, 0, s>>>(B);
}

void refineResidual(const SegCg<float>& B, const SegRefine& R, double tol, int maxref, int first, cudaStream_t s) {
    if (first) {
        GSGPU_CUDA_TRY(cudaMemsetAsync(R.x, 0, sizeof(double) * size_t(B.n), s));
        GSGPU_CUDA_TRY(cudaMemsetAsync(R.xdf, 0, sizeof(df32) * size_t(B.n), s));
        GSGPU_CUDA_TRY(cudaMemsetAsync(R.st, 0, sizeof(SegState) * size_t(B.nseg), s));
        GSGPU_CUDA_TRY(cudaMemsetAsync(R.ndone, 0, sizeof(int), s));
    }
    const int gs = gridFor(B.n, kB / kLanes);
    if (B.coff) k_ref_resid<true><<<gs, kB, 0, s>>>(B, R, first);
    else k_ref_resid<false><<<gs, kB, 0, s>>>(B, R, first);
    k_ref_seg<<<unsigned(B.nseg > 0 ? B.nseg : 1), kSegB, 0, s>>>(B, R, tol, maxref, first);
}

void refineRhs(const SegCg<float>& B, const SegRefine& R, cudaStream_t s) {
    k_ref_rhs<<<gridFor(B.n, kB), kB, 0, s>>>(B, R);
}

void refineReplace(const SegCg<float>& B, const SegRefine& R, double tol, int maxref, cudaStream_t s) {
    k_ref_absorb<<<gridFor(B.n, kB), kB, 0, s>>>(B, R);
    refineResidual(B, R, tol, maxref, 0, s);
    k_ref_replace<<<gridFor(B.n, kB), kB, 0, s>>>(B, R);
    k_ref_replace_seg<<<unsigned(B.nseg > 0 ? B.nseg : 1), kSegB, 0, s>>>(B, R);
}

void refineCount(const SegCg<float>& B, const SegRefine& R, cudaStream_t s) {
    k_ref_count<<<(B.nseg + kB - 1) / kB, kB, 0, s>>>(B, R);
}

void segSdiaBuild(int n, const int* rowSeg, const SegSdiaDesc* desc, const df32* band, float* d, cudaStream_t s) {
    if (n > 0) k_seg_sdia_build<<<unsigned((n + kB - 1) / kB), kB, 0, s>>>(n, rowSeg, desc, band, d);
}

template void segDinv<double>(const SegCg<double>&, const int*, cudaStream_t);
template void segDinv<float>(const SegCg<float>&, const int*, cudaStream_t);
template void segInit<double>(const SegCg<double>&, double, int, cudaStream_t);
template void segInit<float>(const SegCg<float>&, double, int, cudaStream_t);
template void segIteration<double>(const SegCg<double>&, cudaStream_t);
template void segIteration<float>(const SegCg<float>&, cudaStream_t);

}  // namespace launch
}  // namespace gsgpu
