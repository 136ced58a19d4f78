// sm_103a kernels of the segmented Jacobi-PCG over a batch of independent systems: one
// gsConjugateGradient (src/gsSolver/gsConjugateGradient.hpp:19-84) per segment, with the
// segment's scalars (rho, alpha, beta), ||b|| and stopping test kept apart, and all segments
// advanced by the same launches. The kernels are persistent: a grid of at most 8 CTAs per SM walks
// the (segment, first row) block tables, so converged segments cost one table read per block.
// Dot products are per block partial sums in a fixed order, reduced per segment by one warp.
#include "context.h"
#include "kernels_batch.h"
#include "spmv_row.cuh"

namespace gsgpu {
namespace {

constexpr int kB = 256;
constexpr int kGridCap = 8 * 152;
constexpr int kUnroll = 4;

inline int gridFor(int entries) { return entries < 1 ? 1 : (entries < kGridCap ? entries : kGridCap); }

__device__ __forceinline__ double warpSum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// block sums of two values per thread into *o0, *o1 (fixed order); ends with a barrier so the
// shared scratch can be reused by the next table entry
__device__ __forceinline__ void blockSum2(double a, double b, double* o0, double* o1) {
    __shared__ double ws[2][kB / 32];
    a = warpSum(a);
    b = warpSum(b);
    if ((threadIdx.x & 31) == 0) {
        ws[0][threadIdx.x >> 5] = a;
        ws[1][threadIdx.x >> 5] = b;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s0 = 0.0, s1 = 0.0;
        for (int w = 0; w < kB / 32; ++w) {
            s0 += ws[0][w];
            s1 += ws[1][w];
        }
        *o0 = s0;
        if (o1) *o1 = s1;
    }
    __syncthreads();
}

// every thread gets sum(part[a..b))
__device__ __forceinline__ double blockRange(const double* __restrict__ part, int a, int b) {
    __shared__ double ws[kB / 32];
    double v = 0.0;
    for (int i = a + threadIdx.x; i < b; i += kB) v += part[i];
    v = warpSum(v);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    for (int w = 0; w < kB / 32; ++w) s += ws[w];
    __syncthreads();
    return s;
}

// one warp sums part[a..b) (lane-strided, then a fixed shuffle tree)
__device__ __forceinline__ double warpRange(const double* __restrict__ part, int a, int b, int lane) {
    double v = 0.0;
    for (int i = a + lane; i < b; i += 32) v += part[i];
    return warpSum(v);
}

template <typename T>
__global__ void __launch_bounds__(kB) k_seg_dinv(int n, const int* __restrict__ diag, const T* __restrict__ val,
                                                 T* __restrict__ dinv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dinv[i] = T(1) / val[diag[i]];
}

template <typename T>
__global__ void __launch_bounds__(kB) k_seg_init(SegCg<T> B) {
    for (int e = blockIdx.x; e < B.nV; e += gridDim.x) {
        const BlkEnt be = B.tabV[e];
        const int s = be.patch;
        double bb = 0.0, rz = 0.0;
        if (!(B.outer && B.outer[s].done)) {
            const int row = B.segRow[s] + int(be.base) + threadIdx.x;
            if (row < B.segRow[s + 1]) {
                const T bi = B.b[row];
                B.x[row] = T(0);
                B.r[row] = bi;
                const T zi = B.dinv[row] * bi;
                B.z[row] = zi;
                B.p[row] = zi;
                bb = double(bi) * double(bi);
                rz = double(bi) * double(zi);
            }
        }
        blockSum2(bb, rz, B.partV0 + e, B.partV1 + e);
    }
}

template <typename T>
__global__ void __launch_bounds__(kB) k_seg_init_seg(SegCg<T> B, double tol, int maxit) {
    const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= B.nseg) return;
    const double bb = warpRange(B.partV0, B.segV[s], B.segV[s + 1], lane);
    const double rz = warpRange(B.partV1, B.segV[s], B.segV[s + 1], lane);
    if (lane == 0) {
        SegState& S = B.st[s];
        const bool skip = B.outer && B.outer[s].done;
        S.bnorm = sqrt(bb);
        S.rho = rz;
        S.beta = 0.0;
        S.tol = tol;
        S.maxit = maxit;
        S.iters = 0;
        S.relres = bb > 0.0 ? 1.0 : 0.0;
        S.done = (skip || bb == 0.0) ? 1 : 0;
        if (S.done) atomicAdd(B.ndone, 1);
    }
}

template <typename T, bool REL>
__global__ void __launch_bounds__(kB) k_seg_spmv(SegCg<T> B) {
    const int lane = threadIdx.x % kBatchLanes;
    for (int e = blockIdx.x; e < B.nSp; e += gridDim.x) {
        const BlkEnt be = B.tabSp[e];
        const int s = be.patch;
        if (B.st[s].done) {
            if (threadIdx.x == 0) B.partSp[e] = 0.0;
            continue;
        }
        const int row = B.segRow[s] + int(be.base) + threadIdx.x / kBatchLanes;
        const bool valid = row < B.segRow[s + 1];
        T acc = T(0);
        if (valid)
            dev::rowMac<kBatchLanes, kUnroll, REL>(
                row, B.ptr[row], B.ptr[row + 1], lane, B.col, B.coff, [&](int k) { return B.val[k]; },
                [&](int c) { return B.p[c]; }, [&](T v, T x) { acc += v * x; });
        for (int o = kBatchLanes / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        double c = 0.0;
        if (valid && lane == 0) {
            B.t[row] = acc;
            c = double(acc) * double(B.p[row]);
        }
        blockSum2(c, 0.0, B.partSp + e, nullptr);
    }
}

template <typename T>
__global__ void __launch_bounds__(kB) k_seg_update(SegCg<T> B) {
    for (int e = blockIdx.x; e < B.nV; e += gridDim.x) {
        const BlkEnt be = B.tabV[e];
        const int s = be.patch;
        if (B.st[s].done) continue;
        const double pAp = blockRange(B.partSp, B.segSp[s], B.segSp[s + 1]);
        const T alpha = T(B.st[s].rho / pAp);
        const int row = B.segRow[s] + int(be.base) + threadIdx.x;
        double rr = 0.0, rz = 0.0;
        if (row < B.segRow[s + 1]) {
            B.x[row] += alpha * B.p[row];
            const T ri = B.r[row] - alpha * B.t[row];
            B.r[row] = ri;
            const T zi = B.dinv[row] * ri;
            B.z[row] = zi;
            rr = double(ri) * double(ri);
            rz = double(ri) * double(zi);
        }
        blockSum2(rr, rz, B.partV0 + e, B.partV1 + e);
    }
}

template <typename T>
__global__ void __launch_bounds__(kB) k_seg_scalars(SegCg<T> B) {
    const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= B.nseg || B.st[s].done) return;
    const double rr = warpRange(B.partV0, B.segV[s], B.segV[s + 1], lane);
    const double rz = warpRange(B.partV1, B.segV[s], B.segV[s + 1], lane);
    if (lane == 0) {
        SegState& S = B.st[s];
        S.iters += 1;
        S.relres = sqrt(rr) / S.bnorm;
        if (S.relres < S.tol) S.done = 1;
        else if (S.iters >= S.maxit) S.done = 2;
        if (S.done) atomicAdd(B.ndone, 1);
        S.beta = rz / S.rho;
        S.rho = rz;
    }
}

template <typename T>
__global__ void __launch_bounds__(kB) k_seg_pupd(SegCg<T> B) {
    for (int e = blockIdx.x; e < B.nV; e += gridDim.x) {
        const BlkEnt be = B.tabV[e];
        const int s = be.patch;
        if (B.st[s].done) continue;
        const T beta = T(B.st[s].beta);
        const int row = B.segRow[s] + int(be.base) + threadIdx.x;
        if (row < B.segRow[s + 1]) B.p[row] = B.z[row] + beta * B.p[row];
    }
}

// ---- iterative refinement (outer FP64) ----

template <bool REL>
__global__ void __launch_bounds__(kB) k_ref_resid(SegCg<float> B, SegRefine R) {
    const int lane = threadIdx.x % kBatchLanes;
    for (int e = blockIdx.x; e < B.nSp; e += gridDim.x) {
        const BlkEnt be = B.tabSp[e];
        const int s = be.patch;
        if (R.st[s].done) {
            if (threadIdx.x == 0) B.partSp[e] = 0.0;
            continue;
        }
        const int row = B.segRow[s] + int(be.base) + threadIdx.x / kBatchLanes;
        const bool valid = row < B.segRow[s + 1];
        double acc = 0.0;
        if (valid)
            dev::rowMac<kBatchLanes, kUnroll, REL>(
                row, B.ptr[row], B.ptr[row + 1], lane, B.col, B.coff,
                [&](int k) { return double(R.hi[k]) + double(R.lo[k]); }, [&](int c) { return R.x[c]; },
                [&](double v, double x) { acc += v * x; });
        for (int o = kBatchLanes / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        double c = 0.0;
        if (valid && lane == 0) {
            const double ri = R.b[row] - acc;
            R.r[row] = ri;
            c = ri * ri;
        }
        blockSum2(c, 0.0, B.partSp + e, nullptr);
    }
}

__global__ void __launch_bounds__(kB) k_ref_seg(SegCg<float> B, SegRefine R, double tol, int maxref, int first) {
    const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (s >= B.nseg || R.st[s].done) return;
    const double rr = warpRange(B.partSp, B.segSp[s], B.segSp[s + 1], lane);
    if (lane == 0) {
        SegState& S = R.st[s];
        if (first) {
            S.bnorm = sqrt(rr);
            S.iters = 0;
            S.total = 0;
            S.tol = tol;
            S.maxit = maxref;
        } else {
            S.iters += 1;  // refinements done
        }
        S.relres = S.bnorm > 0.0 ? sqrt(rr) / S.bnorm : 0.0;
        if (S.relres < tol) S.done = 1;
        else if (S.iters >= maxref) S.done = 2;
        if (S.done) atomicAdd(R.ndone, 1);
    }
}

__global__ void __launch_bounds__(kB) k_ref_rhs(SegCg<float> B, SegRefine R) {
    for (int e = blockIdx.x; e < B.nV; e += gridDim.x) {
        const BlkEnt be = B.tabV[e];
        const int s = be.patch;
        if (R.st[s].done) continue;
        const int row = B.segRow[s] + int(be.base) + threadIdx.x;
        if (row < B.segRow[s + 1]) R.r32[row] = float(R.r[row]);
    }
}

__global__ void __launch_bounds__(kB) k_ref_correct(SegCg<float> B, SegRefine R) {
    for (int e = blockIdx.x; e < B.nV; e += gridDim.x) {
        const BlkEnt be = B.tabV[e];
        const int s = be.patch;
        if (R.st[s].done) continue;
        const int row = B.segRow[s] + int(be.base) + threadIdx.x;
        if (row < B.segRow[s + 1]) R.x[row] += double(R.d32[row]);
    }
}

__global__ void __launch_bounds__(kB) k_ref_count(SegCg<float> B, SegRefine R) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < B.nseg) R.st[s].total += B.st[s].iters;
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
    k_seg_init<T><<<gridFor(B.nV), kB, 0, s>>>(B);
    k_seg_init_seg<T><<<(B.nseg * 32 + kB - 1) / kB, kB, 0, s>>>(B, tol, maxit);
}

template <typename T>
void segIteration(const SegCg<T>& B, cudaStream_t s) {
    if (B.coff) k_seg_spmv<T, true><<<gridFor(B.nSp), kB, 0, s>>>(B);
    else k_seg_spmv<T, false><<<gridFor(B.nSp), kB, 0, s>>>(B);
    k_seg_update<T><<<gridFor(B.nV), kB, 0, s>>>(B);
    k_seg_scalars<T><<<(B.nseg * 32 + kB - 1) / kB, kB, 0, s>>>(B);
    k_seg_pupd<T><<<gridFor(B.nV), kB, 0, s>>>(B);
}

void refineResidual(const SegCg<float>& B, const SegRefine& R, double tol, int maxref, int first, cudaStream_t s) {
    if (first) {
        GSGPU_CUDA_TRY(cudaMemsetAsync(R.x, 0, sizeof(double) * size_t(B.n), s));
        GSGPU_CUDA_TRY(cudaMemsetAsync(R.st, 0, sizeof(SegState) * size_t(B.nseg), s));
        GSGPU_CUDA_TRY(cudaMemsetAsync(R.ndone, 0, sizeof(int), s));
    }
    if (B.coff) k_ref_resid<true><<<gridFor(B.nSp), kB, 0, s>>>(B, R);
    else k_ref_resid<false><<<gridFor(B.nSp), kB, 0, s>>>(B, R);
    k_ref_seg<<<(B.nseg * 32 + kB - 1) / kB, kB, 0, s>>>(B, R, tol, maxref, first);
}

void refineRhs(const SegCg<float>& B, const SegRefine& R, cudaStream_t s) {
    k_ref_rhs<<<gridFor(B.nV), kB, 0, s>>>(B, R);
}

void refineCorrect(const SegCg<float>& B, const SegRefine& R, cudaStream_t s) {
    k_ref_correct<<<gridFor(B.nV), kB, 0, s>>>(B, R);
}

void refineCount(const SegCg<float>& B, const SegRefine& R, cudaStream_t s) {
    k_ref_count<<<(B.nseg + kB - 1) / kB, kB, 0, s>>>(B, R);
}

template void segDinv<double>(const SegCg<double>&, const int*, cudaStream_t);
template void segDinv<float>(const SegCg<float>&, const int*, cudaStream_t);
template void segInit<double>(const SegCg<double>&, double, int, cudaStream_t);
template void segInit<float>(const SegCg<float>&, double, int, cudaStream_t);
template void segIteration<double>(const SegCg<double>&, cudaStream_t);
template void segIteration<float>(const SegCg<float>&, cudaStream_t);

}  // namespace launch
}  // namespace gsgpu
