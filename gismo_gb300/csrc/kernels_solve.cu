// sm_103a solver kernels: CSR SpMV (K5) fused with the p.Ap reduction, the fused CG vector
// update with Jacobi preconditioning (K6/K7), and the deterministic two-level reductions that
// keep alpha / beta / the stopping test on the device, so that an iteration needs no host
// round trip and a fixed run of iterations can be captured in a CUDA graph.
//
// Iteration (gsConjugateGradient::step, src/gsSolver/gsConjugateGradient.hpp:54-84):
//   t = A p; alpha = rho / (p.t); x += alpha p; r -= alpha t; stop if ||r||/||b|| < tol;
//   z = D^-1 r; beta = (r.z)/rho; p = z + beta p.
#include <algorithm>

#include "df32.cuh"
#include "kernels_solve.h"
#include "pdl.cuh"
#include "spmv_row.cuh"

namespace gsgpu {
namespace {

constexpr int kB = 256;
constexpr int kUnroll = 4;  // independent (value, column) -> x load chains per lane in the SpMV loops
// FP32 SpMV steps (predicated, no serial tail): 8 loads in flight per lane for CSR rows, 11 for
// box rows (a 7x7x7 box row of 343 slots in two steps of 16 lanes)
constexpr int kUnrollP = 8;
constexpr int kUnrollBox = 11;
constexpr int kSpmv32BlocksPerSm = 6;  // 40 registers a thread for those load chains
// the FP64 SpMV keeps rowMac (4-load steps and a scalar tail): the predicated form measured
// slower there (C2: 74.6 vs 70.1 ms per FP64 step), the FP64 FMA rate limits it

__device__ __forceinline__ double warpSum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ void blockSumStore2(double a, double b, double* outa, double* outb) {
    __shared__ double wa[kB / 32], wb[kB / 32];
    a = warpSum(a);
    b = warpSum(b);
    if ((threadIdx.x & 31) == 0) { wa[threadIdx.x >> 5] = a; wb[threadIdx.x >> 5] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double sa = 0.0, sb = 0.0;
        for (int w = 0; w < kB / 32; ++w) { sa += wa[w]; sb += wb[w]; }
        outa[blockIdx.x] = sa;
        outb[blockIdx.x] = sb;
    }
}
// FP32 values: warp sums in FP32, per-warp results summed in FP64 (fixed order)
__device__ __forceinline__ float warpSumF(float v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ void blockSumStoreF2(float a, float b, double* outa, double* outb) {
    __shared__ double wa[kB / 32], wb[kB / 32];
    a = warpSumF(a);
    b = warpSumF(b);
    if ((threadIdx.x & 31) == 0) { wa[threadIdx.x >> 5] = a; wb[threadIdx.x >> 5] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double sa = 0.0, sb = 0.0;
        for (int w = 0; w < kB / 32; ++w) { sa += wa[w]; sb += wb[w]; }
        outa[blockIdx.x] = sa;
        outb[blockIdx.x] = sb;
    }
}
__device__ __forceinline__ void blockSumStoreF(float a, double* outa) {
    __shared__ double wa[kB / 32];
    a = warpSumF(a);
    if ((threadIdx.x & 31) == 0) wa[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sa = 0.0;
        for (int w = 0; w < kB / 32; ++w) sa += wa[w];
        outa[blockIdx.x] = sa;
    }
}
// only the leader lane of each row group holds a value: sum the groups' values (fixed order)
template <int RPB>
__device__ __forceinline__ void leaderSumStore(double v, bool leader, int group, double* out) {
    __shared__ double sm[RPB];
    if (leader) sm[group] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int g = 0; g < RPB; ++g) s += sm[g];
        out[blockIdx.x] = s;
    }
}

// single-block reduction of n partials (fixed order)
__device__ __forceinline__ double reducePartials(const double* part, int n) {
    __shared__ double ws[kB / 32];
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += part[i];
    v = warpSum(v);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    for (int w = 0; w < kB / 32; ++w) s += ws[w];
    __syncthreads();
    return s;
}

// the same sum for the block that finishes last (partials written by other blocks of this
// launch: read past L1)
__device__ __forceinline__ double reducePartialsLast(const double* part, int n) {
    __shared__ double ws[kB / 32];
    double v = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) v += __ldcg(part + i);
    v = warpSum(v);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    for (int w = 0; w < kB / 32; ++w) s += ws[w];
    __syncthreads();
    return s;
}

// true in every thread of the block that is the last of the grid to store its partial sums (each
// block fences its stores before counting itself; no block waits for another)
__device__ __forceinline__ bool lastBlock(unsigned* arrive) {
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(arrive, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    return last;
}

// the block's copy of the box-row offset table (BOX kernels)
template <bool BOX>
__device__ __forceinline__ void stageBox(int* sbox, const int* __restrict__ off, int nbox) {
    if constexpr (BOX) {
        for (int j = threadIdx.x; j < nbox; j += blockDim.x) sbox[j] = off[j];
        __syncthreads();
    }
}

// t = A p (LPR lanes per row, grid-stride over row groups) and block partial sums of p.t
template <int LPR, bool REL, bool BOX>
__global__ void __launch_bounds__(kB) k_spmv_dot(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                 const int16_t* __restrict__ coff, const uint8_t* __restrict__ box,
                                                 const int* __restrict__ boxOff, int nbox,
                                                 const double* __restrict__ val, const double* __restrict__ p,
                                                 double* __restrict__ t, double* __restrict__ part,
                                                 CgState* __restrict__ st) {
    if (st->done) return;
    __shared__ int sbox[BOX ? launch::kMaxBox : 1];
    stageBox<BOX>(sbox, boxOff, nbox);
    const int rowsPerBlock = kB / LPR;
    const int lane = threadIdx.x % LPR;
    double contrib = 0.0;
    for (int base = blockIdx.x * rowsPerBlock; base < n; base += gridDim.x * rowsPerBlock) {
        const int row = base + threadIdx.x / LPR;
        double s = 0.0;
        if (row < n) {
            auto fv = [&](int k) { return val[k]; };
            auto fx = [&](int c) { return p[c]; };
            auto fm = [&](double v, double x) { s += v * x; };
            if (BOX && box[row]) dev::rowMacBox<LPR, kUnroll>(row, ptr[row], ptr[row + 1], lane, sbox, fv, fx, fm);
            else dev::rowMac<LPR, kUnroll, REL>(row, ptr[row], ptr[row + 1], lane, col, coff, fv, fx, fm);
        }
        // every lane of the warp takes part in the shuffles (rows past n contribute 0)
        for (int o = LPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (row < n && lane == 0) {
            t[row] = s;
            contrib += s * p[row];
        }
    }
    leaderSumStore<kB / LPR>(contrib, lane == 0, threadIdx.x / LPR, part);
    // the block that finishes last forms alpha = rho / p.Ap from the partials (fixed order)
    if (lastBlock(&st->arrive)) {
        const double pAp = reducePartialsLast(part, gridDim.x);
        if (threadIdx.x == 0) {
            st->alpha = st->rho / pAp;
            st->arrive = 0;
        }
    }
}

// x += alpha p; r -= alpha t; z = dinv r; partial sums of r.r and r.z; the block that finishes
// last takes the stopping test (gsConjugateGradient::step) and forms beta = (r.z) / rho
__global__ void __launch_bounds__(kB) k_update(int n, double* __restrict__ x, double* __restrict__ r,
                                               double* __restrict__ z, const double* __restrict__ p,
                                               const double* __restrict__ t, const double* __restrict__ dinv,
                                               double* __restrict__ prr, double* __restrict__ prz,
                                               CgState* __restrict__ st) {
    if (st->done) return;
    const double alpha = st->alpha;
    double rr = 0.0, rz = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] += alpha * p[i];
        const double ri = r[i] - alpha * t[i];
        r[i] = ri;
        const double zi = dinv[i] * ri;
        z[i] = zi;
        rr += ri * ri;
        rz += ri * zi;
    }
    blockSumStore2(rr, rz, prr, prz);
    if (!lastBlock(&st->arrive)) return;
    const double rrs = reducePartialsLast(prr, gridDim.x);
    const double rzs = reducePartialsLast(prz, gridDim.x);
    if (threadIdx.x == 0) {
        st->arrive = 0;
        const double rr = rrs, rz = rzs;
        st->iters += 1;
        st->relres = sqrt(rr) / st->bnorm;
        if (st->relres < st->tol) {
            st->done = 1;
        } else if (st->iters >= st->maxit) {
            st->done = 2;
        } else {
            st->beta = rz / st->rho;
            st->rho = rz;
        }
    }
}

__global__ void __launch_bounds__(kB) k_pupd(int n, double* __restrict__ p, const double* __restrict__ z,
                                             const CgState* __restrict__ st) {
    if (st->done) return;
    const double beta = st->beta;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = z[i] + beta * p[i];
}

// start: x = 0, r = b, z = D^-1 b, p = z; partial sums of b.b and r.z
__global__ void __launch_bounds__(kB) k_init(int n, const double* __restrict__ b, double* __restrict__ x,
                                             double* __restrict__ r, double* __restrict__ z, double* __restrict__ p,
                                             const double* __restrict__ dinv, double* __restrict__ pbb,
                                             double* __restrict__ prz) {
    double bb = 0.0, rz = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double bi = b[i];
        x[i] = 0.0;
        r[i] = bi;
        const double zi = dinv[i] * bi;
        z[i] = zi;
        p[i] = zi;
        bb += bi * bi;
        rz += bi * zi;
    }
    blockSumStore2(bb, rz, pbb, prz);
}

__global__ void __launch_bounds__(kB) k_init_reduce(int nparts, const double* __restrict__ pbb,
                                                    const double* __restrict__ prz, CgState* __restrict__ st,
                                                    double tol, int maxit, double delta) {
    const double bb = reducePartials(pbb, nparts);
    const double rz = reducePartials(prz, nparts);
    if (threadIdx.x == 0) {
        st->tol = tol;
        st->maxit = maxit;
        st->iters = 0;
        st->bnorm = sqrt(bb);
        st->rho = rz;
        st->alpha = st->beta = 0.0;
        st->relres = bb > 0.0 ? 1.0 : 0.0;
        st->pause = 0;
        st->pupd_skip = 0;
        st->replacements = 0;
        st->replaced = 0;
        st->restart = 0;
        st->last_true = 1.0;
        st->delta = delta;
        st->arrive = 0;
        // zero rhs: x = 0 is the solution; x0 = 0 gives ||r||/||b|| = 1 >= tol otherwise
        st->done = (bb == 0.0 || 1.0 < tol) ? 1 : (maxit <= 0 ? 2 : 0);
    }
}

__global__ void __launch_bounds__(kB) k_dinv(int n, const int* __restrict__ diag, const double* __restrict__ val,
                                             double damping, double* __restrict__ dinv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dinv[i] = damping / val[diag[i]];
}

// ---------------------------------------------------------------------------------------------
// mixed precision: the inner PCG runs in FP32 on the operator A_hi = fl32(A); every chunk of
// iterations ends with a residual replacement r = b - (A_hi + A_lo) x evaluated in df32 from the
// FP64 iterate, so the stopping test is on the true FP64-accurate residual (iterative refinement
// with the Krylov direction kept across replacements). Dot products accumulate in FP64.

template <int LPR, bool REL, bool BOX>
__global__ void __launch_bounds__(kB, kSpmv32BlocksPerSm) k_spmv32_dot(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                   const int16_t* __restrict__ coff, const uint8_t* __restrict__ box,
                                                   const int* __restrict__ boxOff, int nbox,
                                                   const float* __restrict__ val, const float* __restrict__ p,
                                                   float* __restrict__ t, double* __restrict__ part,
                                                   const CgState* __restrict__ st) {
    if (st->done || st->pause) return;
    __shared__ int sbox[BOX ? launch::kMaxBox : 1];
    stageBox<BOX>(sbox, boxOff, nbox);
    const int rowsPerBlock = kB / LPR;
    const int lane = threadIdx.x % LPR;
    double contrib = 0.0;
    for (int base = blockIdx.x * rowsPerBlock; base < n; base += gridDim.x * rowsPerBlock) {
        const int row = base + threadIdx.x / LPR;
        float s = 0.f;
        if (row < n) {
            auto fv = [&](int k) { return val[k]; };
            auto fx = [&](int c) { return p[c]; };
            auto fm = [&](float v, float x) { s = fmaf(v, x, s); };
            if (BOX && box[row])
                dev::rowMacBoxP<LPR, kUnrollBox>(row, ptr[row], ptr[row + 1], lane, sbox, fv, fx, fm);
            else dev::rowMacP<LPR, kUnrollP, REL>(row, ptr[row], ptr[row + 1], lane, col, coff, fv, fx, fm);
        }
        for (int o = LPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (row < n && lane == 0) {
            t[row] = s;
            contrib += double(s) * double(p[row]);
        }
    }
    leaderSumStore<kB / LPR>(contrib, lane == 0, threadIdx.x / LPR, part);
}

__global__ void __launch_bounds__(kB) k_alpha_m(int nparts, const double* __restrict__ part, CgState* __restrict__ st) {
    pdlWait();
    pdlTrigger();
    if (st->done || st->pause) return;
    const double pAp = reducePartials(part, nparts);
    if (threadIdx.x == 0) st->alpha = st->rho / pAp;
}

__global__ void __launch_bounds__(kB) k_update32(int n, float* __restrict__ dx, float* __restrict__ r,
                                                 float* __restrict__ z, const float* __restrict__ p,
                                                 const float* __restrict__ t, const float* __restrict__ dinv,
                                                 double* __restrict__ prr, double* __restrict__ prz,
                                                 const CgState* __restrict__ st) {
    if (st->done || st->pause) return;
    const float alpha = float(st->alpha);
    float rr = 0.f, rz = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        dx[i] = fmaf(alpha, p[i], dx[i]);
        const float ri = fmaf(-alpha, t[i], r[i]);
        r[i] = ri;
        const float zi = dinv[i] * ri;
        z[i] = zi;
        rr = fmaf(ri, ri, rr);
        rz = fmaf(ri, zi, rz);
    }
    blockSumStoreF2(rr, rz, prr, prz);
}

// k_update32 with the stopping / pause test and beta of k_beta_m formed by the block that stores
// its partials last (the half-diagonal path, whose product forms alpha the same way); a skipped
// iteration marks the direction update as skipped, as k_beta_m does
__global__ void __launch_bounds__(kB) k_update32b(int n, float* __restrict__ dx, float* __restrict__ r,
                                                  float* __restrict__ z, const float* __restrict__ p,
                                                  const float* __restrict__ t, const float* __restrict__ dinv,
                                                  double* __restrict__ prr, double* __restrict__ prz,
                                                  CgState* __restrict__ st) {
    if (st->done || st->pause) {
        if (blockIdx.x == 0 && threadIdx.x == 0) st->pupd_skip = 1;
        return;
    }
    const float alpha = float(st->alpha);
    float rr = 0.f, rz = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        dx[i] = fmaf(alpha, p[i], dx[i]);
        const float ri = fmaf(-alpha, t[i], r[i]);
        r[i] = ri;
        const float zi = dinv[i] * ri;
        z[i] = zi;
        rr = fmaf(ri, ri, rr);
        rz = fmaf(ri, zi, rz);
    }
    blockSumStoreF2(rr, rz, prr, prz);
    if (!lastBlock(&st->arrive)) return;
    const double rrs = reducePartialsLast(prr, gridDim.x);
    const double rzs = reducePartialsLast(prz, gridDim.x);
    if (threadIdx.x == 0) {
        st->arrive = 0;
        st->pupd_skip = 0;
        st->iters += 1;
        st->relres = sqrt(rrs) / st->bnorm;
        if (st->relres < st->tol || st->relres < st->delta * st->last_true || st->iters >= st->maxit) st->pause = 1;
        st->beta = rzs / st->rho;
        st->rho = rzs;
    }
}

// k_update32b over four consecutive entries per thread (16-byte loads and stores of 16-byte
// aligned vectors; thread 0 also takes the n mod 4 last entries): a quarter of the threads and of
// the block partials that the last block reduces. Each entry's arithmetic is that of k_update32b;
// the dot products sum the four entries of a thread in order.
__global__ void __launch_bounds__(kB) k_update32b4(int n, float* __restrict__ dx, float* __restrict__ r,
                                                   float* __restrict__ z, const float* __restrict__ p,
                                                   const float* __restrict__ t, const float* __restrict__ dinv,
                                                   double* __restrict__ prr, double* __restrict__ prz,
                                                   CgState* __restrict__ st) {
    pdlWait();
    if (st->done || st->pause) {
        if (blockIdx.x == 0 && threadIdx.x == 0) st->pupd_skip = 1;
        return;
    }
    const float alpha = float(st->alpha);
    float rr = 0.f, rz = 0.f;
    auto one = [&](float& x, float& ri, float& zi, float pi, float ti, float di) {
        x = fmaf(alpha, pi, x);
        ri = fmaf(-alpha, ti, ri);
        zi = di * ri;
        rr = fmaf(ri, ri, rr);
        rz = fmaf(ri, zi, rz);
    };
    const int n4 = n >> 2;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x) {
        float4 xv = reinterpret_cast<float4*>(dx)[i], rv = reinterpret_cast<float4*>(r)[i], zv;
        const float4 pv = reinterpret_cast<const float4*>(p)[i], tv = reinterpret_cast<const float4*>(t)[i],
                     dv = reinterpret_cast<const float4*>(dinv)[i];
        one(xv.x, rv.x, zv.x, pv.x, tv.x, dv.x);
        one(xv.y, rv.y, zv.y, pv.y, tv.y, dv.y);
        one(xv.z, rv.z, zv.z, pv.z, tv.z, dv.z);
        one(xv.w, rv.w, zv.w, pv.w, tv.w, dv.w);
        reinterpret_cast<float4*>(dx)[i] = xv;
        reinterpret_cast<float4*>(r)[i] = rv;
        reinterpret_cast<float4*>(z)[i] = zv;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        for (int i = n4 << 2; i < n; ++i) {
            float zi;
            one(dx[i], r[i], zi, p[i], t[i], dinv[i]);
            z[i] = zi;
        }
    pdlTrigger();
    blockSumStoreF2(rr, rz, prr, prz);
    if (!lastBlock(&st->arrive)) return;
    const double rrs = reducePartialsLast(prr, gridDim.x);
    const double rzs = reducePartialsLast(prz, gridDim.x);
    if (threadIdx.x == 0) {
        st->arrive = 0;
        st->pupd_skip = 0;
        st->iters += 1;
        st->relres = sqrt(rrs) / st->bnorm;
        if (st->relres < st->tol || st->relres < st->delta * st->last_true || st->iters >= st->maxit) st->pause = 1;
        st->beta = rzs / st->rho;
        st->rho = rzs;
    }
}

// p = z + beta p over four entries per thread (the tail by thread 0), as k_pupd32
__global__ void __launch_bounds__(kB) k_pupd32_4(int n, float* __restrict__ p, const float* __restrict__ z,
                                                 const CgState* __restrict__ st) {
    pdlWait();
    pdlTrigger();
    if (st->done || st->pupd_skip) return;
    const float beta = float(st->beta);
    const int n4 = n >> 2;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += gridDim.x * blockDim.x) {
        float4 pv = reinterpret_cast<float4*>(p)[i];
        const float4 zv = reinterpret_cast<const float4*>(z)[i];
        pv.x = fmaf(beta, pv.x, zv.x);
        pv.y = fmaf(beta, pv.y, zv.y);
        pv.z = fmaf(beta, pv.z, zv.z);
        pv.w = fmaf(beta, pv.w, zv.w);
        reinterpret_cast<float4*>(p)[i] = pv;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        for (int i = n4 << 2; i < n; ++i) p[i] = fmaf(beta, p[i], z[i]);
}

__global__ void __launch_bounds__(kB) k_beta_m(int nparts, const double* __restrict__ prr,
                                               const double* __restrict__ prz, CgState* __restrict__ st) {
    if (st->done || st->pause) {
        if (threadIdx.x == 0) st->pupd_skip = 1;
        return;
    }
    const double rr = reducePartials(prr, nparts);
    const double rz = reducePartials(prz, nparts);
    if (threadIdx.x == 0) {
        st->pupd_skip = 0;
        st->iters += 1;
        st->relres = sqrt(rr) / st->bnorm;  // recursive estimate; the true value comes at replacement
        // replace the residual once the recursion has gained delta (the FP32 recursion cannot
        // follow the true residual much further), at the tolerance, or at the iteration limit
        if (st->relres < st->tol || st->relres < st->delta * st->last_true || st->iters >= st->maxit) st->pause = 1;
        st->beta = rz / st->rho;
        st->rho = rz;
    }
}

__global__ void __launch_bounds__(kB) k_pupd32(int n, float* __restrict__ p, const float* __restrict__ z,
                                               const CgState* __restrict__ st) {
    if (st->done || st->pupd_skip) return;
    const float beta = float(st->beta);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        p[i] = fmaf(beta, p[i], z[i]);
}

// x += dx (FP64), dx = 0, and the df32 split of x for the residual SpMV
__global__ void __launch_bounds__(kB) k_xupd(int n, double* __restrict__ x, float* __restrict__ dx,
                                             float* __restrict__ xhi, float* __restrict__ xlo,
                                             const CgState* __restrict__ st) {
    if (st->done || !st->pause) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double xi = x[i] + double(dx[i]);
        x[i] = xi;
        dx[i] = 0.f;
        const df32 v(xi);
        xhi[i] = v.hi;
        xlo[i] = v.lo;
    }
}

// r = b - (A_hi + A_lo) x with df32 products and compensated accumulation; partial sums of r.r
// (box rows take their column offsets from the shared table, as in the FP32 SpMV: the same slots in
// the same order, 8 instead of 10 bytes per non-zero)
template <int LPR, bool REL, bool BOX>
__global__ void __launch_bounds__(kB) k_resid_df(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                 const int16_t* __restrict__ coff, const uint8_t* __restrict__ box,
                                                 const int* __restrict__ boxOff, int nbox,
                                                 const float* __restrict__ hi, const float* __restrict__ lo,
                                                 const float* __restrict__ xhi, const float* __restrict__ xlo,
                                                 const double* __restrict__ b, double* __restrict__ r,
                                                 double* __restrict__ part, const CgState* __restrict__ st) {
    if (st->done || !st->pause) return;
    __shared__ int sbox[BOX ? launch::kMaxBox : 1];
    stageBox<BOX>(sbox, boxOff, nbox);
    const int rowsPerBlock = kB / LPR;
    const int lane = threadIdx.x % LPR;
    double contrib = 0.0;
    for (int base = blockIdx.x * rowsPerBlock; base < n; base += gridDim.x * rowsPerBlock) {
        const int row = base + threadIdx.x / LPR;
        Dot2 acc;
        if (row < n) {
            auto fv = [&](int k) { return df32(hi[k], lo[k]); };
            auto fx = [&](int c) { return df32(xhi[c], xlo[c]); };
            auto fm = [&](df32 v, df32 x) { acc.mac(v, x); };
            if (BOX && box[row]) dev::rowMacBox<LPR, kUnroll>(row, ptr[row], ptr[row + 1], lane, sbox, fv, fx, fm);
            else dev::rowMac<LPR, kUnroll, REL>(row, ptr[row], ptr[row + 1], lane, col, coff, fv, fx, fm);
        }
        df32 y = acc.result();
        for (int o = LPR / 2; o > 0; o >>= 1) {
            df32 oth(__shfl_xor_sync(0xffffffffu, y.hi, o), __shfl_xor_sync(0xffffffffu, y.lo, o));
            y = y + oth;
        }
        if (row < n && lane == 0) {
            const double ri = b[row] - y.toDouble();
            r[row] = ri;
            contrib += ri * ri;
        }
    }
    leaderSumStore<kB / LPR>(contrib, lane == 0, threadIdx.x / LPR, part);
}

__global__ void __launch_bounds__(kB) k_rel_check(int nparts, const double* __restrict__ part,
                                                  CgState* __restrict__ st) {
    if (st->done || !st->pause) return;
    const double rr = reducePartials(part, nparts);
    if (threadIdx.x == 0) {
        const double rec = st->relres;  // the recursive estimate that triggered the replacement
        st->replacements += 1;
        st->relres = sqrt(rr) / st->bnorm;
        st->restart = st->relres > 4.0 * rec ? 1 : 0;
        st->last_true = st->relres;
        if (st->relres < st->tol) st->done = 1;
        else if (st->iters >= st->maxit) st->done = 2;
        else {
            st->pause = 0;
            st->replaced = 1;
        }
    }
}

// restart the FP32 recursion from the replaced residual: r32 = fl32(r), z = D^-1 r32, partial r.z;
// the search direction is kept unless the replacement moved the residual a lot
__global__ void __launch_bounds__(kB) k_r32(int n, const double* __restrict__ r, float* __restrict__ r32,
                                            float* __restrict__ z, float* __restrict__ p,
                                            const float* __restrict__ dinv, double* __restrict__ prz,
                                            const CgState* __restrict__ st) {
    if (!st->replaced) return;
    const int restart = st->restart;
    float rz = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float ri = float(r[i]);
        r32[i] = ri;
        const float zi = dinv[i] * ri;
        z[i] = zi;
        if (restart) p[i] = zi;
        rz = fmaf(ri, zi, rz);
    }
    blockSumStoreF(rz, prz);
}

__global__ void __launch_bounds__(kB) k_rho(int nparts, const double* __restrict__ prz, CgState* __restrict__ st) {
    if (!st->replaced) return;
    const double rz = reducePartials(prz, nparts);
    if (threadIdx.x == 0) {
        st->rho = rz;
        st->replaced = 0;
    }
}

// start: x = 0, dx = 0, r = b, r32 = fl32(b), z = D^-1 r32, p = z; partial b.b and r.z
__global__ void __launch_bounds__(kB) k_init_m(int n, const double* __restrict__ b, double* __restrict__ x,
                                               double* __restrict__ r, float* __restrict__ dx, float* __restrict__ r32,
                                               float* __restrict__ z, float* __restrict__ p,
                                               const float* __restrict__ dinv, double* __restrict__ pbb,
                                               double* __restrict__ prz) {
    double bb = 0.0, rz = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double bi = b[i];
        x[i] = 0.0;
        r[i] = bi;
        dx[i] = 0.f;
        const float ri = float(bi);
        r32[i] = ri;
        const float zi = dinv[i] * ri;
        z[i] = zi;
        p[i] = zi;
        bb += bi * bi;
        rz += double(ri) * double(zi);
    }
    blockSumStore2(bb, rz, pbb, prz);
}

__global__ void __launch_bounds__(kB) k_dinv32(int n, const int* __restrict__ diag, const float* __restrict__ val,
                                               float* __restrict__ dinv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dinv[i] = 1.0f / val[diag[i]];
}

inline unsigned g1(long long n) { return unsigned((n + kB - 1) / kB); }

// one warp per row: box[row] = 1 iff the row has nbox slots with columns row + off[j]
__global__ void __launch_bounds__(kB) k_box_flags(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                  const int* __restrict__ off, int nbox, uint8_t* __restrict__ box,
                                                  unsigned long long* __restrict__ count) {
    const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= n) return;  // whole warps
    const int row = int(warp);
    const int kb = ptr[row];
    bool ok = ptr[row + 1] - kb == nbox;
    if (ok)
        for (int j = lane; j < nbox; j += 32) ok = ok && col[kb + j] == row + off[j];
    ok = __all_sync(0xffffffffu, ok);
    if (lane == 0) {
        box[row] = ok ? 1 : 0;
        if (ok) atomicAdd(count, 1ULL);
    }
}

}  // namespace

namespace launch {

// vector kernels run grid-stride on at most kMaxVecBlocks blocks, so dot products leave few partials
constexpr int kMaxVecBlocks = 512;
int cgPartials(int n) {
    const int g = int(g1(n > 0 ? n : 1));
    return g < kMaxVecBlocks ? g : kMaxVecBlocks;
}

void jacobiDiag(int n, const int* diag, const double* val, double damping, double* dinv, cudaStream_t s) {
    if (n > 0) k_dinv<<<g1(n), kB, 0, s>>>(n, diag, val, damping, dinv);
}

void cgInit(const CgBuffers& B, double tol, int maxit, cudaStream_t s) {
    const int np = cgPartials(B.n);
    k_init<<<np, kB, 0, s>>>(B.n, B.b, B.x, B.r, B.z, B.p, B.dinv, B.part0, B.part1);
    k_init_reduce<<<1, kB, 0, s>>>(np, B.part0, B.part1, B.st, tol, maxit, B.delta);
}

// launch a row kernel template for the lanes-per-row and column-format choice of B
// kernels with the box-row template flag: <LPR, REL, BOX>
#define GSGPU_BOX_ROW(KERNEL, L, NB, ...)                                                               \
    do {                                                                                                \
        const bool rel = B.coff != nullptr;                                                             \
        if (B.box) {                                                                                    \
            if (rel) KERNEL<L, true, true><<<NB, kB, 0, s>>>(__VA_ARGS__);                              \
            else KERNEL<L, false, true><<<NB, kB, 0, s>>>(__VA_ARGS__);                                 \
        } else {                                                                                        \
            if (rel) KERNEL<L, true, false><<<NB, kB, 0, s>>>(__VA_ARGS__);                             \
            else KERNEL<L, false, false><<<NB, kB, 0, s>>>(__VA_ARGS__);                                \
        }                                                                                               \
    } while (0)
#define GSGPU_BOX_DISPATCH(KERNEL, NB, ...)                                                             \
    do {                                                                                                \
        switch (B.lanes_per_row) {                                                                      \
            case 4: GSGPU_BOX_ROW(KERNEL, 4, NB, __VA_ARGS__); break;                                   \
            case 8: GSGPU_BOX_ROW(KERNEL, 8, NB, __VA_ARGS__); break;                                   \
            case 16: GSGPU_BOX_ROW(KERNEL, 16, NB, __VA_ARGS__); break;                                 \
            default: GSGPU_BOX_ROW(KERNEL, 32, NB, __VA_ARGS__); break;                                 \
        }                                                                                               \
    } while (0)

void cgSpmv(const CgBuffers& B, cudaStream_t s) {
    const int nb = spmvPartials(B.n, B.lanes_per_row);
    GSGPU_BOX_DISPATCH(k_spmv_dot, nb, B.n, B.ptr, B.col, B.coff, B.box, B.box_off, B.nbox, B.val, B.p, B.t, B.part2,
                       B.st);
}

void cgRest(const CgBuffers& B, cudaStream_t s) {
    const int np = cgPartials(B.n);
    k_update<<<np, kB, 0, s>>>(B.n, B.x, B.r, B.z, B.p, B.t, B.dinv, B.part0, B.part1, B.st);
    k_pupd<<<np, kB, 0, s>>>(B.n, B.p, B.z, B.st);
}

void cgIteration(const CgBuffers& B, cudaStream_t s) {
    cgSpmv(B, s);
    cgRest(B, s);
}

void boxFlags(int n, const int* ptr, const int* col, const int* off, int nbox, uint8_t* box,
              unsigned long long* count, cudaStream_t s) {
    if (n <= 0) return;
    const long long threads = 32LL * n;
    k_box_flags<<<unsigned((threads + kB - 1) / kB), kB, 0, s>>>(n, ptr, col, off, nbox, box, count);
}

int spmvPartials(int n, int lanes_per_row) {
    const int rows_per_block = kB / lanes_per_row;
    const int nb = (n + rows_per_block - 1) / rows_per_block;
    return nb < kMaxSpmvBlocks ? (nb > 0 ? nb : 1) : kMaxSpmvBlocks;
}

void jacobiDiag32(int n, const int* diag, const float* val_hi, float* dinv32, cudaStream_t s) {
    if (n > 0) k_dinv32<<<g1(n), kB, 0, s>>>(n, diag, val_hi, dinv32);
}

void mixedInit(const CgBuffers& B, double tol, int maxit, cudaStream_t s) {
    const int np = cgPartials(B.n);
    k_init_m<<<np, kB, 0, s>>>(B.n, B.b, B.x, B.r, B.dx32, B.r32, B.z32, B.p32, B.dinv32, B.part0, B.part1);
    k_init_reduce<<<1, kB, 0, s>>>(np, B.part0, B.part1, B.st, tol, maxit, B.delta);
}

// FP32 SpMV grid: kSpmv32BlocksPerSm resident blocks on every SM
int spmv32Partials(int n, int lanes_per_row) {
    return std::min(spmvPartials(n, lanes_per_row), 152 * kSpmv32BlocksPerSm);
}

// block partials left by the inner FP32 product
int mixedSpmvPartials(const CgBuffers& B) {
    return B.sdia.d ? sdiaPartials(B.sdia) : spmv32Partials(B.n, B.lanes_per_row);
}

void mixedSpmv(const CgBuffers& B, cudaStream_t s) {
    if (B.sdia.d) {
        sdiaSpmv(B.sdia, B.p32, B.t32, B.part2, B.st, s);
        return;
    }
    const int nb = spmv32Partials(B.n, B.lanes_per_row);
    GSGPU_BOX_DISPATCH(k_spmv32_dot, nb, B.n, B.ptr, B.col, B.coff, B.box, B.box_off, B.nbox, B.val_hi, B.p32, B.t32,
                       B.part2, B.st);
}

void mixedRest(const CgBuffers& B, cudaStream_t s) {
    const int np = cgPartials(B.n);
    const int nb = mixedSpmvPartials(B);
    if (B.sdia.d) {  // beta from the update's last block (measured: -3 us per iteration on the C2 volume;
                     // alpha from the product's last block measured +15 us and stays a kernel)
        launchMaybePdl(k_alpha_m, dim3(1), dim3(kB), s, B.pdl && B.vec4, nb, B.part2, B.st);
        if (B.vec4) {  // 16-byte aligned vectors: four entries per thread
            const int np4 = std::max(1, (B.n / 4 + kB - 1) / kB);
            launchMaybePdl(k_update32b4, dim3(np4), dim3(kB), s, B.pdl, B.n, B.dx32, B.r32, B.z32, B.p32, B.t32,
                           B.dinv32, B.part0, B.part1, B.st);
            launchMaybePdl(k_pupd32_4, dim3(np4), dim3(kB), s, B.pdl, B.n, B.p32, B.z32, B.st);
            return;
        }
        k_update32b<<<np, kB, 0, s>>>(B.n, B.dx32, B.r32, B.z32, B.p32, B.t32, B.dinv32, B.part0, B.part1, B.st);
        k_pupd32<<<np, kB, 0, s>>>(B.n, B.p32, B.z32, B.st);
        return;
    }
    k_alpha_m<<<1, kB, 0, s>>>(nb, B.part2, B.st);
    k_update32<<<np, kB, 0, s>>>(B.n, B.dx32, B.r32, B.z32, B.p32, B.t32, B.dinv32, B.part0, B.part1, B.st);
    k_beta_m<<<1, kB, 0, s>>>(np, B.part0, B.part1, B.st);
    k_pupd32<<<np, kB, 0, s>>>(B.n, B.p32, B.z32, B.st);
}

void mixedIteration(const CgBuffers& B, cudaStream_t s) {
    mixedSpmv(B, s);
    mixedRest(B, s);
}

void mixedReplace(const CgBuffers& B, cudaStream_t s) {
    const int np = cgPartials(B.n);
    const int nb = spmvPartials(B.n, B.lanes_per_row);
    k_xupd<<<np, kB, 0, s>>>(B.n, B.x, B.dx32, B.xhi, B.xlo, B.st);
    GSGPU_BOX_DISPATCH(k_resid_df, nb, B.n, B.ptr, B.col, B.coff, B.box, B.box_off, B.nbox, B.val_hi, B.val_lo, B.xhi,
                       B.xlo, B.b, B.r, B.part2, B.st);
    k_rel_check<<<1, kB, 0, s>>>(nb, B.part2, B.st);
    k_r32<<<np, kB, 0, s>>>(B.n, B.r, B.r32, B.z32, B.p32, B.dinv32, B.part1, B.st);
    k_rho<<<1, kB, 0, s>>>(np, B.part1, B.st);
}

}  // namespace launch
}  // namespace gsgpu
