// sm_103a kernels of the h-multigrid V-cycle (gsMultiGridOp::multiGridStep,
// src/gsMultiGrid/gsMultiGrid.hpp:147-201) and of the CG driven by it (gsConjugateGradient,
// src/gsSolver/gsConjugateGradient.hpp:19-84). The V-cycle is templated on its working precision
// T: FP64 for the plain path, FP32 for the mixed path. The outer CG, its residual and its dot
// products are FP64 in both.
//
// V-cycle on level l (level 0 finest), started from x = 0:
//   nu1 damped Jacobi sweeps x += w D^-1 (b - A x)  (the first one is x = w D^-1 b);
//   r = A x - b; b_c = P^T r; x_c = V(l+1, b_c); x -= P x_c; nu2 sweeps.
// The coarsest level is solved by Jacobi-PCG to a relative tolerance under an iteration cap
// instead of the reference's sparse Cholesky factor: that keeps the coarse solve on the device
// with no sequential triangular solves. The outer CG uses the Polak-Ribiere beta
// (r_k - r_{k-1}).z_k / r_{k-1}.z_{k-1}, which stays a CG for a fixed preconditioner and is robust
// when the coarse solve leaves a small inexactness.
#include <algorithm>
#include <cstdint>

#include "df32.cuh"
#include "kernels_mg.h"
#include "spmv_row.cuh"

namespace gsgpu {
namespace {

constexpr int kB = 256;
// grid cap: 8 resident blocks of 256 threads on each of the 152 SMs (full occupancy)
constexpr int kMaxBlocks = 8 * 152;

constexpr int kUnroll = 4;  // independent (value, column) -> x load chains per lane

template <typename T>
__device__ __forceinline__ T warpSum(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// out[blockIdx.x] = sum of v over the block (fixed order)
__device__ __forceinline__ void blockSum(double v, double* out) {
    __shared__ double ws[kB / 32];
    v = warpSum(v);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kB / 32; ++w) s += ws[w];
        out[blockIdx.x] = s;
    }
}
// every thread gets the sum of part[0..n)
__device__ __forceinline__ double blockReduce(const double* part, int n) {
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

__device__ __forceinline__ bool stopped(const CgState* a, const CgState* b) {
    return (a && a->done) || (b && b->done);
}

// (A x)_row with LPR lanes per row, then epi(row, value) on the row's lane 0. All threads of a
// block run the same number of outer iterations, so the full-warp shuffles are convergent.
template <typename T, int LPR, bool REL, class Val, class Epi>
__device__ __forceinline__ void rowLoop(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                        const int16_t* __restrict__ coff, Val val, const T* __restrict__ x, Epi epi) {
    const int rowsPerBlock = kB / LPR;
    const int lane = threadIdx.x % LPR;
    for (int base = blockIdx.x * rowsPerBlock; base < n; base += gridDim.x * rowsPerBlock) {
        const int row = base + threadIdx.x / LPR;
        T s = T(0);
        if (row < n)
            dev::rowMac<LPR, kUnroll, REL>(row, ptr[row], ptr[row + 1], lane, col, coff, val,
                                           [&](int c) { return x[c]; }, [&](T v, T xv) { s += v * xv; });
        for (int o = LPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (row < n && lane == 0) epi(row, s);
    }
}

// damped Jacobi sweep xo = xi + w D^-1 (b - A xi); zero start (xi = 0): xo = w D^-1 b
template <typename T, int LPR, bool REL>
__global__ void __launch_bounds__(kB) k_jacobi(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                               const int16_t* __restrict__ coff, const T* __restrict__ val,
                                               const T* __restrict__ dinv, T w, const T* __restrict__ b,
                                               const T* __restrict__ xi, T* __restrict__ xo, int zero,
                                               const CgState* __restrict__ outer) {
    if (stopped(outer, nullptr)) return;
    if (zero) {
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
            xo[i] = w * dinv[i] * b[i];
        return;
    }
    rowLoop<T, LPR, REL>(n, ptr, col, coff, [&](int k) { return val[k]; }, xi,
                         [&](int row, T ax) { xo[row] = xi[row] + w * dinv[row] * (b[row] - ax); });
}

// r = A x - b
template <typename T, int LPR, bool REL>
__global__ void __launch_bounds__(kB) k_resid_mg(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                 const int16_t* __restrict__ coff, const T* __restrict__ val,
                                                 const T* __restrict__ x, const T* __restrict__ b, T* __restrict__ r,
                                                 const CgState* __restrict__ outer) {
    if (stopped(outer, nullptr)) return;
    rowLoop<T, LPR, REL>(n, ptr, col, coff, [&](int k) { return val[k]; }, x,
                         [&](int row, T ax) { r[row] = ax - b[row]; });
}

// y = M x (restriction with M = P^T) or y -= M x (prolongation and correction with M = P)
template <typename T, int LPR>
__global__ void __launch_bounds__(kB) k_transfer(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                 const T* __restrict__ val, const T* __restrict__ x,
                                                 T* __restrict__ y, int sub, T scale,
                                                 const CgState* __restrict__ outer) {
    if (stopped(outer, nullptr)) return;
    rowLoop<T, LPR, false>(n, ptr, col, nullptr, [&](int k) { return val[k]; }, x, [&](int row, T ax) {
        if (sub) y[row] -= scale * ax;
        else y[row] = ax;
    });
}

template <typename T>
__global__ void __launch_bounds__(kB) k_dinv_mg(int n, const int* __restrict__ diag, const T* __restrict__ val,
                                                T* __restrict__ dinv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dinv[i] = T(1) / val[diag[i]];
}

template <typename Ti, typename To>
__global__ void __launch_bounds__(kB) k_cast(int n, const Ti* __restrict__ in, To* __restrict__ out,
                                             const CgState* __restrict__ outer) {
    if (stopped(outer, nullptr)) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = To(in[i]);
}

// --------------------------------------------------------------------------------------------
// coarsest level: Jacobi-PCG from x = 0 with its own state (reductions in FP64)

template <typename T>
__global__ void __launch_bounds__(kB) k_ccg_init(int n, const T* __restrict__ b, T* __restrict__ x, T* __restrict__ r,
                                                 T* __restrict__ z, T* __restrict__ p, const T* __restrict__ dinv,
                                                 double* __restrict__ pbb, double* __restrict__ prz,
                                                 const CgState* __restrict__ outer) {
    if (stopped(outer, nullptr)) return;
    double bb = 0.0, rz = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const T bi = b[i];
        x[i] = T(0);
        r[i] = bi;
        const T zi = dinv[i] * bi;
        z[i] = zi;
        p[i] = zi;
        bb += double(bi) * double(bi);
        rz += double(bi) * double(zi);
    }
    blockSum(bb, pbb);
    __syncthreads();
    blockSum(rz, prz);
}

__global__ void __launch_bounds__(kB) k_ccg_init_reduce(int np, const double* __restrict__ pbb,
                                                        const double* __restrict__ prz, CgState* __restrict__ st,
                                                        double tol, const CgState* __restrict__ outer) {
    if (stopped(outer, nullptr)) return;
    const double bb = blockReduce(pbb, np);
    const double rz = blockReduce(prz, np);
    if (threadIdx.x == 0) {
        st->bnorm = sqrt(bb);
        st->rho = rz;
        st->tol = tol;
        st->iters = 0;
        st->done = (bb == 0.0) ? 1 : 0;
    }
}

template <typename T, int LPR, bool REL>
__global__ void __launch_bounds__(kB) k_ccg_spmv(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                 const int16_t* __restrict__ coff, const T* __restrict__ val,
                                                 const T* __restrict__ p, T* __restrict__ t, double* __restrict__ part,
                                                 const CgState* __restrict__ st, const CgState* __restrict__ outer) {
    if (stopped(st, outer)) return;
    double contrib = 0.0;
    rowLoop<T, LPR, REL>(n, ptr, col, coff, [&](int k) { return val[k]; }, p, [&](int row, T ax) {
        t[row] = ax;
        contrib += double(ax) * double(p[row]);
    });
    blockSum(contrib, part);
}

template <typename T>
__global__ void __launch_bounds__(kB) k_ccg_update(int n, int nparts_spmv, const double* __restrict__ pspmv,
                                                   T* __restrict__ x, T* __restrict__ r, T* __restrict__ z,
                                                   const T* __restrict__ p, const T* __restrict__ t,
                                                   const T* __restrict__ dinv, double* __restrict__ prr,
                                                   double* __restrict__ prz, const CgState* __restrict__ st,
                                                   const CgState* __restrict__ outer) {
    if (stopped(st, outer)) return;
    // every block reduces the SpMV partials itself: alpha needs no launch of its own
    const double pAp = blockReduce(pspmv, nparts_spmv);
    const T alpha = T(st->rho / pAp);
    double rr = 0.0, rz = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] += alpha * p[i];
        const T ri = r[i] - alpha * t[i];
        r[i] = ri;
        const T zi = dinv[i] * ri;
        z[i] = zi;
        rr += double(ri) * double(ri);
        rz += double(ri) * double(zi);
    }
    blockSum(rr, prr);
    __syncthreads();
    blockSum(rz, prz);
}

__global__ void __launch_bounds__(kB) k_ccg_beta(int np, const double* __restrict__ prr, const double* __restrict__ prz,
                                                 CgState* __restrict__ st, const CgState* __restrict__ outer) {
    if (stopped(st, outer)) return;
    const double rr = blockReduce(prr, np);
    const double rz = blockReduce(prz, np);
    if (threadIdx.x == 0) {
        st->iters += 1;
        if (sqrt(rr) <= st->tol * st->bnorm) st->done = 1;
        st->beta = rz / st->rho;
        st->rho = rz;
    }
}

template <typename T>
__global__ void __launch_bounds__(kB) k_ccg_pupd(int n, T* __restrict__ p, const T* __restrict__ z,
                                                 const CgState* __restrict__ st, const CgState* __restrict__ outer) {
    if (stopped(st, outer)) return;
    const T beta = T(st->beta);
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = z[i] + beta * p[i];
}

// --------------------------------------------------------------------------------------------
// outer flexible PCG (FP64)

__global__ void __launch_bounds__(kB) k_mg_start(int n, const double* __restrict__ b, double* __restrict__ x,
                                                 double* __restrict__ r, double* __restrict__ rold,
                                                 double* __restrict__ p, double* __restrict__ pbb) {
    double bb = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double bi = b[i];
        x[i] = 0.0;
        r[i] = bi;
        rold[i] = bi;  // the first Polak-Ribiere beta is then 0
        p[i] = 0.0;
        bb += bi * bi;
    }
    blockSum(bb, pbb);
}

__global__ void __launch_bounds__(kB) k_mg_start_reduce(int np, const double* __restrict__ pbb, CgState* __restrict__ st,
                                                        double tol, int maxit) {
    const double bb = blockReduce(pbb, np);
    if (threadIdx.x == 0) {
        st->bnorm = sqrt(bb);
        st->tol = tol;
        st->maxit = maxit;
        st->iters = 0;
        st->relres = bb > 0 ? 1.0 : 0.0;
        st->done = bb == 0.0 ? 1 : 0;
        st->rho = 1.0;
        st->beta = 0.0;
    }
}

// partial sums of r.z and (r - r_old).z
template <typename Tz>
__global__ void __launch_bounds__(kB) k_mg_dots(int n, const double* __restrict__ r, const double* __restrict__ rold,
                                                const Tz* __restrict__ z, double* __restrict__ prz,
                                                double* __restrict__ pdz, const CgState* __restrict__ st) {
    if (stopped(st, nullptr)) return;
    double rz = 0.0, dz = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double zi = double(z[i]);
        const double ri = r[i];
        rz += ri * zi;
        dz += (ri - rold[i]) * zi;
    }
    blockSum(rz, prz);
    __syncthreads();
    blockSum(dz, pdz);
}

__global__ void __launch_bounds__(kB) k_mg_beta(int np, const double* __restrict__ prz, const double* __restrict__ pdz,
                                                CgState* __restrict__ st) {
    if (stopped(st, nullptr)) return;
    const double rz = blockReduce(prz, np);
    const double dz = blockReduce(pdz, np);
    if (threadIdx.x == 0) {
        st->beta = dz / st->rho;
        st->rho = rz;
    }
}

template <typename Tz>
__global__ void __launch_bounds__(kB) k_mg_pupd(int n, double* __restrict__ p, const Tz* __restrict__ z,
                                                float* __restrict__ phi, float* __restrict__ plo,
                                                const CgState* __restrict__ st) {
    if (stopped(st, nullptr)) return;
    const double beta = st->beta;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double pi = double(z[i]) + beta * p[i];
        p[i] = pi;
        if (phi) {
            const df32 v(pi);
            phi[i] = v.hi;
            plo[i] = v.lo;
        }
    }
}

// t = A p and partial sums of p.t; A = val or hi + lo
// (the hi + lo form multiplies double-floats on the FP32 pipe with compensated accumulation, as
// the residual replacement of the mixed CG does: FP64 products would be FP64-pipe bound on GB300)
template <int LPR, bool REL, bool SPLIT>
__global__ void __launch_bounds__(kB) k_mg_spmv(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                const int16_t* __restrict__ coff, const double* __restrict__ val,
                                                const float* __restrict__ hi, const float* __restrict__ lo,
                                                const float* __restrict__ phi, const float* __restrict__ plo,
                                                const double* __restrict__ p, double* __restrict__ t,
                                                double* __restrict__ part, const CgState* __restrict__ st) {
    if (stopped(st, nullptr)) return;
    double contrib = 0.0;
    if constexpr (SPLIT) {
        const int rowsPerBlock = kB / LPR;
        const int lane = threadIdx.x % LPR;
        for (int base = blockIdx.x * rowsPerBlock; base < n; base += gridDim.x * rowsPerBlock) {
            const int row = base + threadIdx.x / LPR;
            Dot2 acc;
            if (row < n)
                dev::rowMac<LPR, kUnroll, REL>(
                    row, ptr[row], ptr[row + 1], lane, col, coff, [&](int k) { return df32(hi[k], lo[k]); },
                    [&](int c) { return df32(phi[c], plo[c]); }, [&](df32 a, df32 x) { acc.mac(a, x); });
            df32 y = acc.result();
            for (int o = LPR / 2; o > 0; o >>= 1) {
                const df32 oth(__shfl_xor_sync(0xffffffffu, y.hi, o), __shfl_xor_sync(0xffffffffu, y.lo, o));
                y = y + oth;
            }
            if (row < n && lane == 0) {
                const double ax = y.toDouble();
                t[row] = ax;
                contrib += ax * p[row];
            }
        }
    } else {
        rowLoop<double, LPR, REL>(n, ptr, col, coff, [&](int k) { return val[k]; }, p, [&](int row, double ax) {
            t[row] = ax;
            contrib += ax * p[row];
        });
    }
    blockSum(contrib, part);
}

__global__ void __launch_bounds__(kB) k_mg_update(int n, int nparts_spmv, const double* __restrict__ pspmv,
                                                  double* __restrict__ x, double* __restrict__ r,
                                                  double* __restrict__ rold, const double* __restrict__ p,
                                                  const double* __restrict__ t, double* __restrict__ prr,
                                                  CgState* __restrict__ st) {
    if (stopped(st, nullptr)) return;
    const double pAp = blockReduce(pspmv, nparts_spmv);
    const double alpha = st->rho / pAp;
    if (blockIdx.x == 0 && threadIdx.x == 0) st->alpha = alpha;
    double rr = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        x[i] += alpha * p[i];
        const double ro = r[i];
        rold[i] = ro;
        const double ri = ro - alpha * t[i];
        r[i] = ri;
        rr += ri * ri;
    }
    blockSum(rr, prr);
}

__global__ void __launch_bounds__(kB) k_mg_check(int np, const double* __restrict__ prr, CgState* __restrict__ st) {
    if (stopped(st, nullptr)) return;
    const double rr = blockReduce(prr, np);
    if (threadIdx.x == 0) {
        st->iters += 1;
        st->relres = sqrt(rr) / st->bnorm;
        if (st->relres < st->tol) st->done = 1;
        else if (st->iters >= st->maxit) st->done = 2;
    }
}

inline int blocksFor(long long n) {
    const long long g = (n + kB - 1) / kB;
    return int(g < 1 ? 1 : (g > kMaxBlocks ? kMaxBlocks : g));
}
inline int rowBlocks(int n, int lpr) {
    const int rpb = kB / lpr;
    const int g = (n + rpb - 1) / rpb;
    return g < 1 ? 1 : (g > kMaxBlocks ? kMaxBlocks : g);
}

// launch KERNEL<T, lanes, relative-columns> for the level's lanes per row
#define MG_ROW_DISPATCH(KERNEL, T, LV, NB, ...)                                                    \
    do {                                                                                           \
        const bool rel_ = (LV).coff != nullptr;                                                    \
        switch ((LV).lpr) {                                                                        \
            case 4:                                                                                \
                if (rel_) KERNEL<T, 4, true><<<NB, kB, 0, s>>>(__VA_ARGS__);                       \
                else KERNEL<T, 4, false><<<NB, kB, 0, s>>>(__VA_ARGS__);                           \
                break;                                                                             \
            case 8:                                                                                \
                if (rel_) KERNEL<T, 8, true><<<NB, kB, 0, s>>>(__VA_ARGS__);                       \
                else KERNEL<T, 8, false><<<NB, kB, 0, s>>>(__VA_ARGS__);                           \
                break;                                                                             \
            case 16:                                                                               \
                if (rel_) KERNEL<T, 16, true><<<NB, kB, 0, s>>>(__VA_ARGS__);                      \
                else KERNEL<T, 16, false><<<NB, kB, 0, s>>>(__VA_ARGS__);                          \
                break;                                                                             \
            default:                                                                               \
                if (rel_) KERNEL<T, 32, true><<<NB, kB, 0, s>>>(__VA_ARGS__);                      \
                else KERNEL<T, 32, false><<<NB, kB, 0, s>>>(__VA_ARGS__);                          \
                break;                                                                             \
        }                                                                                          \
    } while (0)

}  // namespace

namespace launch {

int mgPartials() { return kMaxBlocks; }

template <typename T>
void mgDinv(const MgLevelDev<T>& L, cudaStream_t s) {
    if (L.n > 0) k_dinv_mg<T><<<(L.n + kB - 1) / kB, kB, 0, s>>>(L.n, L.diag, L.val, L.dinv);
}

template <typename Ti, typename To>
void castVec(int n, const Ti* in, To* out, cudaStream_t s) {
    if (n > 0) k_cast<Ti, To><<<blocksFor(n), kB, 0, s>>>(n, in, out, nullptr);
}

template <typename T>
void coarseStart(const MgLevelDev<T>& L, double tol, const CgState* outer, cudaStream_t s) {
    const int nb = blocksFor(L.n);
    k_ccg_init<T><<<nb, kB, 0, s>>>(L.n, L.b, L.x, L.r, L.z, L.p, L.dinv, L.part0, L.part1, outer);
    k_ccg_init_reduce<<<1, kB, 0, s>>>(nb, L.part0, L.part1, L.st, tol, outer);
}

template <typename T>
void coarseIters(const MgLevelDev<T>& L, int k, const CgState* outer, cudaStream_t s) {
    const int nrb = rowBlocks(L.n, L.lpr);
    const int nb = blocksFor(L.n);
    for (int it = 0; it < k; ++it) {
        MG_ROW_DISPATCH(k_ccg_spmv, T, L, nrb, L.n, L.ptr, L.col, L.coff, L.val, L.p, L.t, L.part2, L.st, outer);
        k_ccg_update<T><<<nb, kB, 0, s>>>(L.n, nrb, L.part2, L.x, L.r, L.z, L.p, L.t, L.dinv, L.part0, L.part1, L.st,
                                          outer);
        k_ccg_beta<<<1, kB, 0, s>>>(nb, L.part0, L.part1, L.st, outer);
        k_ccg_pupd<T><<<nb, kB, 0, s>>>(L.n, L.p, L.z, L.st, outer);
    }
}

// gsMultiGridOp::multiGridStep (gsMultiGrid.hpp:147-201) with r = A x - b and x -= cgc P e; the
// coarse correction e starts at zero and runs prm.cycles cycles, one on the coarsest level, whose
// Jacobi-PCG solve overwrites its x as the reference's direct coarse solver does
template <typename T>
void vcycle(const std::vector<MgLevelDev<T>>& lv, int l, const MgParams& prm, const CgState* outer, cudaStream_t s,
            bool zero) {
    const MgLevelDev<T>& L = lv[l];
    const int nrb = rowBlocks(L.n, L.lpr);
    const int nb = blocksFor(L.n);
    if (l + 1 == (int)lv.size()) {
        coarseStart<T>(L, prm.coarse_tol, outer, s);
        coarseIters<T>(L, prm.coarse_iters, outer, s);
        return;
    }
    const T w = T(prm.damping);
    // sweeps alternate between x and z; an even total leaves the result in x
    T* cur = L.x;
    T* nxt = L.z;
    for (int k = 0; k < prm.npre; ++k) {
        MG_ROW_DISPATCH(k_jacobi, T, L, nrb, L.n, L.ptr, L.col, L.coff, L.val, L.dinv, w, L.b, cur, nxt,
                        k == 0 && zero ? 1 : 0, outer);
        T* tmp = cur; cur = nxt; nxt = tmp;
    }
    if (prm.npre == 0 && zero)  // x = 0
        k_jacobi<T, 4, false><<<nb, kB, 0, s>>>(L.n, L.ptr, L.col, L.coff, L.val, L.dinv, T(0), L.b, cur, cur, 1, outer);
    MG_ROW_DISPATCH(k_resid_mg, T, L, nrb, L.n, L.ptr, L.col, L.coff, L.val, cur, L.b, L.r, outer);
    const MgLevelDev<T>& C = lv[l + 1];
    k_transfer<T, 16><<<rowBlocks(C.n, 16), kB, 0, s>>>(C.n, C.Rptr, C.Rcol, C.Rval, L.r, C.b, 0, T(1), outer);
    const int nc = l + 2 == (int)lv.size() ? 1 : std::max(1, prm.cycles);
    for (int c = 0; c < nc; ++c) vcycle<T>(lv, l + 1, prm, outer, s, c == 0);
    k_transfer<T, 8><<<rowBlocks(L.n, 8), kB, 0, s>>>(L.n, C.Pptr, C.Pcol, C.Pval, C.x, cur, 1, T(prm.cgc), outer);
    for (int k = 0; k < prm.npost; ++k) {
        MG_ROW_DISPATCH(k_jacobi, T, L, nrb, L.n, L.ptr, L.col, L.coff, L.val, L.dinv, w, L.b, cur, nxt, 0, outer);
        T* tmp = cur; cur = nxt; nxt = tmp;
    }
    if (cur != L.x) k_cast<T, T><<<nb, kB, 0, s>>>(L.n, cur, L.x, outer);
}

void mgPcgStart(const MgOuter& O, double tol, int maxit, cudaStream_t s) {
    const int nb = blocksFor(O.n);
    k_mg_start<<<nb, kB, 0, s>>>(O.n, O.b, O.x, O.r, O.rold, O.p, O.part0);
    k_mg_start_reduce<<<1, kB, 0, s>>>(nb, O.part0, O.st, tol, maxit);
}

template <typename T>
void mgPcgPrecond(const MgOuter& O, const std::vector<MgLevelDev<T>>& lv, const MgParams& prm, cudaStream_t s) {
    const int nb = blocksFor(O.n);
    k_cast<double, T><<<nb, kB, 0, s>>>(O.n, O.r, lv[0].b, O.st);
    vcycle<T>(lv, 0, prm, O.st, s);
    k_mg_dots<T><<<nb, kB, 0, s>>>(O.n, O.r, O.rold, lv[0].x, O.part0, O.part1, O.st);
    k_mg_beta<<<1, kB, 0, s>>>(nb, O.part0, O.part1, O.st);
    k_mg_pupd<T><<<nb, kB, 0, s>>>(O.n, O.p, lv[0].x, O.phi, O.plo, O.st);
}

void mgPcgStep(const MgOuter& O, cudaStream_t s) {
    const int nb = blocksFor(O.n);
    const int nrb = rowBlocks(O.n, O.lpr);
    const bool split = O.val == nullptr;
    const bool rel = O.coff != nullptr;
#define MG_OUTER_ARGS O.n, O.ptr, O.col, O.coff, O.val, O.hi, O.lo, O.phi, O.plo, O.p, O.t, O.part2, O.st
#define MG_OUTER(LPR)                                                                        \
    do {                                                                                     \
        if (split && rel) k_mg_spmv<LPR, true, true><<<nrb, kB, 0, s>>>(MG_OUTER_ARGS);      \
        else if (split) k_mg_spmv<LPR, false, true><<<nrb, kB, 0, s>>>(MG_OUTER_ARGS);       \
        else if (rel) k_mg_spmv<LPR, true, false><<<nrb, kB, 0, s>>>(MG_OUTER_ARGS);         \
        else k_mg_spmv<LPR, false, false><<<nrb, kB, 0, s>>>(MG_OUTER_ARGS);                 \
    } while (0)
    switch (O.lpr) {
        case 4: MG_OUTER(4); break;
        case 8: MG_OUTER(8); break;
        case 16: MG_OUTER(16); break;
        default: MG_OUTER(32); break;
    }
#undef MG_OUTER
#undef MG_OUTER_ARGS
    k_mg_update<<<nb, kB, 0, s>>>(O.n, nrb, O.part2, O.x, O.r, O.rold, O.p, O.t, O.part0, O.st);
    k_mg_check<<<1, kB, 0, s>>>(nb, O.part0, O.st);
}

template void mgDinv<double>(const MgLevelDev<double>&, cudaStream_t);
template void mgDinv<float>(const MgLevelDev<float>&, cudaStream_t);
template void castVec<double, float>(int, const double*, float*, cudaStream_t);
template void castVec<float, double>(int, const float*, double*, cudaStream_t);
template void castVec<double, double>(int, const double*, double*, cudaStream_t);
template void coarseStart<double>(const MgLevelDev<double>&, double, const CgState*, cudaStream_t);
template void coarseStart<float>(const MgLevelDev<float>&, double, const CgState*, cudaStream_t);
template void coarseIters<double>(const MgLevelDev<double>&, int, const CgState*, cudaStream_t);
template void coarseIters<float>(const MgLevelDev<float>&, int, const CgState*, cudaStream_t);
template void vcycle<double>(const std::vector<MgLevelDev<double>>&, int, const MgParams&, const CgState*, cudaStream_t,
                             bool);
template void vcycle<float>(const std::vector<MgLevelDev<float>>&, int, const MgParams&, const CgState*, cudaStream_t,
                            bool);
template void mgPcgPrecond<double>(const MgOuter&, const std::vector<MgLevelDev<double>>&, const MgParams&, cudaStream_t);
template void mgPcgPrecond<float>(const MgOuter&, const std::vector<MgLevelDev<float>>&, const MgParams&, cudaStream_t);

}  // namespace launch
}  // namespace gsgpu
