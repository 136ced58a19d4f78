// sm_103a solver kernels: CSR SpMV (K5) fused with the p.Ap reduction, the fused CG vector
// update with Jacobi preconditioning (K6/K7), and the deterministic two-level reductions that
// keep alpha / beta / the stopping test on the device, so that an iteration needs no host
// round trip and a fixed run of iterations can be captured in a CUDA graph.
//
// Iteration (gsConjugateGradient::step, src/gsSolver/gsConjugateGradient.hpp:54-84):
//   t = A p; alpha = rho / (p.t); x += alpha p; r -= alpha t; stop if ||r||/||b|| < tol;
//   z = D^-1 r; beta = (r.z)/rho; p = z + beta p.
#include "kernels_solve.h"

namespace gsgpu {
namespace {

constexpr int kB = 256;

__device__ __forceinline__ double warpSum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// block sum of one value per thread into out[blockIdx.x] (fixed order -> deterministic)
__device__ __forceinline__ void blockSumStore(double v, double* out) {
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

// t = A p (LPR lanes per row) and partial sums of p.t
template <int LPR>
__global__ void __launch_bounds__(kB) k_spmv_dot(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                 const double* __restrict__ val, const double* __restrict__ p,
                                                 double* __restrict__ t, double* __restrict__ part,
                                                 const CgState* __restrict__ st) {
    if (st->done) return;
    const int rowsPerBlock = kB / LPR;
    const int lane = threadIdx.x % LPR;
    const int row = blockIdx.x * rowsPerBlock + threadIdx.x / LPR;
    double contrib = 0.0;
    double s = 0.0;
    if (row < n)
        for (int k = ptr[row] + lane; k < ptr[row + 1]; k += LPR) s += val[k] * p[col[k]];
    // every lane of the warp takes part in the shuffles (rows past n contribute 0)
    for (int o = LPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (row < n && lane == 0) {
        t[row] = s;
        contrib = s * p[row];
    }
    blockSumStore(contrib, part);
}

__global__ void __launch_bounds__(kB) k_alpha(int nparts, const double* __restrict__ part, CgState* __restrict__ st) {
    if (st->done) return;
    const double pAp = reducePartials(part, nparts);
    if (threadIdx.x == 0) st->alpha = st->rho / pAp;
}

// x += alpha p; r -= alpha t; z = dinv r; partial sums of r.r and r.z
__global__ void __launch_bounds__(kB) k_update(int n, double* __restrict__ x, double* __restrict__ r,
                                               double* __restrict__ z, const double* __restrict__ p,
                                               const double* __restrict__ t, const double* __restrict__ dinv,
                                               double* __restrict__ prr, double* __restrict__ prz,
                                               const CgState* __restrict__ st) {
    if (st->done) return;
    const double alpha = st->alpha;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double rr = 0.0, rz = 0.0;
    if (i < n) {
        x[i] += alpha * p[i];
        const double ri = r[i] - alpha * t[i];
        r[i] = ri;
        const double zi = dinv[i] * ri;
        z[i] = zi;
        rr = ri * ri;
        rz = ri * zi;
    }
    blockSumStore2(rr, rz, prr, prz);
}

__global__ void __launch_bounds__(kB) k_beta(int nparts, const double* __restrict__ prr, const double* __restrict__ prz,
                                             CgState* __restrict__ st) {
    if (st->done) return;
    const double rr = reducePartials(prr, nparts);
    const double rz = reducePartials(prz, nparts);
    if (threadIdx.x == 0) {
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
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = z[i] + beta * p[i];
}

// start: x = 0, r = b, z = D^-1 b, p = z; partial sums of b.b and r.z
__global__ void __launch_bounds__(kB) k_init(int n, const double* __restrict__ b, double* __restrict__ x,
                                             double* __restrict__ r, double* __restrict__ z, double* __restrict__ p,
                                             const double* __restrict__ dinv, double* __restrict__ pbb,
                                             double* __restrict__ prz) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double bb = 0.0, rz = 0.0;
    if (i < n) {
        const double bi = b[i];
        x[i] = 0.0;
        r[i] = bi;
        const double zi = dinv[i] * bi;
        z[i] = zi;
        p[i] = zi;
        bb = bi * bi;
        rz = bi * zi;
    }
    blockSumStore2(bb, rz, pbb, prz);
}

__global__ void __launch_bounds__(kB) k_init_reduce(int nparts, const double* __restrict__ pbb,
                                                    const double* __restrict__ prz, CgState* __restrict__ st,
                                                    double tol, int maxit) {
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
        // zero rhs: x = 0 is the solution; x0 = 0 gives ||r||/||b|| = 1 >= tol otherwise
        st->done = (bb == 0.0 || 1.0 < tol) ? 1 : (maxit <= 0 ? 2 : 0);
    }
}

__global__ void __launch_bounds__(kB) k_dinv(int n, const int* __restrict__ diag, const double* __restrict__ val,
                                             double damping, double* __restrict__ dinv) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dinv[i] = damping / val[diag[i]];
}

inline unsigned g1(long long n) { return unsigned((n + kB - 1) / kB); }

}  // namespace

namespace launch {

int cgPartials(int n) { return int(g1(n > 0 ? n : 1)); }

void jacobiDiag(int n, const int* diag, const double* val, double damping, double* dinv, cudaStream_t s) {
    if (n > 0) k_dinv<<<g1(n), kB, 0, s>>>(n, diag, val, damping, dinv);
}

void cgInit(const CgBuffers& B, double tol, int maxit, cudaStream_t s) {
    const int np = cgPartials(B.n);
    k_init<<<np, kB, 0, s>>>(B.n, B.b, B.x, B.r, B.z, B.p, B.dinv, B.part0, B.part1);
    k_init_reduce<<<1, kB, 0, s>>>(np, B.part0, B.part1, B.st, tol, maxit);
}

void cgSpmv(const CgBuffers& B, cudaStream_t s) {
    const int lpr = B.lanes_per_row;
    const int rows_per_block = kB / lpr;
    const int nb = (B.n + rows_per_block - 1) / rows_per_block;
    // B.part2 holds spmvPartials(n, 32) >= nb entries for every lanes-per-row choice below
    switch (lpr) {
        case 4: k_spmv_dot<4><<<nb, kB, 0, s>>>(B.n, B.ptr, B.col, B.val, B.p, B.t, B.part2, B.st); break;
        case 8: k_spmv_dot<8><<<nb, kB, 0, s>>>(B.n, B.ptr, B.col, B.val, B.p, B.t, B.part2, B.st); break;
        case 16: k_spmv_dot<16><<<nb, kB, 0, s>>>(B.n, B.ptr, B.col, B.val, B.p, B.t, B.part2, B.st); break;
        default: k_spmv_dot<32><<<nb, kB, 0, s>>>(B.n, B.ptr, B.col, B.val, B.p, B.t, B.part2, B.st); break;
    }
}

void cgRest(const CgBuffers& B, cudaStream_t s) {
    const int np = cgPartials(B.n);
    const int nb = spmvPartials(B.n, B.lanes_per_row);
    k_alpha<<<1, kB, 0, s>>>(nb, B.part2, B.st);
    k_update<<<np, kB, 0, s>>>(B.n, B.x, B.r, B.z, B.p, B.t, B.dinv, B.part0, B.part1, B.st);
    k_beta<<<1, kB, 0, s>>>(np, B.part0, B.part1, B.st);
    k_pupd<<<np, kB, 0, s>>>(B.n, B.p, B.z, B.st);
}

void cgIteration(const CgBuffers& B, cudaStream_t s) {
    cgSpmv(B, s);
    cgRest(B, s);
}

int spmvPartials(int n, int lanes_per_row) {
    const int rows_per_block = kB / lanes_per_row;
    return (n + rows_per_block - 1) / rows_per_block;
}

}  // namespace launch
}  // namespace gsgpu
