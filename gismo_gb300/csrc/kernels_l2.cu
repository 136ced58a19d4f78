// Discrete L2 error of the last solution (gsField::distanceL2, src/gsCore/gsField.hpp:23-41, on
// the solution patches of gsAssembler::constructSolution, src/gsAssembler/gsAssembler.hpp:536-581):
// Gauss quadrature of (u_h - u)^2 |det J| over every element of every patch, with the assembly's
// (p+1)^d rule. u_h sums the solution coefficients of the active basis functions (free dofs from
// x, eliminated dofs from the Dirichlet values); u is the closed-form manufactured solution.
// The H1 form (gsField::distanceH1, gsField.hpp:44-60, parametric solution field against the
// physical exact function) integrates |J^-T grad_xi u_h - grad u|^2 |det J| with the same rule.
#include "kernels.h"

namespace gsgpu {
namespace {

using launch::kBlock;

// per patch-local dof: x[index] (free) or ddof[index - nfree] (eliminated)
__global__ void __launch_bounds__(kBlock) k_solcoef(long long nlocal, const int* __restrict__ index, int nfree,
                                                    const double* __restrict__ x, const double* __restrict__ ddof,
                                                    double* __restrict__ coef) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nlocal) return;
    const int g = index[i];
    coef[i] = g < nfree ? x[g] : ddof[g - nfree];
}

template <bool H1>
__global__ void __launch_bounds__(kBlock) k_l2(const DevPatch* __restrict__ P, const BlkEnt* __restrict__ tab,
                                               const dev::FieldConst<double>* __restrict__ F,
                                               const double* __restrict__ Y1, const double* __restrict__ Y2,
                                               const double* __restrict__ gtab, const int* __restrict__ ibuf,
                                               const double* __restrict__ wq, const double* __restrict__ btab,
                                               const double* __restrict__ coef, double* __restrict__ part) {
    const BlkEnt be = tab[blockIdx.x];
    const DevPatch& D = P[be.patch];
    const long long item = be.base + threadIdx.x;
    double v = 0.0;
    if (item < D.nq) {
        const int d = D.dim;
        double x[3], J[3][3];
        dev::pointMap<double>(D, item, Y1, Y2, gtab, ibuf, x, J);
        int g[3];
        g[0] = int(item % D.Q[0]);
        g[1] = int((item / D.Q[0]) % D.Q[1]);
        g[2] = d == 3 ? int(item / ((long long)D.Q[0] * D.Q[1])) : 0;
        double det;
        if (d == 3)
            det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                  J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
        else
            det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        double w = wq[D.qoff[0] + g[0]] * wq[D.qoff[1] + g[1]];
        if (d == 3) w *= wq[D.qoff[2] + g[2]];
        // u_h: tensor sum over the (p+1)^d active functions of the element
        const double* b[3];
        int f[3] = {0, 0, 0}, pk[3] = {0, 0, 0};
        for (int k = 0; k < d; ++k) {
            pk[k] = D.p[k];
            f[k] = ibuf[D.eoff[k] + g[k] / D.q[k]];
            b[k] = btab + D.toff[k] + (long long)g[k] * 2 * (pk[k] + 1);
        }
        const double* c = coef + D.lvec_off;
        if (!H1) {
            double uh = 0.0;
            if (d == 3) {
                for (int s2 = 0; s2 <= pk[2]; ++s2) {
                    double a1 = 0.0;
                    for (int s1 = 0; s1 <= pk[1]; ++s1) {
                        const double* cr = c + ((long long)(f[2] + s2) * D.n[1] + f[1] + s1) * D.n[0] + f[0];
                        double a0 = 0.0;
                        for (int s0 = 0; s0 <= pk[0]; ++s0) a0 += b[0][s0] * cr[s0];
                        a1 += b[1][s1] * a0;
                    }
                    uh += b[2][s2] * a1;
                }
            } else {
                for (int s1 = 0; s1 <= pk[1]; ++s1) {
                    const double* cr = c + (long long)(f[1] + s1) * D.n[0] + f[0];
                    double a0 = 0.0;
                    for (int s0 = 0; s0 <= pk[0]; ++s0) a0 += b[0][s0] * cr[s0];
                    uh += b[1][s1] * a0;
                }
            }
            double u = 1.0;
            for (int k = 0; k < d; ++k) {
                double sn, cs;
                sincospi(double(F[D.field_id].ufreq) * x[k], &sn, &cs);
                u *= sn;
            }
            const double e = uh - u;
            v = e * e * w * fabs(det);
        } else {
            // parametric gradient of u_h: derivative factor in one direction, values in the others
            // (b[k][p+1+s] holds the derivative of function s)
            double gx[3] = {0, 0, 0};
            if (d == 3) {
                for (int s2 = 0; s2 <= pk[2]; ++s2) {
                    double a1[3] = {0, 0, 0};
                    for (int s1 = 0; s1 <= pk[1]; ++s1) {
                        const double* cr = c + ((long long)(f[2] + s2) * D.n[1] + f[1] + s1) * D.n[0] + f[0];
                        double v0 = 0.0, d0 = 0.0;
                        for (int s0 = 0; s0 <= pk[0]; ++s0) {
                            v0 += b[0][s0] * cr[s0];
                            d0 += b[0][pk[0] + 1 + s0] * cr[s0];
                        }
                        a1[0] += b[1][s1] * d0;
                        a1[1] += b[1][pk[1] + 1 + s1] * v0;
                        a1[2] += b[1][s1] * v0;
                    }
                    gx[0] += b[2][s2] * a1[0];
                    gx[1] += b[2][s2] * a1[1];
                    gx[2] += b[2][pk[2] + 1 + s2] * a1[2];
                }
            } else {
                for (int s1 = 0; s1 <= pk[1]; ++s1) {
                    const double* cr = c + (long long)(f[1] + s1) * D.n[0] + f[0];
                    double v0 = 0.0, d0 = 0.0;
                    for (int s0 = 0; s0 <= pk[0]; ++s0) {
                        v0 += b[0][s0] * cr[s0];
                        d0 += b[0][pk[0] + 1 + s0] * cr[s0];
                    }
                    gx[0] += b[1][s1] * d0;
                    gx[1] += b[1][pk[1] + 1 + s1] * v0;
                }
            }
            // physical gradient J^-T grad_xi = cof(J) grad_xi / det J
            double cof[3][3];
            if (d == 3) {
                for (int m = 0; m < 3; ++m)
                    for (int k = 0; k < 3; ++k) {
                        const int m1 = (m + 1) % 3, m2 = (m + 2) % 3, k1 = (k + 1) % 3, k2 = (k + 2) % 3;
                        cof[m][k] = J[m1][k1] * J[m2][k2] - J[m1][k2] * J[m2][k1];
                    }
            } else {
                cof[0][0] = J[1][1];
                cof[0][1] = -J[1][0];
                cof[1][0] = -J[0][1];
                cof[1][1] = J[0][0];
            }
            // exact gradient: freq pi cos(freq pi x_j) prod_{i != j} sin(freq pi x_i)
            const int fq = F[D.field_id].ufreq;
            double sn[3], cs[3];
            for (int k = 0; k < d; ++k) sincospi(double(fq) * x[k], &sn[k], &cs[k]);
            double e2 = 0.0;
            for (int m = 0; m < d; ++m) {
                double gh = 0.0;
                for (int k = 0; k < d; ++k) gh += cof[m][k] * gx[k];
                gh /= det;
                double gu = F[D.field_id].wpi * cs[m];
                for (int i = 0; i < d; ++i)
                    if (i != m) gu *= sn[i];
                const double e = gh - gu;
                e2 += e * e;
            }
            v = e2 * w * fabs(det);
        }
    }
    // block sum in a fixed order
    __shared__ double ws[kBlock / 32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < kBlock / 32; ++k) s += ws[k];
        part[blockIdx.x] = s;
    }
}

}  // namespace

namespace launch {

void solutionCoefs(long long nlocal, const int* index, int nfree, const double* x, const double* ddof, double* coef,
                   cudaStream_t s) {
    if (nlocal > 0) k_solcoef<<<unsigned((nlocal + kBlock - 1) / kBlock), kBlock, 0, s>>>(nlocal, index, nfree, x, ddof, coef);
}

void l2Partials(const DevPatch* P, const BlkEnt* tab, long long nblk, const dev::FieldConst<double>* F,
                const double* Y1, const double* Y2, const double* gtab, const int* ibuf, const double* wq,
                const double* btab, const double* coef, double* part, bool h1, cudaStream_t s) {
    if (nblk <= 0) return;
    if (h1) k_l2<true><<<unsigned(nblk), kBlock, 0, s>>>(P, tab, F, Y1, Y2, gtab, ibuf, wq, btab, coef, part);
    else k_l2<false><<<unsigned(nblk), kBlock, 0, s>>>(P, tab, F, Y1, Y2, gtab, ibuf, wq, btab, coef, part);
}

}  // namespace launch
}  // namespace gsgpu
