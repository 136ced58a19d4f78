// Neumann boundary integrals (gsVisitorNeumann, src/gsAssembler/gsVisitorNeumann.h:60-135, pushed
// by gsPoissonAssembler::assemble, gsPoissonAssembler.hpp:59, and gsCDRAssembler::assemble,
// gsCDRAssembler.hpp:58): for every Neumann side and every discretisation function i on it,
//   b_i += sum_q w_q |n(x_q)| h(x_q) N_i(xi_q),
// with the assembly's Gauss rule in the side directions and the boundary parameter in the fixed
// one (weight 1: gsQuadRule::mapTo halves the 2 of a one-node rule on a zero-length interval,
// gsQuadRule.h:192-200), |n| the norm of the outer normal of outerNormal (gsAssembler.h:79-130),
// i.e. of the cofactor column of the fixed direction, and h the closed-form Neumann data.
// Two kernels: one thread per face quadrature point writes w |n| h; one thread per patch-local dof
// on a Neumann side collects the sums of all its sides in side order (no atomics: the result does
// not depend on scheduling). Eliminated dofs receive their sums too; the rhs gather drops them, as
// gsSparseSystem::pushToRhs skips eliminated rows.
#include "kernels.h"

namespace gsgpu {
namespace {

using launch::kBlock;

__global__ void __launch_bounds__(kBlock) k_neu_face(const NeuSide* __restrict__ sides, const BlkEnt* __restrict__ tab,
                                                     const DevPatch* __restrict__ P,
                                                     const dev::FieldConst<double>* __restrict__ F,
                                                     const double* __restrict__ coefs, const double* __restrict__ gtab,
                                                     const int* __restrict__ ibuf, const double* __restrict__ wq,
                                                     double* __restrict__ vals) {
    const BlkEnt be = tab[blockIdx.x];
    const NeuSide& S = sides[be.patch];
    const long long item = be.base + threadIdx.x;
    if (item >= S.nq) return;
    const DevPatch& D = P[S.patch];
    const int d = D.dim;
    const int t0 = S.t[0], t1 = S.t[1];
    const int Q0 = D.Q[t0];
    const int g0 = int(item % Q0);
    const int g1 = d == 3 ? int(item / Q0) : 0;
    // geometry basis of the side directions at the abscissae (values, then derivatives)
    const int gp0 = D.gp[t0];
    const double* G0 = gtab + D.gtoff[t0] + (long long)g0 * 2 * (gp0 + 1);
    const int f0 = ibuf[D.gqoff[t0] + g0];
    int gp1 = 0, f1 = 0;
    const double* G1 = nullptr;
    if (d == 3) {
        gp1 = D.gp[t1];
        G1 = gtab + D.gtoff[t1] + (long long)g1 * 2 * (gp1 + 1);
        f1 = ibuf[D.gqoff[t1] + g1];
    }
    const long long gs[3] = {1, D.gn[0], (long long)D.gn[0] * D.gn[1]};
    const double* C = coefs + D.coef_off;
    double x[3] = {0, 0, 0}, T0[3] = {0, 0, 0}, T1[3] = {0, 0, 0};
    for (int c = 0; c <= S.gp; ++c) {
        const double nv = S.gval[c];
        if (nv == 0.0) continue;
        const long long bc = (long long)(S.gfirst + c) * gs[S.dir];
        for (int b = 0; b <= gp1; ++b) {
            const long long bb = d == 3 ? bc + (long long)(f1 + b) * gs[t1] : bc;
            const double v1 = d == 3 ? G1[b] : 1.0;
            const double d1 = d == 3 ? G1[gp1 + 1 + b] : 0.0;
            double sV[3] = {0, 0, 0}, sD[3] = {0, 0, 0};
            for (int a = 0; a <= gp0; ++a) {
                const long long idx = bb + (long long)(f0 + a) * gs[t0];
                for (int m = 0; m < d; ++m) {
                    const double cm = C[m * D.ngeo + idx];
                    sV[m] += G0[a] * cm;
                    sD[m] += G0[gp0 + 1 + a] * cm;
                }
            }
            for (int m = 0; m < d; ++m) {
                x[m] += nv * v1 * sV[m];
                T0[m] += nv * v1 * sD[m];
                T1[m] += nv * d1 * sV[m];
            }
        }
    }
    // |outer normal|: the tangent's length in 2D, |T0 x T1| in 3D
    double nrm;
    if (d == 3) {
        const double c0 = T0[1] * T1[2] - T0[2] * T1[1];
        const double c1 = T0[2] * T1[0] - T0[0] * T1[2];
        const double c2 = T0[0] * T1[1] - T0[1] * T1[0];
        nrm = sqrt(c0 * c0 + c1 * c1 + c2 * c2);
    } else {
        nrm = sqrt(T0[0] * T0[0] + T0[1] * T0[1]);
    }
    double w = wq[D.qoff[t0] + g0];
    if (d == 3) w *= wq[D.qoff[t1] + g1];
    // Neumann data h = sgn kappa du/dx_dir
    const dev::FieldConst<double>& Fp = F[D.field_id];
    double kappa, f;
    dev::fields<double>(Fp, x, kappa, f);
    double du = Fp.wpi;
    for (int i = 0; i < d; ++i) {
        double sn, cs;
        sincospi(double(Fp.ufreq) * x[i], &sn, &cs);
        du *= i == S.dir ? cs : sn;
    }
    const double h = (S.upper ? 1.0 : -1.0) * kappa * du;
    vals[S.qbase + item] = w * nrm * h;
}

__global__ void __launch_bounds__(kBlock) k_neu_dof(const NeuDof* __restrict__ dofs, long long ndofs,
                                                    const NeuSide* __restrict__ sides, const DevPatch* __restrict__ P,
                                                    const double* __restrict__ btab, const int* __restrict__ ibuf,
                                                    const double* __restrict__ vals, double* __restrict__ lvec) {
    const long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= ndofs) return;
    const NeuDof J = dofs[j];
    const DevPatch& D = P[J.patch];
    const int d = D.dim;
    double acc = 0.0;
    for (int k = 0; k < J.nside; ++k) {
        const NeuSide& S = sides[J.side[k]];
        const double nv = S.bval[J.i[S.dir] - S.bfirst];
        const int t0 = S.t[0], t1 = S.t[1];
        const int i0 = J.i[t0];
        const int p0 = D.p[t0], q0 = D.q[t0], Q0 = D.Q[t0];
        const int lo0 = ibuf[D.doff[t0] + i0], hi0 = ibuf[D.doff[t0] + D.n[t0] + i0];
        int i1 = 0, p1 = 0, q1 = 1, lo1 = 0, hi1 = 0;
        if (d == 3) {
            i1 = J.i[t1];
            p1 = D.p[t1];
            q1 = D.q[t1];
            lo1 = ibuf[D.doff[t1] + i1];
            hi1 = ibuf[D.doff[t1] + D.n[t1] + i1];
        }
        const double* V = vals + S.qbase;
        double sum = 0.0;
        for (int e1 = lo1; e1 <= hi1; ++e1) {
            const int s1 = d == 3 ? i1 - ibuf[D.eoff[t1] + e1] : 0;
            for (int r1 = 0; r1 < q1; ++r1) {
                const int g1 = e1 * q1 + r1;
                const double v1 = d == 3 ? btab[D.toff[t1] + (long long)g1 * 2 * (p1 + 1) + s1] : 1.0;
                double inner = 0.0;
                for (int e0 = lo0; e0 <= hi0; ++e0) {
                    const int s0 = i0 - ibuf[D.eoff[t0] + e0];
                    for (int r0 = 0; r0 < q0; ++r0) {
                        const int g0 = e0 * q0 + r0;
                        inner += V[g0 + (long long)Q0 * g1] * btab[D.toff[t0] + (long long)g0 * 2 * (p0 + 1) + s0];
                    }
                }
                sum += v1 * inner;
            }
        }
        acc += nv * sum;
    }
    lvec[J.lvec] += acc;
}

}  // namespace

namespace launch {

void neumannFace(const NeuSide* sides, const BlkEnt* tab, long long nblk, const DevPatch* P,
                 const dev::FieldConst<double>* F, const double* coefs, const double* gtab, const int* ibuf,
                 const double* wq, double* vals, cudaStream_t s) {
    if (nblk > 0) k_neu_face<<<unsigned(nblk), kBlock, 0, s>>>(sides, tab, P, F, coefs, gtab, ibuf, wq, vals);
}

void neumannDofs(const NeuDof* dofs, long long ndofs, const NeuSide* sides, const DevPatch* P, const double* btab,
                 const int* ibuf, const double* vals, double* lvec, cudaStream_t s) {
    if (ndofs > 0)
        k_neu_dof<<<unsigned((ndofs + kBlock - 1) / kBlock), kBlock, 0, s>>>(dofs, ndofs, sides, P, btab, ibuf, vals,
                                                                             lvec);
}

}  // namespace launch
}  // namespace gsgpu
