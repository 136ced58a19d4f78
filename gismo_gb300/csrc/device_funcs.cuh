// Per-work-item bodies of the assembly kernels. Each function computes one output element from
// the packed patch data; the __global__ wrappers in kernels_assemble.cu map threads to items.
#pragma once

#include <cmath>
#include <type_traits>

#include "df32.cuh"
#include "gsgpu_internal.h"

#ifdef __CUDACC__
#define GS_HD __host__ __device__ __forceinline__
#define GS_LDG(p) __ldg(p)
#else
#define GS_HD inline
#define GS_LDG(p) (*(p))
#endif

namespace gsgpu {
namespace dev {

constexpr int kMaxKappaWave = 8;  // largest |k_m,i| of a Fourier mode supported on the device

// -------------------------------------------------------------------------------------------
// K1: values and first derivatives of the p+1 B-splines of span s at u (Cox-de Boor triangle;
// derivatives from the degree p-1 values). out[0..p] values, out[p+1..2p+1] derivatives.
// The triangle's roundings are fixed (a product that feeds a later sum is rounded on its own, the
// other one fused: bMul / fma), so that the one-lane form here and the warp-cooperative kernel,
// which computes the same expressions in another order of statements, give the same bits.
GS_HD double bMul(double a, double b) {
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
GS_HD void basis1d(const double* __restrict__ t, int p, int s, double u, double* __restrict__ out) {
    double N[16], Nm1[16];
    N[0] = 1.0;
    if (p == 0) { out[0] = 1.0; out[1] = 0.0; return; }
    for (int k = 1; k <= p; ++k) {
        if (k == p)
            for (int r = 0; r < p; ++r) Nm1[r] = N[r];
        double saved = 0.0;
        for (int r = 0; r < k; ++r) {
            const double tr = t[s + 1 + r], tl = t[s + 1 + r - k];
            const double tmp = N[r] / (tr - tl);
            N[r] = fma(tr - u, tmp, saved);
            saved = bMul(u - tl, tmp);
        }
        N[k] = saved;
    }
    const int a = s - p;
    for (int r = 0; r <= p; ++r) {
        out[r] = N[r];
        double d = 0.0;
        if (r >= 1) d += bMul(double(p), Nm1[r - 1]) / (t[a + r + p] - t[a + r]);
        if (r <= p - 1) d -= bMul(double(p), Nm1[r]) / (t[a + r + p + 1] - t[a + r + 1]);
        out[p + 1 + r] = d;
    }
}

// pair factor PF[tau][e][r][s][t] = B^(alpha)_s(g) B^(beta)_t(g), tau = 2 alpha + beta,
// g = e*q + r; tab holds [V_0..V_p, D_0..D_p] per abscissa
template <typename T>
GS_HD T pairFactor(const double* __restrict__ tab, int p, int q, int E, long long item) {
    const int P1 = p + 1;
    const int t = int(item % P1);
    long long r0 = item / P1;
    const int s = int(r0 % P1);
    r0 /= P1;
    const int r = int(r0 % q);
    r0 /= q;
    const int e = int(r0 % E);
    const int tau = int(r0 / E);
    const double* row = tab + (long long)(e * q + r) * 2 * P1;
    const double a = (tau & 2) ? row[P1 + s] : row[s];
    const double b = (tau & 1) ? row[P1 + t] : row[t];
    return T(a * b);
}

// -------------------------------------------------------------------------------------------
// real-type traits: the geometry / field code below is written once for FP64 (plain path) and
// for df32 (mixed path: FP64-grade accuracy on the FP32 pipe)
template <typename R>
struct Real;
template <>
struct Real<double> {
    GS_HD static double zero() { return 0.0; }
    GS_HD static double abs(double v) { return fabs(v); }
    GS_HD static double toD(double v) { return v; }
    GS_HD static double exp(double v) {
#ifdef __CUDA_ARCH__
        return ::exp(v);
#else
        return std::exp(v);
#endif
    }
    GS_HD static void sincospi(double x, double* s, double* c) {
#ifdef __CUDA_ARCH__
        ::sincospi(x, s, c);
#else
        *s = std::sin(M_PI * x);
        *c = std::cos(M_PI * x);
#endif
    }
    GS_HD static double mulInt(double a, int k) { return a * k; }
};
template <>
struct Real<df32> {
    GS_HD static df32 zero() { return df32(); }
    GS_HD static df32 abs(df32 v) { return dfabs(v); }
    GS_HD static double toD(df32 v) { return v.toDouble(); }
    GS_HD static df32 exp(df32 v) { return expDf(v); }
    GS_HD static void sincospi(df32 x, df32* s, df32* c) { sincospiDf(x, *s, *c); }
    GS_HD static df32 mulInt(df32 a, int k) { return a * float(k); }
};

// sum of products: FP64 accumulates in place (acc += a * b); double-float accumulates compensated
// (Dot2: the exact FP32 products and the rounding errors of the running sum kept in one FP32
// correction), about half the FP32 operations of a chain of double-float multiplies and adds at
// an error of a few 2^-48 of the sum of |products|
template <typename R>
struct Acc {
    R s = Real<R>::zero();
    GS_HD void mac(R a, R b) { s += a * b; }
    GS_HD R result() const { return s; }
};
template <>
struct Acc<df32> {
    Dot2 d;
    GS_HD void mac(df32 a, df32 b) { d.mac(a, b); }
    GS_HD df32 result() const { return d.result(); }
};

// the closed-form field constants in the arithmetic of R (built on the host)
template <typename R>
struct FieldConst {
    int dim, fourier, nmodes, ufreq, kmax, pad;
    R kconst, alpha, scale, wpi, pi;  // wpi = ufreq * pi
    R amp[kMaxModes], cph[kMaxModes], sph[kMaxModes];
    R ace[kMaxModes], ase[kMaxModes];  // amp cos(phase), amp sin(phase), rounded once from FP64
    int kk[kMaxModes][3];
};
template <typename R>
inline FieldConst<R> fieldConst(const FieldParams& F) {
    FieldConst<R> c{};
    c.dim = F.dim;
    c.fourier = F.fourier;
    c.nmodes = F.nmodes;
    c.ufreq = F.ufreq;
    c.kmax = F.kmax;
    c.kconst = R(F.kconst);
    c.alpha = R(F.alpha);
    c.scale = R(F.scale);
    c.wpi = R(F.ufreq * M_PI);
    c.pi = R(M_PI);
    for (int m = 0; m < kMaxModes; ++m) {
        c.amp[m] = R(F.amp[m]);
        c.cph[m] = R(F.cph[m]);
        c.sph[m] = R(F.sph[m]);
        c.ace[m] = R(F.amp[m] * F.cph[m]);
        c.ase[m] = R(F.amp[m] * F.sph[m]);
        for (int k = 0; k < 3; ++k) c.kk[m][k] = F.kk[m][k];
    }
    return c;
}

// -------------------------------------------------------------------------------------------
// geometry map, sum-factorised over the control net: stage 1 (direction 0)
// 3D: Y1[m][tau][i2][i1][g0] ; 2D: Y1[m][tau][i1][g0]  (tau: 0 value, 1 derivative)
// I: the type of the item's index arithmetic (unsigned where the stage's work fits in 31 bits:
// its divisions are then a fraction of the 64-bit ones, which dominate these short dot products)
template <typename R, typename I = long long>
GS_HD R geoStage1(const DevPatch& D, long long itemL, const R* __restrict__ coefs, const R* __restrict__ gtab,
                  const int* __restrict__ ibuf) {
    const I item = I(itemL);
    const int Q0 = D.Q[0];
    const int g0 = int(item % I(Q0));
    I r = item / I(Q0);
    I rest;  // (i2*gn1 + i1) or i1
    if (D.dim == 3) {
        const I plane = I(D.gn[2]) * I(D.gn[1]);
        rest = r % plane;
        r /= plane;
    } else {
        rest = r % I(D.gn[1]);
        r /= I(D.gn[1]);
    }
    const int tau = int(r % 2);
    const int m = int(r / 2);
    const int gp = D.gp[0];
    const int f0 = ibuf[D.gqoff[0] + g0];
    const R* tb = gtab + D.gtoff[0] + (long long)g0 * 2 * (gp + 1) + tau * (gp + 1);
    const R* c = coefs + D.coef_off + m * D.ngeo + (long long)rest * D.gn[0] + f0;
    Acc<R> acc;
    for (int s = 0; s <= gp; ++s) acc.mac(tb[s], c[s]);
    return acc.result();
}

// 3D stage 2 (direction 1): Y2[m][tau][i2][g1][g0], tau: 0 vv, 1 dv (d/dxi0), 2 vd (d/dxi1)
template <typename R, typename I = long long>
GS_HD R geoStage2(const DevPatch& D, long long itemL, const R* __restrict__ Y1, const R* __restrict__ gtab,
                  const int* __restrict__ ibuf) {
    const I item = I(itemL);
    const int Q0 = D.Q[0], Q1 = D.Q[1];
    const int g0 = int(item % I(Q0));
    I r = item / I(Q0);
    const int g1 = int(r % I(Q1));
    r /= I(Q1);
    const int i2 = int(r % I(D.gn[2]));
    r /= I(D.gn[2]);
    const int tau = int(r % 3);
    const int m = int(r / 3);
    const int t1 = (tau == 1) ? 1 : 0;  // derivative in direction 0 (from stage 1)
    const int t2 = (tau == 2) ? 1 : 0;  // derivative in direction 1
    const int gp = D.gp[1];
    const int f1 = ibuf[D.gqoff[1] + g1];
    const R* tb = gtab + D.gtoff[1] + (long long)g1 * 2 * (gp + 1) + t2 * (gp + 1);
    const R* y = Y1 + D.y1_off + ((((long long)m * 2 + t1) * D.gn[2] + i2) * D.gn[1] + f1) * Q0 + g0;
    Acc<R> acc;
    for (int s = 0; s <= gp; ++s) acc.mac(tb[s], y[(long long)s * Q0]);
    return acc.result();
}

// closed-form fields at a physical point: kappa and f = -div(kappa grad u)
// (g = scale sum_m amp_m cos(pi k_m.x + phase_m), kappa = exp(alpha g), u = prod sin(freq pi x_i)).
// cos/sin of the mode phases use e^{i theta} = e^{i phase} prod_i (e^{i pi x_i})^{k_i}.
template <typename R>
struct Cplx {
    R re, im;
};
template <typename R>
GS_HD Cplx<R> cmul(const Cplx<R>& a, const Cplx<R>& b) {
    return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
// the same product with each component rounded once (double-float: dot2Terms), the form of the
// mode sums below
template <typename R>
GS_HD Cplx<R> cmulFused(const Cplx<R>& a, const Cplx<R>& b) {
    if constexpr (std::is_same<R, df32>::value)
        return {dot2Terms(a.re, b.re, a.im, b.im, -1.f), dot2Terms(a.re, b.im, a.im, b.re, 1.f)};
    else
        return cmul(a, b);
}

// sum over the Fourier modes of g = sum_m amp_m cos(pi k_m.x + phase_m) and of
// gg_i = -sum_m amp_m k_mi sin(pi k_m.x + phase_m), from the powers zp[i][k] = exp(i pi k x_i)
template <typename R, int NW>
GS_HD void modeSums(const FieldConst<R>& F, const Cplx<R> (*zp)[NW], int d, R& g, R* gg) {
    g = Real<R>::zero();
    for (int i = 0; i < 3; ++i) gg[i] = Real<R>::zero();
    for (int m = 0; m < F.nmodes; ++m) {
        Cplx<R> e{F.cph[m], F.sph[m]};
        for (int i = 0; i < d; ++i) e = cmul(e, zp[i][F.kk[m][i]]);
        g += F.amp[m] * e.re;
        const R as = F.amp[m] * e.im;
        for (int i = 0; i < d; ++i) gg[i] -= Real<R>::mulInt(as, F.kk[m][i]);
    }
}
// df32: the amplitude enters with the phase, each complex product rounds once per component
// (dot2Terms) and the mode sums accumulate compensated (Dot2), about half the FP32 operations of
// the generic form at an error of a few 2^-48 of sum_m amp_m
template <int NW>
GS_HD void modeSums(const FieldConst<df32>& F, const Cplx<df32> (*zp)[NW], int d, df32& g, df32* gg) {
    Dot2 ag, ag0, ag1, ag2;
    for (int m = 0; m < F.nmodes; ++m) {
        Cplx<df32> e{F.ace[m], F.ase[m]};
        for (int i = 0; i < d; ++i) {
            const Cplx<df32>& z = zp[i][F.kk[m][i]];
            e = Cplx<df32>{dot2Terms(e.re, z.re, e.im, z.im, -1.f), dot2Terms(e.re, z.im, e.im, z.re, 1.f)};
        }
        ag.add(e.re);
        ag0.mac(e.im, float(F.kk[m][0]));
        ag1.mac(e.im, float(F.kk[m][1]));
        if (d == 3) ag2.mac(e.im, float(F.kk[m][2]));
    }
    g = ag.result();
    gg[0] = -ag0.result();
    gg[1] = -ag1.result();
    gg[2] = -ag2.result();
}

// KW: the largest wave number the powers table holds (>= F.kmax); the table is a local array indexed
// by the modes' wave numbers at run time, so its size is what the point kernel's local memory holds
template <typename R, int KW = kMaxKappaWave>
GS_HD void fields(const FieldConst<R>& F, const R* x, R& kappa, R& f) {
    const int d = F.dim;
    R sn[3], cs[3];
    for (int i = 0; i < d; ++i) Real<R>::sincospi(Real<R>::mulInt(x[i], F.ufreq), &sn[i], &cs[i]);
    R u = sn[0];
    for (int i = 1; i < d; ++i) u = u * sn[i];
    R gu[3];
    for (int j = 0; j < d; ++j) {
        R t = F.wpi * cs[j];
        for (int i = 0; i < d; ++i)
            if (i != j) t = t * sn[i];
        gu[j] = t;
    }
    const R lap = Real<R>::mulInt(F.wpi * F.wpi * u, d);  // -Laplace(u) = d (freq pi)^2 u
    if (!F.fourier) {
        kappa = F.kconst;
        f = kappa * lap;
        return;
    }
    Cplx<R> zp[3][KW + 1];
    for (int i = 0; i < d; ++i) {
        R s, c;
        if (F.ufreq == 1) { s = sn[i]; c = cs[i]; }
        else Real<R>::sincospi(x[i], &s, &c);
        zp[i][0].re = Real<R>::zero();
        zp[i][0].re += R(1);
        zp[i][0].im = Real<R>::zero();
        const Cplx<R> z{c, s};
        for (int k = 1; k <= F.kmax; ++k) zp[i][k] = cmulFused(zp[i][k - 1], z);
    }
    R g, gg[3];
    modeSums(F, zp, d, g, gg);
    g = g * F.scale;
    R dot = Real<R>::zero();
    for (int i = 0; i < d; ++i) dot += gg[i] * gu[i];
    dot = dot * F.scale * F.pi;
    kappa = Real<R>::exp(F.alpha * g);
    f = kappa * (lap - F.alpha * dot);
}

// last geometry stage at quadrature point `item` of patch D: physical point x and Jacobian J
// (J[m][k] = d x_m / d xi_k) from the stage-1/2 partial contractions
// the Gauss-point indices of quadrature point `item` of patch D (32-bit divisions where the patch's
// point count allows: 64-bit ones cost several times more)
GS_HD void pointIndex(const DevPatch& D, long long item, int& g0, int& g1, int& g2) {
    const int Q0 = D.Q[0], Q1 = D.Q[1];
    if (D.nq < (1LL << 31)) {
        const unsigned it = unsigned(item), r = it / unsigned(Q0);
        g0 = int(it - r * unsigned(Q0));
        g1 = int(r % unsigned(Q1));
        g2 = int(r / unsigned(Q1));
    } else {
        const long long r = item / Q0;
        g0 = int(item - r * Q0);
        g1 = int(r % Q1);
        g2 = int(r / Q1);
    }
}
template <typename R>
GS_HD void pointMap(const DevPatch& D, long long item, const R* __restrict__ Y1, const R* __restrict__ Y2,
                    const R* __restrict__ gtab, const int* __restrict__ ibuf, R x[3], R J[3][3]) {
    const int d = D.dim;
    const int Q0 = D.Q[0], Q1 = D.Q[1];
    int g0, g1, g2;
    pointIndex(D, item, g0, g1, g2);
    if (d == 3) {
        const int gp = D.gp[2];
        const int f2 = ibuf[D.gqoff[2] + g2];
        const R* tb = gtab + D.gtoff[2] + (long long)g2 * 2 * (gp + 1);
        const long long plane = (long long)Q1 * Q0;
        for (int m = 0; m < 3; ++m) {
            const R* yvv = Y2 + D.y2_off + (((long long)m * 3 + 0) * D.gn[2] + f2) * plane + (long long)g1 * Q0 + g0;
            const R* ydv = yvv + (long long)D.gn[2] * plane;
            const R* yvd = ydv + (long long)D.gn[2] * plane;
            Acc<R> a, b, c, e;
            for (int s = 0; s <= gp; ++s) {
                const R v = tb[s], dv = tb[gp + 1 + s];
                const long long o = (long long)s * plane;
                a.mac(v, yvv[o]);
                b.mac(v, ydv[o]);
                c.mac(v, yvd[o]);
                e.mac(dv, yvv[o]);
            }
            x[m] = a.result();
            J[m][0] = b.result();
            J[m][1] = c.result();
            J[m][2] = e.result();
        }
    } else {
        const int gp = D.gp[1];
        const int f1 = ibuf[D.gqoff[1] + g1];
        const R* tb = gtab + D.gtoff[1] + (long long)g1 * 2 * (gp + 1);
        for (int m = 0; m < 2; ++m) {
            const R* yv = Y1 + D.y1_off + (((long long)m * 2 + 0) * D.gn[1] + f1) * Q0 + g0;
            const R* yd = yv + (long long)D.gn[1] * Q0;
            Acc<R> a, b, c;
            for (int s = 0; s <= gp; ++s) {
                const R v = tb[s], dv = tb[gp + 1 + s];
                const long long o = (long long)s * Q0;
                a.mac(v, yv[o]);
                b.mac(v, yd[o]);
                c.mac(dv, yv[o]);
            }
            x[m] = a.result();
            J[m][0] = b.result();
            J[m][1] = c.result();
        }
    }
}

// point-wise step: last geometry stage, metric and coefficient fields.
// C^{ab} = w kappa |det J| (J^-1 J^-T)_{ab} = w kappa / |det J| sum_m cof_{ma} cof_{mb},
// L = w |det J| f.  Component order 3D: 00 01 02 11 12 22 ; 2D: 00 01 11.
// Returns det J.
template <typename R, int KW = kMaxKappaWave>
GS_HD double pointStep(const DevPatch& D, const FieldConst<R>& F, long long item, const R* __restrict__ Y1,
                       const R* __restrict__ Y2, const R* __restrict__ gtab, const int* __restrict__ ibuf,
                       const R* __restrict__ wq, R* __restrict__ C, R* __restrict__ Lf) {
    const int d = D.dim;
    int g0, g1, g2;
    pointIndex(D, item, g0, g1, g2);
    R x[3], J[3][3];
    pointMap<R>(D, item, Y1, Y2, gtab, ibuf, x, J);
    R w = wq[D.qoff[0] + g0] * wq[D.qoff[1] + g1];
    if (d == 3) w = w * wq[D.qoff[2] + g2];
    R kappa, f;
    fields<R, KW>(F, x, kappa, f);
    const long long nq = D.nq;
    R det;
    if constexpr (std::is_same<R, df32>::value) {
        // double-float: every cofactor, the determinant and every metric component as one
        // compensated sum of exact products (same formulas as the FP64 branch below)
        if (d == 3) {
            df32 cof[3][3];
            auto cf = [&](int a, int b, int c, int e) { return dot2Terms(J[a][b], J[c][e], J[a][e], J[c][b], -1.f); };
            cof[0][0] = cf(1, 1, 2, 2);
            cof[0][1] = cf(1, 2, 2, 0);
            cof[0][2] = cf(1, 0, 2, 1);
            cof[1][0] = cf(0, 2, 2, 1);
            cof[1][1] = cf(0, 0, 2, 2);
            cof[1][2] = cf(0, 1, 2, 0);
            cof[2][0] = cf(0, 1, 1, 2);
            cof[2][1] = cf(0, 2, 1, 0);
            cof[2][2] = cf(0, 0, 1, 1);
            Dot2 dt;
            dt.mac(J[0][0], cof[0][0]);
            dt.mac(J[0][1], cof[0][1]);
            dt.mac(J[0][2], cof[0][2]);
            det = dt.result();
            const df32 sc = w * kappa / Real<R>::abs(det);
            df32* c = C + D.field_off + item;
            int k = 0;
            for (int a = 0; a < 3; ++a)
                for (int b = a; b < 3; ++b, ++k) {
                    Dot2 q;
                    q.mac(cof[0][a], cof[0][b]);
                    q.mac(cof[1][a], cof[1][b]);
                    q.mac(cof[2][a], cof[2][b]);
                    c[k * nq] = sc * q.result();
                }
        } else {
            det = dot2Terms(J[0][0], J[1][1], J[0][1], J[1][0], -1.f);
            const df32 c00 = J[1][1], c01 = -J[1][0], c10 = -J[0][1], c11 = J[0][0];
            const df32 sc = w * kappa / Real<R>::abs(det);
            df32* c = C + D.field_off + item;
            c[0] = sc * dot2Terms(c00, c00, c10, c10, 1.f);
            c[nq] = sc * dot2Terms(c00, c01, c10, c11, 1.f);
            c[2 * nq] = sc * dot2Terms(c01, c01, c11, c11, 1.f);
        }
        Lf[D.lfield_off + item] = w * Real<R>::abs(det) * f;
        return Real<R>::toD(det);
    }
    if (d == 3) {
        R cof[3][3];
        cof[0][0] = J[1][1] * J[2][2] - J[1][2] * J[2][1];
        cof[0][1] = J[1][2] * J[2][0] - J[1][0] * J[2][2];
        cof[0][2] = J[1][0] * J[2][1] - J[1][1] * J[2][0];
        cof[1][0] = J[0][2] * J[2][1] - J[0][1] * J[2][2];
        cof[1][1] = J[0][0] * J[2][2] - J[0][2] * J[2][0];
        cof[1][2] = J[0][1] * J[2][0] - J[0][0] * J[2][1];
        cof[2][0] = J[0][1] * J[1][2] - J[0][2] * J[1][1];
        cof[2][1] = J[0][2] * J[1][0] - J[0][0] * J[1][2];
        cof[2][2] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        det = J[0][0] * cof[0][0] + J[0][1] * cof[0][1] + J[0][2] * cof[0][2];
        const R sc = w * kappa / Real<R>::abs(det);
        R* c = C + D.field_off + item;
        int k = 0;
        for (int a = 0; a < 3; ++a)
            for (int b = a; b < 3; ++b, ++k)
                c[k * nq] = sc * (cof[0][a] * cof[0][b] + cof[1][a] * cof[1][b] + cof[2][a] * cof[2][b]);
    } else {
        det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
        // cof = [[J11, -J10], [-J01, J00]]
        const R c00 = J[1][1], c01 = -J[1][0], c10 = -J[0][1], c11 = J[0][0];
        const R sc = w * kappa / Real<R>::abs(det);
        R* c = C + D.field_off + item;
        c[0] = sc * (c00 * c00 + c10 * c10);
        c[nq] = sc * (c00 * c01 + c10 * c11);
        c[2 * nq] = sc * (c01 * c01 + c11 * c11);
    }
    Lf[D.lfield_off + item] = w * Real<R>::abs(det) * f;
    return Real<R>::toD(det);
}

// -------------------------------------------------------------------------------------------
// sum-factorised stiffness contraction along one axis.
//   out_h[o][i][oi][c] = sum_terms sum_{g in supp(i) & supp(j)} PF_tau(g; i, j) in_f[o][g][c],
//   j = i + oi - p. The term lists below group the d^2 products C^{ab} d_a(phi_i) d_b(phi_j) by
//   the derivative pattern of the remaining directions.
struct Term {
    int h, f, tau;
};

template <int KIND>
struct Stage;
// 3D stage 1 (axis 0): C(00,01,02,11,12,22) -> S0..S7
template <>
struct Stage<31> {
    static constexpr int AX = 0, NIN = 6, NOUT = 8, NT = 8;
    GS_HD static Term term(int k) {
        const Term t[8] = {{0, 0, 3}, {1, 1, 2}, {2, 1, 1}, {3, 2, 2}, {4, 2, 1}, {5, 3, 0}, {6, 4, 0}, {7, 5, 0}};
        return t[k];
    }
};
// 3D stage 2 (axis 1): S -> U_vv, U_vd, U_dv, U_dd (grouped by the direction-2 factor)
template <>
struct Stage<32> {
    static constexpr int AX = 1, NIN = 8, NOUT = 4, NT = 9;
    GS_HD static Term term(int k) {
        const Term t[9] = {{0, 0, 0}, {0, 1, 1}, {0, 2, 2}, {0, 5, 3}, {1, 3, 0},
                           {1, 6, 2}, {2, 4, 0}, {2, 6, 1}, {3, 7, 0}};
        return t[k];
    }
};
// 3D stage 3 (axis 2): U -> band
template <>
struct Stage<33> {
    static constexpr int AX = 2, NIN = 4, NOUT = 1, NT = 4;
    GS_HD static Term term(int k) {
        const Term t[4] = {{0, 0, 0}, {0, 1, 1}, {0, 2, 2}, {0, 3, 3}};
        return t[k];
    }
};
// 2D stage 1 (axis 0): C(00,01,11) -> S0..S3
template <>
struct Stage<21> {
    static constexpr int AX = 0, NIN = 3, NOUT = 4, NT = 4;
    GS_HD static Term term(int k) {
        const Term t[4] = {{0, 0, 3}, {1, 1, 2}, {2, 1, 1}, {3, 2, 0}};
        return t[k];
    }
};
// 2D stage 2 (axis 1): S -> band
template <>
struct Stage<22> {
    static constexpr int AX = 1, NIN = 4, NOUT = 1, NT = 4;
    GS_HD static Term term(int k) {
        const Term t[4] = {{0, 0, 0}, {0, 1, 1}, {0, 2, 2}, {0, 3, 3}};
        return t[k];
    }
};

// the mass matrix (gsGenericAssembler::assembleMass): one field M = w |det J| (stored in the load
// field's slot), one output, the value-value pair factors along every axis; the stages have the
// geometry of the stiffness stages 31 / 32 / 33 (3D) and 21 / 22 (2D)
template <>
struct Stage<41> {
    static constexpr int AX = 0, NIN = 1, NOUT = 1, NT = 1;
    GS_HD static Term term(int) { return {0, 0, 0}; }
};
template <>
struct Stage<42> {
    static constexpr int AX = 1, NIN = 1, NOUT = 1, NT = 1;
    GS_HD static Term term(int) { return {0, 0, 0}; }
};
template <>
struct Stage<43> {
    static constexpr int AX = 2, NIN = 1, NOUT = 1, NT = 1;
    GS_HD static Term term(int) { return {0, 0, 0}; }
};
template <>
struct Stage<51> {
    static constexpr int AX = 0, NIN = 1, NOUT = 1, NT = 1;
    GS_HD static Term term(int) { return {0, 0, 0}; }
};
template <>
struct Stage<52> {
    static constexpr int AX = 1, NIN = 1, NOUT = 1, NT = 1;
    GS_HD static Term term(int) { return {0, 0, 0}; }
};

// geometry of a stage for one patch: outer / inner extents, field strides and base offsets
struct StageGeom {
    long long outer, inner, in_fs, out_fs, in_base, out_base;
};
template <int KIND>
GS_HD StageGeom stageGeom(const DevPatch& D) {
    // the mass stages: the stiffness stages' geometry, input from the load field's slot
    if (KIND == 41 || KIND == 42 || KIND == 43 || KIND == 51 || KIND == 52) {
        StageGeom g = stageGeom<KIND == 41 ? 31 : KIND == 42 ? 32 : KIND == 43 ? 33 : KIND == 51 ? 21 : 22>(D);
        if (KIND == 41 || KIND == 51) g.in_base = D.lfield_off;
        return g;
    }
    StageGeom g{};
    const long long n0W = (long long)D.n[0] * D.W[0], n1W = (long long)D.n[1] * D.W[1];
    if (KIND == 31) {
        g.outer = (long long)D.Q[2] * D.Q[1]; g.inner = 1;
        g.in_fs = D.nq; g.in_base = D.field_off;
        g.out_fs = g.outer * n0W; g.out_base = D.s_off;
    } else if (KIND == 32) {
        g.outer = D.Q[2]; g.inner = n0W;
        g.in_fs = (long long)D.Q[2] * D.Q[1] * n0W; g.in_base = D.s_off;
        g.out_fs = (long long)D.Q[2] * n1W * n0W; g.out_base = D.u_off;
    } else if (KIND == 33) {
        g.outer = 1; g.inner = n1W * n0W;
        g.in_fs = (long long)D.Q[2] * n1W * n0W; g.in_base = D.u_off;
        g.out_fs = D.bandsize; g.out_base = D.band_off;
    } else if (KIND == 21) {
        g.outer = D.Q[1]; g.inner = 1;
        g.in_fs = D.nq; g.in_base = D.field_off;
        g.out_fs = (long long)D.Q[1] * n0W; g.out_base = D.s_off;
    } else {  // 22
        g.outer = 1; g.inner = n0W;
        g.in_fs = (long long)D.Q[1] * n0W; g.in_base = D.s_off;
        g.out_fs = D.bandsize; g.out_base = D.band_off;
    }
    return g;
}

template <int KIND>
GS_HD long long stageWork(const DevPatch& D) {
    const StageGeom g = stageGeom<KIND>(D);
    const int ax = Stage<KIND>::AX;
    return g.outer * D.n[ax] * D.W[ax] * g.inner;
}

template <typename T, int KIND>
GS_HD void contractItem(const DevPatch& D, long long item, const T* __restrict__ in, T* __restrict__ out,
                        const int* __restrict__ ibuf, const T* __restrict__ pf) {
    using S = Stage<KIND>;
    const int ax = S::AX;
    const StageGeom G = stageGeom<KIND>(D);
    const int n = D.n[ax], W = D.W[ax], q = D.q[ax], p = D.p[ax], Qa = D.Q[ax], E = D.E[ax];
    const long long c = item % G.inner;
    long long r = item / G.inner;
    const int oi = int(r % W);
    r /= W;
    const int i = int(r % n);
    const long long o = r / n;
    const int j = i + oi - p;
    T acc[S::NOUT];
    for (int h = 0; h < S::NOUT; ++h) acc[h] = T(0);
    if (j >= 0 && j < n) {
        const int* first = ibuf + D.eoff[ax];
        const int* elo = ibuf + D.doff[ax];
        const int* ehi = elo + n;
        const int e0 = elo[i] > elo[j] ? elo[i] : elo[j];
        const int e1 = ehi[i] < ehi[j] ? ehi[i] : ehi[j];
        const int P1 = p + 1;
        const long long tstride = (long long)E * q * P1 * P1;  // per pair type
        const T* pfa = pf + D.pfoff[ax];
        for (int e = e0; e <= e1; ++e) {
            const int fe = first[e];
            const int s = i - fe, t = j - fe;
            for (int rr = 0; rr < q; ++rr) {
                const int g = e * q + rr;
                const long long pidx = ((long long)(e * q + rr) * P1 + s) * P1 + t;
                T x[S::NIN];
                const T* ip = in + G.in_base + (o * Qa + g) * G.inner + c;
                for (int f = 0; f < S::NIN; ++f) x[f] = ip[f * G.in_fs];
                T pv[4];
                for (int tau = 0; tau < 4; ++tau) pv[tau] = GS_LDG(pfa + tau * tstride + pidx);
                for (int k = 0; k < S::NT; ++k) {
                    const Term tm = S::term(k);
                    acc[tm.h] += pv[tm.tau] * x[tm.f];
                }
            }
        }
    }
    T* op = out + G.out_base + ((o * n + i) * W + oi) * G.inner + c;
    for (int h = 0; h < S::NOUT; ++h) op[h * G.out_fs] = acc[h];
}

// the same contraction in df32 with compensated (Dot2) accumulation: each output keeps an FP32
// running sum plus an error term, so the band comes out with FP64-grade accuracy
template <int KIND>
GS_HD void contractItemDF(const DevPatch& D, long long item, const df32* __restrict__ in, df32* __restrict__ out,
                          const int* __restrict__ ibuf, const df32* __restrict__ pf) {
    using S = Stage<KIND>;
    const int ax = S::AX;
    const StageGeom G = stageGeom<KIND>(D);
    const int n = D.n[ax], W = D.W[ax], q = D.q[ax], p = D.p[ax], Qa = D.Q[ax], E = D.E[ax];
    const long long c = item % G.inner;
    long long r = item / G.inner;
    const int oi = int(r % W);
    r /= W;
    const int i = int(r % n);
    const long long o = r / n;
    const int j = i + oi - p;
    Dot2 acc[S::NOUT];
    if (j >= 0 && j < n) {
        const int* first = ibuf + D.eoff[ax];
        const int* elo = ibuf + D.doff[ax];
        const int* ehi = elo + n;
        const int e0 = elo[i] > elo[j] ? elo[i] : elo[j];
        const int e1 = ehi[i] < ehi[j] ? ehi[i] : ehi[j];
        const int P1 = p + 1;
        const long long tstride = (long long)E * q * P1 * P1;
        const df32* pfa = pf + D.pfoff[ax];
        for (int e = e0; e <= e1; ++e) {
            const int fe = first[e];
            const int s = i - fe, t = j - fe;
            for (int rr = 0; rr < q; ++rr) {
                const int g = e * q + rr;
                const long long pidx = ((long long)(e * q + rr) * P1 + s) * P1 + t;
                df32 x[S::NIN];
                const df32* ip = in + G.in_base + (o * Qa + g) * G.inner + c;
                for (int f = 0; f < S::NIN; ++f) x[f] = ip[f * G.in_fs];
                df32 pv[4];
                for (int tau = 0; tau < 4; ++tau) pv[tau] = pfa[tau * tstride + pidx];
                for (int k = 0; k < S::NT; ++k) {
                    const Term tm = S::term(k);
                    acc[tm.h].mac(pv[tm.tau], x[tm.f]);
                }
            }
        }
    }
    df32* op = out + G.out_base + ((o * n + i) * W + oi) * G.inner + c;
    for (int h = 0; h < S::NOUT; ++h) op[h * G.out_fs] = acc[h].result();
}

// Row-blocked df32 contraction: one work item owns (o, i, c) and produces all W band offsets of
// the output fields H0..H0+NH-1. For every quadrature abscissa g in the support of function i
// the inputs are loaded once and combined with the pair factors of the p+1 functions j active
// on g's element, so loads are amortised over (p+1) x terms multiply-adds.
template <int KIND>
GS_HD long long stageRowWork(const DevPatch& D) {
    const StageGeom g = stageGeom<KIND>(D);
    return g.outer * D.n[Stage<KIND>::AX] * g.inner;
}

// merge one element's partial sums (indexed by the local function t of j) into the band
// accumulators (indexed by the band offset shift + t); shift is uniform across a warp whenever
// the warp shares the row function i
template <int P, int NH>
GS_HD void mergeShift(Dot2 (&acc)[2 * P + 1][NH], const Dot2 (&tmp)[P + 1][NH], int shift) {
#pragma unroll
    for (int sh = 0; sh <= P; ++sh) {
        if (sh != shift) continue;
#pragma unroll
        for (int t = 0; t <= P; ++t)
#pragma unroll
            for (int h = 0; h < NH; ++h) acc[sh + t][h].add(tmp[t][h]);
    }
}

// QC > 0: the Gauss-point count per element is the compile-time QC (the default rule p+1), so
// the element's whole quadrature loop unrolls and its loads issue together; QC == 0: runtime q
template <int KIND, int P, int H0, int NH, int QC = 0>
GS_HD void contractRowDF(const DevPatch& D, long long item, const df32* __restrict__ in, df32* __restrict__ out,
                         const int* __restrict__ ibuf, const df32* __restrict__ pf) {
    using S = Stage<KIND>;
    constexpr int P1 = P + 1, W = 2 * P + 1;
    const int ax = S::AX;
    const StageGeom G = stageGeom<KIND>(D);
    const int n = D.n[ax], q = QC > 0 ? QC : D.q[ax], Qa = D.Q[ax], E = D.E[ax];
    const long long c = item % G.inner;
    long long r = item / G.inner;
    const int i = int(r % n);
    const long long o = r / n;
    Dot2 acc[W][NH];
    const int* first = ibuf + D.eoff[ax];
    const int* elo = ibuf + D.doff[ax];
    const int* ehi = elo + n;
    const long long tstride = (long long)E * q * P1 * P1;
    const df32* pfa = pf + D.pfoff[ax];
    for (int e = elo[i]; e <= ehi[i]; ++e) {
        const int fe = first[e];
        const int si = i - fe;
        Dot2 tmp[P1][NH];
#pragma unroll
        for (int rr = 0; rr < (QC > 0 ? QC : q); ++rr) {
            const int g = e * q + rr;
            df32 x[S::NIN];
            const df32* ip = in + G.in_base + (o * Qa + g) * G.inner + c;
#pragma unroll
            for (int f = 0; f < S::NIN; ++f) x[f] = ip[f * G.in_fs];
            const df32* prow = pfa + ((long long)(e * q + rr) * P1 + si) * P1;
#pragma unroll
            for (int t = 0; t < P1; ++t) {
                df32 pv[4];
#pragma unroll
                for (int tau = 0; tau < 4; ++tau) pv[tau] = prow[tau * tstride + t];
#pragma unroll
                for (int k = 0; k < S::NT; ++k) {
                    const Term tm = S::term(k);
                    if (tm.h >= H0 && tm.h < H0 + NH) tmp[t][tm.h - H0].mac(pv[tm.tau], x[tm.f]);
                }
            }
        }
        mergeShift<P, NH>(acc, tmp, P - si);  // band offset of j = fe + t is t + P - si
    }
    df32* op = out + G.out_base + (o * n + i) * W * G.inner + c;
#pragma unroll
    for (int w = 0; w < W; ++w)
#pragma unroll
        for (int h = 0; h < NH; ++h) op[(H0 + h) * G.out_fs + w * G.inner] = acc[w][h].result();
}

// rows of the stage axis with the fixed support shape (D.simple): p <= i <= n-1-p; the others are
// the boundary rows (all rows when the axis is not simple)
// (single-output stages keep the general kernel for every row: their accumulators are few, and
// the unrolled form only raises register pressure there)
template <int KIND>
GS_HD int interiorRows(const DevPatch& D) {
    const int ax = Stage<KIND>::AX;
    const int m = D.n[ax] - 2 * D.p[ax];
    return Stage<KIND>::NOUT > 1 && D.simple[ax] && m > 0 ? m : 0;
}
template <int KIND>
GS_HD long long stageInteriorWork(const DevPatch& D) {
    const StageGeom g = stageGeom<KIND>(D);
    return g.outer * interiorRows<KIND>(D) * g.inner;
}
template <int KIND>
GS_HD long long stageBoundaryWork(const DevPatch& D) {
    const StageGeom g = stageGeom<KIND>(D);
    return g.outer * (D.n[Stage<KIND>::AX] - interiorRows<KIND>(D)) * g.inner;
}
// boundary item -> row-blocked item (rows 0..p-1 and n-p..n-1, or all rows)
template <int KIND>
GS_HD long long boundaryItem(const DevPatch& D, long long item) {
    const StageGeom g = stageGeom<KIND>(D);
    const int ax = Stage<KIND>::AX;
    const int m = interiorRows<KIND>(D), nb = D.n[ax] - m;
    const long long c = item % g.inner;
    const long long r = item / g.inner;
    const int ib = int(r % nb);
    const long long o = r / nb;
    const int i = (m > 0 && ib >= D.p[ax]) ? ib + m : ib;
    return (o * D.n[ax] + i) * g.inner + c;
}

// interior rows: function i = p + (row index) has support elements i-p..i with first[e] = e, so
// element k of the support contributes its local function t to band offset k + t; the element
// and quadrature loops unroll and accumulate straight into the band accumulators
template <int KIND, int P, int H0, int NH>
GS_HD void contractRowDFInterior(const DevPatch& D, long long item, const df32* __restrict__ in,
                                 df32* __restrict__ out, const df32* __restrict__ pf) {
    using S = Stage<KIND>;
    constexpr int P1 = P + 1, W = 2 * P + 1, Q = P + 1;
    const int ax = S::AX;
    const StageGeom G = stageGeom<KIND>(D);
    const int n = D.n[ax], Qa = D.Q[ax], E = D.E[ax];
    const int m = n - 2 * P;
    const long long c = item % G.inner;
    long long r = item / G.inner;
    const int i = P + int(r % m);
    const long long o = r / m;
    Dot2 acc[W][NH];
    const long long tstride = (long long)E * Q * P1 * P1;
    const df32* pfa = pf + D.pfoff[ax];
#pragma unroll
    for (int k = 0; k <= P; ++k) {
        const int e = i - P + k;  // local function of i on element e: si = P - k
#pragma unroll
        for (int rr = 0; rr < Q; ++rr) {
            const int g = e * Q + rr;
            df32 x[S::NIN];
            const df32* ip = in + G.in_base + (o * Qa + g) * G.inner + c;
#pragma unroll
            for (int f = 0; f < S::NIN; ++f) x[f] = ip[f * G.in_fs];
            const df32* prow = pfa + ((long long)g * P1 + (P - k)) * P1;
#pragma unroll
            for (int t = 0; t < P1; ++t) {
                df32 pv[4];
#pragma unroll
                for (int tau = 0; tau < 4; ++tau) pv[tau] = prow[tau * tstride + t];
#pragma unroll
                for (int kk = 0; kk < S::NT; ++kk) {
                    const Term tm = S::term(kk);
                    if (tm.h >= H0 && tm.h < H0 + NH) acc[k + t][tm.h - H0].mac(pv[tm.tau], x[tm.f]);
                }
            }
        }
    }
    df32* op = out + G.out_base + (o * n + i) * W * G.inner + c;
#pragma unroll
    for (int w = 0; w < W; ++w)
#pragma unroll
        for (int h = 0; h < NH; ++h) op[(H0 + h) * G.out_fs + w * G.inner] = acc[w][h].result();
}

// 3D stage 1 for the interior rows of a simple axis 0, in tiles of kTileLines lines (o) by
// kTileRows consecutive rows (i) per block, one launch per output half (h 0-3, h 4-7); degrees 2
// and 3, other degrees keep contractRowDFInterior
constexpr int kTileLines = 8, kTileRows = 32;
GS_HD bool tiledStage31(int P) { return P == 2 || P == 3; }
GS_HD long long stage31Tiles(const DevPatch& D) {
    const int m = interiorRows<31>(D);
    if (D.dim != 3 || m == 0 || !tiledStage31(D.p[0])) return 0;
    const StageGeom g = stageGeom<31>(D);
    return (g.outer + kTileLines - 1) / kTileLines * ((m + kTileRows - 1) / kTileRows);
}
// the stage-1 terms of outputs H0..H0+3 read a contiguous range of input fields and of pair
// factor types (Stage<31>::term): h 0-3 fields 0-2, types 1-3; h 4-7 fields 2-5, types 0-1
GS_HD constexpr int tileField0(int H0) { return H0 == 0 ? 0 : 2; }
GS_HD constexpr int tileNField(int H0) { return H0 == 0 ? 3 : 4; }
GS_HD constexpr int tileTau0(int H0) { return H0 == 0 ? 1 : 0; }
GS_HD constexpr int tileNTau(int H0) { return H0 == 0 ? 3 : 2; }
// shared memory of a tile: pair factors [si][rr][t][tau][ee] and fields [f][rr][line][ee],
// ee = element - first element of the tile
GS_HD constexpr int tileElems(int P) { return kTileRows + P; }
GS_HD constexpr int tilePfCount(int P, int H0) { return (P + 1) * (P + 1) * (P + 1) * tileNTau(H0) * tileElems(P); }
GS_HD constexpr int tileFieldCount(int P, int H0) { return tileNField(H0) * (P + 1) * kTileLines * tileElems(P); }

// degree dispatch of the row-blocked contraction (uniform per patch)
template <int KIND, int H0, int NH>
GS_HD void contractRowDFp(const DevPatch& D, long long item, const df32* __restrict__ in, df32* __restrict__ out,
                          const int* __restrict__ ibuf, const df32* __restrict__ pf) {
    switch (D.p[Stage<KIND>::AX]) {
        case 1: contractRowDF<KIND, 1, H0, NH>(D, item, in, out, ibuf, pf); break;
        case 2: contractRowDF<KIND, 2, H0, NH>(D, item, in, out, ibuf, pf); break;
        case 3: contractRowDF<KIND, 3, H0, NH>(D, item, in, out, ibuf, pf); break;
        default: contractRowDF<KIND, 4, H0, NH>(D, item, in, out, ibuf, pf); break;
    }
}

GS_HD double asDouble(double v) { return v; }
GS_HD double asDouble(df32 v) { return v.toDouble(); }

// -------------------------------------------------------------------------------------------
// load vector: single-index contraction of L with the basis values along one axis
//   3D: 31: L[g2][g1][g0] -> lv1[g2][g1][i0]; 32: lv1 -> lv2[g2][i1][i0]; 33: lv2 -> F[i2][i1][i0]
//   2D: 21: L[g1][g0] -> lv1[g1][i0]; 22: lv1 -> F[i1][i0]
struct LoadGeom {
    long long outer, inner, in_base, out_base;
};
template <int KIND>
GS_HD LoadGeom loadGeom(const DevPatch& D) {
    LoadGeom g{};
    if (KIND == 31) { g.outer = (long long)D.Q[2] * D.Q[1]; g.inner = 1; g.in_base = D.lfield_off; g.out_base = D.lv1_off; }
    else if (KIND == 32) { g.outer = D.Q[2]; g.inner = D.n[0]; g.in_base = D.lv1_off; g.out_base = D.lv2_off; }
    else if (KIND == 33) { g.outer = 1; g.inner = (long long)D.n[1] * D.n[0]; g.in_base = D.lv2_off; g.out_base = D.lvec_off; }
    else if (KIND == 21) { g.outer = D.Q[1]; g.inner = 1; g.in_base = D.lfield_off; g.out_base = D.lv1_off; }
    else { g.outer = 1; g.inner = D.n[0]; g.in_base = D.lv1_off; g.out_base = D.lvec_off; }
    return g;
}
template <int KIND>
GS_HD long long loadWork(const DevPatch& D) {
    const LoadGeom g = loadGeom<KIND>(D);
    const int ax = Stage<KIND>::AX;
    return g.outer * D.n[ax] * g.inner;
}
// the input of stage 31/21 is the L field, of later stages the previous intermediate; the
// caller passes the right base pointers (L field buffer or intermediate buffer)
template <int KIND, typename Tin>
GS_HD double loadItem(const DevPatch& D, long long item, const Tin* __restrict__ in, const double* __restrict__ tab,
                      const int* __restrict__ ibuf) {
    const int ax = Stage<KIND>::AX;
    const LoadGeom G = loadGeom<KIND>(D);
    const int n = D.n[ax], q = D.q[ax], p = D.p[ax], Qa = D.Q[ax];
    const long long c = item % G.inner;
    long long r = item / G.inner;
    const int i = int(r % n);
    const long long o = r / n;
    const int* first = ibuf + D.eoff[ax];
    const int* elo = ibuf + D.doff[ax];
    const int* ehi = elo + n;
    const double* tb = tab + D.toff[ax];
    double acc = 0.0;
    for (int e = elo[i]; e <= ehi[i]; ++e) {
        const int s = i - first[e];
        for (int rr = 0; rr < q; ++rr) {
            const int g = e * q + rr;
            acc += tb[(long long)g * 2 * (p + 1) + s] * asDouble(in[G.in_base + (o * Qa + g) * G.inner + c]);
        }
    }
    return acc;
}

// the same contraction for a double-float load field and basis table: the products summed by a
// compensated dot product on the FP32 pipe, the sum rounded to FP64 once per output (no FP64
// arithmetic and no conversion per term)
template <int KIND>
GS_HD double loadItemDF(const DevPatch& D, long long item, const df32* __restrict__ in, const df32* __restrict__ tab,
                        const int* __restrict__ ibuf) {
    const int ax = Stage<KIND>::AX;
    const LoadGeom G = loadGeom<KIND>(D);
    const int n = D.n[ax], q = D.q[ax], p = D.p[ax], Qa = D.Q[ax];
    const long long c = item % G.inner;
    long long r = item / G.inner;
    const int i = int(r % n);
    const long long o = r / n;
    const int* first = ibuf + D.eoff[ax];
    const int* elo = ibuf + D.doff[ax];
    const int* ehi = elo + n;
    const df32* tb = tab + D.toff[ax];
    Dot2 acc;
    for (int e = elo[i]; e <= ehi[i]; ++e) {
        const int s = i - first[e];
        for (int rr = 0; rr < q; ++rr) {
            const int g = e * q + rr;
            acc.mac(tb[(long long)g * 2 * (p + 1) + s], in[G.in_base + (o * Qa + g) * G.inner + c]);
        }
    }
    const df32 v = acc.result();
    return double(v.hi) + double(v.lo);
}

// -------------------------------------------------------------------------------------------
// CSR values: segmented reduction of band entries over the precomputed slot map
template <typename T>
GS_HD T gatherSlot(uint32_t src, const T* __restrict__ band, const uint32_t* __restrict__ ovf_ptr,
                   const uint32_t* __restrict__ ovf_idx) {
    if (!(src & 0x80000000u)) return band[src];
    const uint32_t o = src & 0x7fffffffu;
    T acc = T(0);
    for (uint32_t k = ovf_ptr[o]; k < ovf_ptr[o + 1]; ++k) acc += band[ovf_idx[k]];
    return acc;
}

GS_HD df32 gatherSlotDF(uint32_t src, const df32* __restrict__ band, const uint32_t* __restrict__ ovf_ptr,
                        const uint32_t* __restrict__ ovf_idx) {
    if (!(src & 0x80000000u)) return band[src];
    const uint32_t o = src & 0x7fffffffu;
    df32 acc;
    for (uint32_t k = ovf_ptr[o]; k < ovf_ptr[o + 1]; ++k) acc += band[ovf_idx[k]];
    return acc;
}

// rhs row: load-vector sources minus the Dirichlet lift sum_j K_ij g_j over eliminated j
// (gsSparseSystem::push, src/gsAssembler/gsSparseSystem.h:972-1010)
template <typename TB>
GS_HD double rhsRow(int I, const double* __restrict__ lvec, const uint32_t* __restrict__ lptr,
                    const uint32_t* __restrict__ lidx, const TB* __restrict__ band,
                    const uint32_t* __restrict__ fptr, const uint32_t* __restrict__ fband,
                    const uint32_t* __restrict__ fbidx, const double* __restrict__ ddof) {
    double acc = 0.0;
    for (uint32_t k = lptr[I]; k < lptr[I + 1]; ++k) acc += lvec[lidx[k]];
    for (uint32_t k = fptr[I]; k < fptr[I + 1]; ++k) acc -= asDouble(band[fband[k]]) * ddof[fbidx[k]];
    return acc;
}

}  // namespace dev
}  // namespace gsgpu
