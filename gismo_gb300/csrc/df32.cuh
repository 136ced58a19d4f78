// Double-float ("df32") arithmetic: a value is the unevaluated sum hi + lo of two FP32 numbers
// with |lo| <= ulp(hi)/2, i.e. a 48-bit significand carried on the FP32 pipe. On GB300 the FP32
// FMA rate is 59x the FP64 rate, so FP64-grade accuracy is cheaper this way than in FP64.
//
// Building blocks are the classical error-free transformations: Knuth's TwoSum, Dekker's
// Fast2Sum and the FMA-based TwoProduct; products and sums of df32 follow Dekker (1971) and the
// double-double algorithms of Hida, Li and Bailey (2001); dot products accumulate with the
// compensated scheme Dot2 of Ogita, Rump and Oishi (2005). sin/cos(pi x) and exp use argument
// reduction plus Taylor series evaluated in df32 (the method of the double-double library cited
// above), written here from those definitions.
#pragma once

#include <cmath>

#ifdef __CUDACC__
#define DF_HD __host__ __device__ __forceinline__
#else
#define DF_HD inline
#endif

namespace gsgpu {

// rounding-exact single operations (no contraction of a*b+c into an FMA)
DF_HD float fadd(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    volatile float r = a + b;
    return r;
#endif
}
DF_HD float fsub(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    volatile float r = a - b;
    return r;
#endif
}
DF_HD float fmul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    volatile float r = a * b;
    return r;
#endif
}
DF_HD float ffma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}

struct alignas(8) df32 {
    float hi, lo;
    DF_HD df32() : hi(0.f), lo(0.f) {}
    DF_HD df32(float h, float l) : hi(h), lo(l) {}
    DF_HD explicit df32(double d) {
        hi = float(d);
        lo = float(d - double(hi));
    }
    DF_HD explicit df32(int v) : hi(float(v)), lo(0.f) {}
    DF_HD double toDouble() const { return double(hi) + double(lo); }
};

// s + e = a + b exactly
DF_HD void twoSum(float a, float b, float& s, float& e) {
    s = fadd(a, b);
    const float bb = fsub(s, a);
    e = fadd(fsub(a, fsub(s, bb)), fsub(b, bb));
}
// s + e = a + b exactly, for |a| >= |b|
DF_HD void fastTwoSum(float a, float b, float& s, float& e) {
    s = fadd(a, b);
    e = fsub(b, fsub(s, a));
}
// p + e = a * b exactly
DF_HD void twoProd(float a, float b, float& p, float& e) {
    p = fmul(a, b);
    e = ffma(a, b, -p);
}

DF_HD df32 operator-(df32 a) { return df32(-a.hi, -a.lo); }

DF_HD df32 operator+(df32 a, df32 b) {
    float s1, s2, t1, t2;
    twoSum(a.hi, b.hi, s1, s2);
    twoSum(a.lo, b.lo, t1, t2);
    s2 = fadd(s2, t1);
    fastTwoSum(s1, s2, s1, s2);
    s2 = fadd(s2, t2);
    fastTwoSum(s1, s2, s1, s2);
    return df32(s1, s2);
}
DF_HD df32 operator-(df32 a, df32 b) { return a + (-b); }
DF_HD df32 operator*(df32 a, df32 b) {
    float p, e;
    twoProd(a.hi, b.hi, p, e);
    e = ffma(a.hi, b.lo, e);
    e = ffma(a.lo, b.hi, e);
    fastTwoSum(p, e, p, e);
    return df32(p, e);
}
DF_HD df32 operator*(df32 a, float b) {
    float p, e;
    twoProd(a.hi, b, p, e);
    e = ffma(a.lo, b, e);
    fastTwoSum(p, e, p, e);
    return df32(p, e);
}
// long division: q1 = a/b in FP32, correction from the df32 remainder
DF_HD df32 operator/(df32 a, df32 b) {
    const float q1 = a.hi / b.hi;
    const df32 r = a - b * q1;
    const float q2 = r.hi / b.hi;
    const df32 r2 = r - b * q2;
    const float q3 = r2.hi / b.hi;
    float s, e;
    fastTwoSum(q1, q2, s, e);
    df32 q(s, e);
    return q + df32(q3, 0.f);
}
DF_HD df32& operator+=(df32& a, df32 b) { return a = a + b; }
DF_HD df32& operator-=(df32& a, df32 b) { return a = a - b; }
DF_HD df32& operator*=(df32& a, df32 b) { return a = a * b; }
DF_HD df32 dfabs(df32 a) { return a.hi < 0.f ? -a : a; }
DF_HD df32 ldexpDf(df32 a, int k) { return df32(ldexpf(a.hi, k), ldexpf(a.lo, k)); }

// compensated dot-product accumulator (Dot2): sum of products kept as s (FP32) plus an
// uncorrected error term c; products of df32 factors add their cross terms into c
struct Dot2 {
    float s = 0.f, c = 0.f;
    DF_HD void mac(df32 a, df32 b) {
        float p, e;
        twoProd(a.hi, b.hi, p, e);
        e = ffma(a.hi, b.lo, e);
        e = ffma(a.lo, b.hi, e);
        float t;
        twoSum(s, p, s, t);
        c = fadd(c, fadd(t, e));
    }
    // += a * b for an FP32 factor b
    DF_HD void mac(df32 a, float b) {
        float p, e;
        twoProd(a.hi, b, p, e);
        e = ffma(a.lo, b, e);
        float t;
        twoSum(s, p, s, t);
        c = fadd(c, fadd(t, e));
    }
    // += a
    DF_HD void add(df32 a) {
        float t;
        twoSum(s, a.hi, s, t);
        c = fadd(c, fadd(t, a.lo));
    }
    DF_HD void add(const Dot2& o) {
        float t;
        twoSum(s, o.s, s, t);
        c = fadd(c, fadd(t, o.c));
    }
    DF_HD df32 result() const {
        float h, l;
        fastTwoSum(s, c, h, l);
        return df32(h, l);
    }
};

// a*b + sgn*c*d with one rounding step: both products exact by TwoProduct, their cross terms and
// the error of the FP32 sum collected in one FP32 correction (the two-term case of Dot2); error
// about 2^-47 (|ab| + |cd|)
DF_HD df32 dot2Terms(df32 a, df32 b, df32 c, df32 d, float sgn) {
    float p1, e1, p2, e2;
    twoProd(a.hi, b.hi, p1, e1);
    e1 = ffma(a.hi, b.lo, e1);
    e1 = ffma(a.lo, b.hi, e1);
    const float ch = fmul(sgn, c.hi), cl = fmul(sgn, c.lo);
    twoProd(ch, d.hi, p2, e2);
    e2 = ffma(ch, d.lo, e2);
    e2 = ffma(cl, d.hi, e2);
    float sh, t;
    twoSum(p1, p2, sh, t);
    const float lo = fadd(fadd(e1, e2), t);
    fastTwoSum(sh, lo, sh, t);
    return df32(sh, t);
}

// -------------------------------------------------------------------------------------------
// constants as df32 (hi + lo of the double value)
DF_HD df32 dfPi() { return df32(3.14159274101257324e+00f, -8.74227800037248965e-08f); }
DF_HD df32 dfLn2() { return df32(6.93147182464599609e-01f, -1.90465429995776755e-09f); }

// sin(pi x), cos(pi x) for df32 x: x = n/2 + t with n integer and |t| <= 1/4, then the Taylor
// series of sin and cos at theta = pi t (|theta| <= pi/4) in df32 and a quarter-turn rotation
DF_HD void sincospiDf(df32 x, df32& s, df32& c) {
    const float n = rintf(fmul(2.f, x.hi));
    float th, tl;
    fastTwoSum(fsub(x.hi, fmul(0.5f, n)), x.lo, th, tl);  // x.hi - n/2 is exact (Sterbenz)
    const df32 t(th, tl);
    const df32 a = t * dfPi();
    const df32 a2 = a * a;
    // inverse factorials 1/k!, k = 0..19, as df32
    const double inv[20] = {1.0,
                            1.0,
                            0.5,
                            1.6666666666666666e-01,
                            4.1666666666666664e-02,
                            8.3333333333333332e-03,
                            1.3888888888888889e-03,
                            1.9841269841269841e-04,
                            2.4801587301587302e-05,
                            2.7557319223985893e-06,
                            2.7557319223985888e-07,
                            2.5052108385441720e-08,
                            2.0876756987868100e-09,
                            1.6059043836821613e-10,
                            1.1470745597729725e-11,
                            7.6471637318198164e-13,
                            4.7794773323873853e-14,
                            2.8114572543455206e-15,
                            1.5619206968586225e-16,
                            8.2206352466243295e-18};
    // sin(a) = a sum_{j=0..7} (-1)^j a^(2j) / (2j+1)!,  cos(a) = sum_{j=0..8} (-1)^j a^(2j) / (2j)!
    // |a| <= pi/4, so the first omitted terms are below (pi/4)^16/17!/0.90 < 7e-17 of sin(a) and
    // (pi/4)^18/18! < 3e-18 of cos(a) >= 0.707, both under the df32 unit 2^-48 = 3.6e-15.
    // The tails j >= 6 of both sums (at most (pi/4)^12/13! = 9e-12 and (pi/4)^12/12! = 1.2e-10 of
    // the sum) are summed in FP32 from the FP32 part of a^2: their rounding (a few 2^-24 of the
    // tail) and the dropped low part of a^2 (relative 2^-24 raised to at most the 8th power) stay
    // below 1e-16; the leading terms run in df32
    const float a2f = a2.hi;
    float st = float(-inv[15]);
    st = ffma(a2f, st, float(inv[13]));
    df32 sp(st, 0.f);
    for (int j = 5; j >= 0; --j) sp = df32((j % 2 ? -1.0 : 1.0) * inv[2 * j + 1]) + a2 * sp;
    float ct = float(inv[16]);
    for (int j = 7; j >= 6; --j) ct = ffma(a2f, ct, float((j % 2 ? -1.0 : 1.0) * inv[2 * j]));
    df32 cp(ct, 0.f);
    for (int j = 5; j >= 0; --j) cp = df32((j % 2 ? -1.0 : 1.0) * inv[2 * j]) + a2 * cp;
    const df32 sa = a * sp, ca = cp;
    const int q = ((int)n) & 3;
    if (q == 0) { s = sa; c = ca; }
    else if (q == 1) { s = ca; c = -sa; }
    else if (q == 2) { s = -sa; c = -ca; }
    else { s = -ca; c = sa; }
}

// exp(y) = 2^k exp(r), y = k ln2 + r, exp(r) = (exp(r/16))^16 with a Taylor series for exp(r/16)
DF_HD df32 expDf(df32 y) {
    const float k = rintf(y.hi * 1.44269504088896341f);
    df32 r = y - dfLn2() * k;
    r = df32(fmul(r.hi, 0.0625f), fmul(r.lo, 0.0625f));
    // degree 7: |r/16| <= ln2/32, so the first omitted term (ln2/32)^8/8! < 1.3e-18, and below
    // 2.1e-17 after the 4 squarings. The tail j >= 5 (at most (ln2/32)^5/5! = 4e-11) is summed in
    // FP32 from the FP32 part of r: its error, 16 times that after the squarings, stays below 1e-16
    const double inv[8] = {1.0, 1.0, 0.5, 1.6666666666666666e-01, 4.1666666666666664e-02, 8.3333333333333332e-03,
                           1.3888888888888889e-03, 1.9841269841269841e-04};
    float et = float(inv[7]);
    for (int j = 6; j >= 5; --j) et = ffma(r.hi, et, float(inv[j]));
    df32 e(et, 0.f);
    for (int j = 4; j >= 0; --j) e = df32(inv[j]) + r * e;
    for (int j = 0; j < 4; ++j) e = e * e;
    return ldexpDf(e, int(k));
}

}  // namespace gsgpu
