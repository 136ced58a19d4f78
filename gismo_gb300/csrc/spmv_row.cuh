// Row products of the CSR SpMV-type kernels: the LPR-strided share of sum_k A(row, col_k) x[col_k]
// taken by one lane. The loop is unrolled U times and issues all U (value, column) loads before
// the U dependent x loads, so each lane keeps U independent load chains in flight. With a single
// chain per lane the kernels wait on load latency instead of filling HBM (measured: 31% of DRAM
// peak on a 512-patch matrix with 32-bit column indices). The accumulation order is the plain
// k = kb+lane, kb+lane+LPR, ... order, so results do not depend on U.
#pragma once

#include <cstdint>

namespace gsgpu {
namespace dev {

// column of CSR slot k: absolute (col) or relative to the row (coff, banded patterns)
template <bool REL>
__device__ __forceinline__ int csrCol(int row, int k, const int* __restrict__ col, const int16_t* __restrict__ coff) {
    if (REL) return row + int(coff[k]);
    return col[k];
}

// fv(k): matrix value of slot k; fx(c): vector entry c; fm(v, x): accumulate v * x
template <int LPR, int U, bool REL, class FV, class FX, class FM>
__device__ __forceinline__ void rowMac(int row, int kb, int ke, int lane, const int* __restrict__ col,
                                       const int16_t* __restrict__ coff, FV fv, FX fx, FM fm) {
    int k = kb + lane;
    for (; k + (U - 1) * LPR < ke; k += U * LPR) {
        decltype(fv(0)) v[U];
        int c[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            v[u] = fv(k + u * LPR);
            c[u] = csrCol<REL>(row, k + u * LPR, col, coff);
        }
        decltype(fx(0)) xv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) xv[u] = fx(c[u]);
#pragma unroll
        for (int u = 0; u < U; ++u) fm(v[u], xv[u]);
    }
    for (; k < ke; k += LPR) fm(fv(k), fx(csrCol<REL>(row, k, col, coff)));
}

// a row whose columns are row + box[j], j = k - kb: the same slots, loads and accumulation order
// as rowMac, with the column offsets read from a shared-memory table instead of HBM
template <int LPR, int U, class FV, class FX, class FM>
__device__ __forceinline__ void rowMacBox(int row, int kb, int ke, int lane, const int* box, FV fv, FX fx, FM fm) {
    const int len = ke - kb;
    int j = lane;
    for (; j + (U - 1) * LPR < len; j += U * LPR) {
        decltype(fv(0)) v[U];
        int c[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            v[u] = fv(kb + j + u * LPR);
            c[u] = row + box[j + u * LPR];
        }
        decltype(fx(0)) xv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) xv[u] = fx(c[u]);
#pragma unroll
        for (int u = 0; u < U; ++u) fm(v[u], xv[u]);
    }
    for (; j < len; j += LPR) fm(fv(kb + j), fx(row + box[j]));
}

// rowMac without a serial tail: every step issues all U loads, slots past the row end predicated
// off (value 0, column row), so a row takes ceil(len / (U LPR)) steps with U loads in flight each.
// A masked slot adds fma(0, x, s) = s, so the sums equal rowMac's bit for bit.
template <int LPR, int U, bool REL, class FV, class FX, class FM>
__device__ __forceinline__ void rowMacP(int row, int kb, int ke, int lane, const int* __restrict__ col,
                                        const int16_t* __restrict__ coff, FV fv, FX fx, FM fm) {
    using V = decltype(fv(0));
    for (int k = kb + lane; k < ke; k += U * LPR) {
        V v[U];
        int c[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int kk = k + u * LPR;
            const bool ok = kk < ke;
            v[u] = ok ? fv(kk) : V(0);
            c[u] = ok ? csrCol<REL>(row, kk, col, coff) : row;
        }
        decltype(fx(0)) xv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) xv[u] = fx(c[u]);
#pragma unroll
        for (int u = 0; u < U; ++u) fm(v[u], xv[u]);
    }
}

// rowMacBox with predicated steps (see rowMacP)
template <int LPR, int U, class FV, class FX, class FM>
__device__ __forceinline__ void rowMacBoxP(int row, int kb, int ke, int lane, const int* box, FV fv, FX fx, FM fm) {
    using V = decltype(fv(0));
    const int len = ke - kb;
    for (int j = lane; j < len; j += U * LPR) {
        V v[U];
        int c[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int jj = j + u * LPR;
            const bool ok = jj < len;
            v[u] = ok ? fv(kb + jj) : V(0);
            c[u] = ok ? row + box[jj] : row;
        }
        decltype(fx(0)) xv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) xv[u] = fx(c[u]);
#pragma unroll
        for (int u = 0; u < U; ++u) fm(v[u], xv[u]);
    }
}

}  // namespace dev
}  // namespace gsgpu
