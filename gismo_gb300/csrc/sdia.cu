// Half-diagonal storage of the FP32 inner operator of a single tensor-product patch, and its SpMV.
//
// When the free dofs of a problem are one box of m0 x m1 x m2 patch-local functions numbered
// lexicographically (a single patch with Dirichlet sides eliminated: gsDofMapper numbers the free
// functions in scan order), the row of free dof i = (i0, i1, i2) couples to the free dofs i + o
// with o in the neighbour box [-p0, p0] x [-p1, p1] x [-p2, p2], and the linear index of i + o is
// i + L(o) with L(o) = o0 + m0 (o1 + m1 o2). The matrix is symmetric, so only the offsets of the
// half box H = {o : (o2, o1, o0) >= 0 lexicographically} are stored, as diagonals:
//   d[h * ns + i] = A(i, i + o_h)  if i + o_h lies in the box, else 0   (ns = n rounded up to 256).
// Row i of A x is then
//   sum_{h} d[h ns + i] x[i + L_h]  +  sum_{h, o_h != 0} d[h ns + i - L_h] x[i - L_h]
// (A(i, i - o) = A(i - o, i) is the stored entry of row i - o). A linear index inside [0, n) whose
// tensor point lies outside the box reads a stored 0, so only the linear bounds are tested.
// Compared with the CSR form (a 4-byte value plus column data per non-zero), the operator streams
// 4 bytes per stored half-box entry: 189 MB instead of 384 MB per product for the degree-3 64^3
// volume. Each stored value is read twice, by its own row and by the mirrored one; all blocks run
// through the diagonals in the same order, so the second read finds the value in L2.
#include <cuda.h>  // CUtensorMap and its encoder's types (the encoder is fetched through the runtime)
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdint>
#include <string>

#include "context.h"
#include "df32.cuh"
#include "kernels_solve.h"
#include "pdl.cuh"

namespace gsgpu {
namespace {

constexpr int kB = 256;

// the half-box offsets in storage order: the centre line (0, 0, o0 >= 0) first, then the lines
// (o2, o1) with o2 > 0 or (o2 = 0, o1 > 0), o0 ascending within a line
__host__ __device__ inline int halfCount(const int* p) {
    return 1 + ((2 * p[0] + 1) * (2 * p[1] + 1) * (2 * p[2] + 1) - 1) / 2;
}

// d from the band of the patch (df32 values: the FP32 inner operator is their hi part, as in the
// CSR gather). One thread per free row; band entry of row c (patch-local) and offset o is
// band_off + (c0 W0 + o0 + p0) + (c1 W1 + o1 + p1) n0 W0 + (c2 W2 + o2 + p2) n0 W0 n1 W1.
__global__ void __launch_bounds__(kB) k_sdia_build(SdiaOp A, SdiaBand B, const df32* __restrict__ band,
                                                  float* __restrict__ d) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const long long ns = A.ns;
    if (r >= ns) return;
    if (r >= A.n) {  // the padding of every diagonal holds zeros (the products read it times x = 0)
        for (int h = 0; h < A.nh; ++h) d[h * ns + r] = 0.f;
        return;
    }
    int b[3];
    b[0] = r % A.m[0];
    b[1] = (r / A.m[0]) % A.m[1];
    b[2] = r / (A.m[0] * A.m[1]);
    const long long n0W = (long long)B.n[0] * B.W[0], n1W = (long long)B.n[1] * B.W[1];
    const long long rowBase = B.band_off + (long long)(b[0] + B.lo[0]) * B.W[0] +
                              (long long)(b[1] + B.lo[1]) * B.W[1] * n0W +
                              (long long)(b[2] + B.lo[2]) * B.W[2] * n0W * n1W;
    auto value = [&](int o0, int o1, int o2) -> float {
        const int c0 = b[0] + o0, c1 = b[1] + o1, c2 = b[2] + o2;
        if (c0 < 0 || c0 >= A.m[0] || c1 < 0 || c1 >= A.m[1] || c2 < 0 || c2 >= A.m[2]) return 0.f;
        const long long bi = rowBase + (o0 + A.p[0]) + (long long)(o1 + A.p[1]) * n0W +
                             (long long)(o2 + A.p[2]) * n0W * n1W;
        return band[bi].hi;
    };
    int h = 0;
    for (int o0 = 0; o0 <= A.p[0]; ++o0, ++h) d[h * ns + r] = value(o0, 0, 0);
    for (int o2 = 0; o2 <= A.p[2]; ++o2)
        for (int o1 = o2 ? -A.p[1] : 1; o1 <= A.p[1]; ++o1)
            for (int o0 = -A.p[0]; o0 <= A.p[0]; ++o0, ++h) d[h * ns + r] = value(o0, o1, o2);
}

__device__ __forceinline__ double warpSumD(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ void prefetchL2(const float* a) {
    asm volatile("prefetch.global.L2 [%0];" ::"l"(a));
}

// t = A x from the half diagonals (one thread per row, grid-stride) and block partial sums of x.t
// (the p.Ap of the inner CG), in FP64 over FP32 products as in the CSR kernel. x carries A.xpad >=
// max L zeros before and after its n entries, and the diagonals' padding [n, ns) holds zeros, so
// every index below stays in allocated memory and a term whose row or column leaves [0, n) is a
// product with a zero: the mirrored index h ns + r - L with r - L < 0 falls into diagonal h - 1
// (finite there) and meets x[r - L] = 0; an upper term with r + L >= n has d = 0 (the tensor point
// r + o lies outside the box) and x[r + L] = 0. The row's own values d[h ns + r] are the only
// ones read from HBM first (the mirrored ones were read by their own rows at about the same
// time): each warp prefetches them into L2 two lines ahead.
template <int P0>
__global__ void __launch_bounds__(kB) k_sdia32_dot(SdiaOp A, const float* __restrict__ x, float* __restrict__ t,
                                                   double* __restrict__ part, const CgState* __restrict__ st) {
    if (st->done || st->pause) return;
    constexpr int W0 = 2 * P0 + 1;
    constexpr int kAhead = 2;
    const int n = A.n;
    const long long ns = A.ns;
    const int nlines = A.p[1] + A.p[2] * (2 * A.p[1] + 1);
    double contrib = 0.0;
    for (int base = blockIdx.x * kB; base < n; base += gridDim.x * kB) {
        const int r = base + threadIdx.x;
        if (r < n) {
            float acc = 0.f;
            const float* dh = A.d + r;
            for (int l = 0; l < kAhead && l < nlines; ++l)
#pragma unroll
                for (int k = 0; k < W0; ++k) prefetchL2(dh + (P0 + 1 + l * W0 + k) * ns);
            // centre line: o = (0, 0, o0), o0 = 0..P0 (the diagonal first)
#pragma unroll
            for (int o0 = 0; o0 <= P0; ++o0) {
                acc = fmaf(__ldcg(dh), __ldg(x + r + o0), acc);
                if (o0 > 0) acc = fmaf(__ldcg(dh - o0), __ldg(x + r - o0), acc);
                dh += ns;
            }
            int line = 0;
            for (int o2 = 0; o2 <= A.p[2]; ++o2)
                for (int o1 = o2 ? -A.p[1] : 1; o1 <= A.p[1]; ++o1, ++line) {
                    if (line + kAhead < nlines)
#pragma unroll
                        for (int k = 0; k < W0; ++k) prefetchL2(dh + (kAhead * W0 + k) * ns);
                    const int L21 = (o2 * A.m[1] + o1) * A.m[0];
                    float vu[W0], xu[W0], vd[W0], xd[W0];
#pragma unroll
                    for (int k = 0; k < W0; ++k) {
                        const int L = L21 + k - P0;
                        vu[k] = __ldcg(dh + k * ns);
                        vd[k] = __ldcg(dh + k * ns - L);
                        xu[k] = __ldg(x + r + L);
                        xd[k] = __ldg(x + r - L);
                    }
                    // a line's 2 (2 P0 + 1) products are summed first, then added to the row sum:
                    // two short FP32 chains instead of one of (2p+1)^3 terms
                    float lsum = 0.f;
#pragma unroll
                    for (int k = 0; k < W0; ++k) {
                        lsum = fmaf(vu[k], xu[k], lsum);
                        lsum = fmaf(vd[k], xd[k], lsum);
                    }
                    acc += lsum;
                    dh += W0 * ns;
                }
            t[r] = acc;
            contrib += double(acc) * double(x[r]);
        }
    }
    __shared__ double ws[kB / 32];
    contrib = warpSumD(contrib);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = contrib;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int w = 0; w < kB / 32; ++w) sum += ws[w];
        part[blockIdx.x] = sum;
    }
}

// ---------------------------------------------------------------------------------------------
// The same product with four consecutive rows r0 .. r0 + 3 (r0 = 4 g) per thread. The row's own
// values of a diagonal are one 16-byte load; x is read as aligned windows of 16-byte loads that
// the four rows and the 2 P0 + 1 offsets of a line share (x[r0 + L + j] for every offset L of the
// line and row j); the mirrored values d[h ns + r0 + j - L] of diagonal h as the two aligned
// 16-byte loads around them. Where a window starts inside its first 16 bytes depends only on the
// line offset L21 modulo 4, so the line body is instantiated per residue and every pick from a
// window is a register move. Each row sums its terms in the order of k_sdia32_dot: both products
// give the same bits. Compared with one row per thread this issues a quarter of the load
// instructions and reads x with a fraction of the L1 wavefronts (one pass over each window
// instead of one unaligned load per offset). Blocks take equal contiguous shares of the row
// groups (kG4Blocks per SM, all resident), so no SM gets a block more than another.
constexpr int kG = 4;           // rows per thread
constexpr int kBG = 128;        // threads per block
constexpr int kG4BlocksPerSm = 4;
constexpr int kG4Ahead = 1;     // lines of own values prefetched into L2 ahead of their use (swept: 0-4)

constexpr int mod4(int a) { return ((a % 4) + 4) % 4; }

template <int NV>
__device__ __forceinline__ void loadWin(const float* p, float (&w)[4 * NV]) {
#pragma unroll
    for (int v = 0; v < NV; ++v) {
        const float4 q = __ldg(reinterpret_cast<const float4*>(p) + v);
        w[4 * v] = q.x;
        w[4 * v + 1] = q.y;
        w[4 * v + 2] = q.z;
        w[4 * v + 3] = q.w;
    }
}
__device__ __forceinline__ void loadD2(const float* p, float (&w)[8]) {
    const float4 a = __ldcg(reinterpret_cast<const float4*>(p));
    const float4 b = __ldcg(reinterpret_cast<const float4*>(p) + 1);
    w[0] = a.x, w[1] = a.y, w[2] = a.z, w[3] = a.w;
    w[4] = b.x, w[5] = b.y, w[6] = b.z, w[7] = b.w;
}

// one (o2, o1) line for rows r0 .. r0 + 3: dh = d + h_l ns + r0, L21 = (o2 m1 + o1) m0 = C mod 4
template <int P0, int C>
__device__ __forceinline__ void lineG4(const float* __restrict__ dh, long long ns, const float* __restrict__ x, int r0,
                                       int L21, float (&acc)[kG]) {
    constexpr int W0 = 2 * P0 + 1;
    constexpr int SU = mod4(C - P0);         // x[r0 + L21 - P0 + i] = xu[SU + i]
    constexpr int SD = mod4(-C - P0);        // x[r0 - L21 - P0 + i] = xd[SD + i]
    constexpr int NU = (SU + W0 + 2) / 4 + 1;  // 16-byte loads covering indices 0 .. SU + W0 + 2
    constexpr int ND = (SD + W0 + 2) / 4 + 1;
    float xu[4 * NU], xd[4 * ND];
    loadWin<NU>(x + r0 + L21 - P0 - SU, xu);
    loadWin<ND>(x + r0 - L21 - P0 - SD, xd);
    float lsum[kG] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int k = 0; k < W0; ++k) {
        // own: d[(h_l + k) ns + r0 + j]; mirrored: d[(h_l + k) ns + r0 + j - L], L = L21 + k - P0,
        // read from the aligned pair starting SM floats before r0 - L
        const float4 v = __ldcg(reinterpret_cast<const float4*>(dh + k * ns));
        const int SM = mod4(P0 - C - k);
        float m[8];
        loadD2(dh + k * ns - L21 + P0 - k - SM, m);
        const float vu[kG] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int j = 0; j < kG; ++j) {
            lsum[j] = fmaf(vu[j], xu[SU + k + j], lsum[j]);
            lsum[j] = fmaf(m[SM + j], xd[SD + 2 * P0 - k + j], lsum[j]);
        }
    }
#pragma unroll
    for (int j = 0; j < kG; ++j) acc[j] += lsum[j];
}

template <int P0>
__global__ void __launch_bounds__(kBG, kG4BlocksPerSm) k_sdia32_g4(SdiaOp A, const float* __restrict__ x,
                                                                   float* __restrict__ t, double* __restrict__ part,
                                                                   const CgState* __restrict__ st) {
    pdlWait();
    if (st->done || st->pause) return;
    constexpr int W0 = 2 * P0 + 1;
    constexpr int kAhead = kG4Ahead;
    const int n = A.n;
    const long long ns = A.ns;
    const int nlines = A.p[1] + A.p[2] * (2 * A.p[1] + 1);
    const int ngroups = (n + kG - 1) / kG;
    const int share = (ngroups + int(gridDim.x) - 1) / int(gridDim.x);
    const int gEnd = min(ngroups, (int(blockIdx.x) + 1) * share);
    double contrib = 0.0;
    for (int g = int(blockIdx.x) * share + int(threadIdx.x); g < gEnd; g += kBG) {
        const int r0 = g * kG;
        const float* dh = A.d + r0;
        for (int l = 0; l < kAhead && l < nlines; ++l)
#pragma unroll
            for (int k = 0; k < W0; ++k) prefetchL2(dh + (P0 + 1 + l * W0 + k) * ns);
        // centre line: x[r0 - 4 .. r0 + 8) covers r0 + j +- o0; the mirrored values of diagonal o0
        // (d[o0 ns + r0 + j - o0]) lie in the aligned pair starting at r0 - 4
        float xc[12];
        loadWin<3>(x + r0 - 4, xc);
        float acc[kG];
        {
            const float4 v = __ldcg(reinterpret_cast<const float4*>(dh));
            const float v0[kG] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int j = 0; j < kG; ++j) acc[j] = fmaf(v0[j], xc[4 + j], 0.f);
        }
#pragma unroll
        for (int o0 = 1; o0 <= P0; ++o0) {
            dh += ns;
            const float4 v = __ldcg(reinterpret_cast<const float4*>(dh));
            const float vu[kG] = {v.x, v.y, v.z, v.w};
            float m[8];
            loadD2(dh - 4, m);
#pragma unroll
            for (int j = 0; j < kG; ++j) {
                acc[j] = fmaf(vu[j], xc[4 + j + o0], acc[j]);
                acc[j] = fmaf(m[4 + j - o0], xc[4 + j - o0], acc[j]);
            }
        }
        dh += ns;
        int line = 0;
        for (int o2 = 0; o2 <= A.p[2]; ++o2)
            for (int o1 = o2 ? -A.p[1] : 1; o1 <= A.p[1]; ++o1, ++line) {
                if (line + kAhead < nlines)
#pragma unroll
                    for (int k = 0; k < W0; ++k) prefetchL2(dh + (kAhead * W0 + k) * ns);
                const int L21 = (o2 * A.m[1] + o1) * A.m[0];
                switch (L21 & 3) {
                    case 0: lineG4<P0, 0>(dh, ns, x, r0, L21, acc); break;
                    case 1: lineG4<P0, 1>(dh, ns, x, r0, L21, acc); break;
                    case 2: lineG4<P0, 2>(dh, ns, x, r0, L21, acc); break;
                    default: lineG4<P0, 3>(dh, ns, x, r0, L21, acc); break;
                }
                dh += W0 * ns;
            }
        if (r0 + kG <= n) {
            *reinterpret_cast<float4*>(t + r0) = make_float4(acc[0], acc[1], acc[2], acc[3]);
#pragma unroll
            for (int j = 0; j < kG; ++j) contrib += double(acc[j]) * double(xc[4 + j]);
        } else {
            for (int j = 0; j < kG && r0 + j < n; ++j) {
                t[r0 + j] = acc[j];
                contrib += double(acc[j]) * double(xc[4 + j]);
            }
        }
    }
    pdlTrigger();
    __shared__ double ws[kBG / 32];
    contrib = warpSumD(contrib);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = contrib;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int w = 0; w < kBG / 32; ++w) sum += ws[w];
        part[blockIdx.x] = sum;
    }
}

// ---------------------------------------------------------------------------------------------
// The same product fed by the Tensor Memory Accelerator. A block owns tiles of kTmaT consecutive
// rows [r0, r0 + kTmaT); per tile it walks the lines of the half box (the centre line, then the
// (o2, o1) lines), and per line one elected thread issues four tiled bulk copies into a
// shared-memory stage of a kTmaStages-deep ring, completing on the stage's mbarrier:
//   Dup: diagonals h_l .. h_l + W0 - 1, columns [r0, r0 + kTmaBox)          (the row's own values)
//   Ddn: the same diagonals, columns [a_d, a_d + kTmaBox), a_d = floor4(r0 - L21 - P0)
//        (the mirrored values d[h][i - L]: i - L = i - L21 - o0 runs over [r0 - L21 - P0, ...))
//   Xup: x[a_u, a_u + kTmaBox), a_u = floor4(r0 + L21 - P0)                   (x[i + L])
//   Xdn: x[a_d, a_d + kTmaBox)                                                (x[i - L])
// Box starts are rounded down to 16 bytes (the tiled-copy rule for the innermost coordinate);
// coordinates outside the arrays read zeros, which is the value of every term whose row or
// column leaves [0, n): no clamping in the inner loop, which reads shared memory only. The centre
// line uses L21 = P0 with the first P0 + 1 diagonals (o0 = k, k = 0..P0), so one index formula
// serves all lines. A stage is refilled once every thread has passed the block barrier after
// reading it. Every mbarrier wait is bounded: on expiry the block records the failure in *err,
// waits (bounded) for the copies it issued and returns.
constexpr int kTmaT = 240;       // rows per tile (a multiple of 4: r0 is 16-byte aligned)
constexpr int kTmaBox = 252;     // box width in floats: kTmaT + 2 P0 + 3 rounded up to 4, P0 <= 4
constexpr int kTmaThreads = 256;
constexpr int kTmaStages = 4;
constexpr int kTmaBlocksPerSm = 3;
constexpr unsigned kWaitPolls = 1u << 22;  // ~0.5 s of polling at the back-off below

template <int P0>
struct TmaShape {
    static constexpr int W0 = 2 * P0 + 1;
    static constexpr int DREG = (W0 * kTmaBox * 4 + 127) / 128 * 128;  // bytes of one D box
    static constexpr int XREG = (kTmaBox * 4 + 127) / 128 * 128;       // bytes of one x box
    static constexpr int STAGE = 2 * DREG + 2 * XREG;
    static constexpr unsigned TX = 2u * W0 * kTmaBox * 4 + 2u * kTmaBox * 4;  // bytes a stage receives
    static constexpr int SMEM = kTmaStages * STAGE + kTmaStages * 8 + 128;  // + alignment slack
};

__device__ __forceinline__ unsigned smemAddr(const void* p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbarInit(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbarExpectTx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbarTest(uint64_t* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smemAddr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// bounded wait for the phase of `parity` to complete
__device__ __forceinline__ bool mbarWait(uint64_t* bar, unsigned parity) {
    for (unsigned k = 0; k < kWaitPolls; ++k) {
        if (mbarTest(bar, parity)) return true;
        if (k > 64) __nanosleep(64);
    }
    return false;
}
__device__ __forceinline__ void tmaLoad2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smemAddr(dst)),
        "l"(map), "r"(x), "r"(y), "r"(smemAddr(bar))
        : "memory");
}
__device__ __forceinline__ void tmaLoad1d(void* dst, const CUtensorMap* map, int x, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.1d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2}], [%3];" ::"r"(
            smemAddr(dst)),
        "l"(map), "r"(x), "r"(smemAddr(bar))
        : "memory");
}

// line q of a tile: its offset L21 (the centre line: P0) and first diagonal h_l
__device__ __forceinline__ void lineOf(int q, int P0, const SdiaOp& A, int& L21, int& hl) {
    if (q == 0) {
        L21 = P0;
        hl = 0;
        return;
    }
    const int l = q - 1;
    int o2, o1;
    if (l < A.p[1]) {
        o2 = 0;
        o1 = l + 1;
    } else {
        const int w = 2 * A.p[1] + 1;
        o2 = 1 + (l - A.p[1]) / w;
        o1 = (l - A.p[1]) % w - A.p[1];
    }
    L21 = (o2 * A.m[1] + o1) * A.m[0];
    hl = P0 + 1 + l * (2 * P0 + 1);
}

template <int P0>
__global__ void __launch_bounds__(kTmaThreads) k_sdia32_tma(const __grid_constant__ CUtensorMap mapD,
                                                            const __grid_constant__ CUtensorMap mapX, SdiaOp A,
                                                            float* __restrict__ t, double* __restrict__ part,
                                                            const CgState* __restrict__ st, int* __restrict__ err) {
    if (st->done || st->pause) return;
    using S = TmaShape<P0>;
    constexpr int W0 = S::W0;
    extern __shared__ __align__(128) unsigned char smemRaw[];
    // tiled copies land on 128-byte aligned stages
    unsigned char* smem = smemRaw + ((128u - (smemAddr(smemRaw) & 127u)) & 127u);
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + kTmaStages * S::STAGE);
    const int n = A.n;
    const int nlines = 1 + A.p[1] + A.p[2] * (2 * A.p[1] + 1);
    const int ntiles = (n + kTmaT - 1) / kTmaT;
    const int mytiles = (ntiles - int(blockIdx.x) + int(gridDim.x) - 1) / int(gridDim.x);
    const int njobs = mytiles * nlines;
    if (threadIdx.x == 0) {
        for (int k = 0; k < kTmaStages; ++k) mbarInit(&full[k], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    auto issue = [&](int j) {
        unsigned char* sb = smem + (j % kTmaStages) * S::STAGE;
        uint64_t* bar = &full[j % kTmaStages];
        const int r0 = (int(blockIdx.x) + (j / nlines) * int(gridDim.x)) * kTmaT;
        int L21, hl;
        lineOf(j % nlines, P0, A, L21, hl);
        const int au = (r0 + L21 - P0) & ~3;
        const int ad = (r0 - L21 - P0) & ~3;
        mbarExpectTx(bar, S::TX);
        tmaLoad2d(sb, &mapD, r0, hl, bar);
        tmaLoad2d(sb + S::DREG, &mapD, ad, hl, bar);
        tmaLoad1d(sb + 2 * S::DREG, &mapX, au, bar);
        tmaLoad1d(sb + 2 * S::DREG + S::XREG, &mapX, ad, bar);
    };
    if (threadIdx.x == 0)
        for (int j = 0; j < kTmaStages && j < njobs; ++j) issue(j);
    const int tt = threadIdx.x;
    float acc = 0.f, xr = 0.f;
    double contrib = 0.0;
    bool failed = false;
    int j = 0;
    for (; j < njobs; ++j) {
        const int stage = j % kTmaStages;
        const bool ok = mbarWait(&full[stage], unsigned(j / kTmaStages) & 1u);
        if (!__syncthreads_and(ok)) {
            failed = true;
            break;
        }
        const unsigned char* sb = smem + stage * S::STAGE;
        const float* Du = reinterpret_cast<const float*>(sb);
        const float* Dd = reinterpret_cast<const float*>(sb + S::DREG);
        const float* Xu = reinterpret_cast<const float*>(sb + 2 * S::DREG);
        const float* Xd = reinterpret_cast<const float*>(sb + 2 * S::DREG + S::XREG);
        const int q = j % nlines;
        const int r0 = (int(blockIdx.x) + (j / nlines) * int(gridDim.x)) * kTmaT;
        int L21, hl;
        lineOf(q, P0, A, L21, hl);
        const int su = (r0 + L21 - P0) - ((r0 + L21 - P0) & ~3);
        const int sd = (r0 - L21 - P0) - ((r0 - L21 - P0) & ~3);
        if (tt < kTmaT) {
            if (q == 0) {
                acc = 0.f;
                xr = Xu[tt + su];
#pragma unroll
                for (int k = 0; k <= P0; ++k) {
                    acc = fmaf(Du[k * kTmaBox + tt], Xu[tt + k + su], acc);
                    if (k > 0) acc = fmaf(Dd[k * kTmaBox + tt + sd + 2 * P0 - k], Xd[tt + sd + 2 * P0 - k], acc);
                }
            } else {
                float lsum = 0.f;
#pragma unroll
                for (int k = 0; k < W0; ++k) {
                    lsum = fmaf(Du[k * kTmaBox + tt], Xu[tt + k + su], lsum);
                    lsum = fmaf(Dd[k * kTmaBox + tt + sd + 2 * P0 - k], Xd[tt + sd + 2 * P0 - k], lsum);
                }
                acc += lsum;
            }
            if (q == nlines - 1 && r0 + tt < n) {
                t[r0 + tt] = acc;
                contrib += double(acc) * double(xr);
            }
        }
        __syncthreads();  // the stage has been read by every thread: refill it
        if (threadIdx.x == 0 && j + kTmaStages < njobs) issue(j + kTmaStages);
    }
    if (failed) {
        if (threadIdx.x == 0) {
            atomicExch(err, 1);
            // the copies this block issued and has not seen complete: jobs j .. min(j + stages, njobs) - 1
            for (int k = j; k < njobs && k < j + kTmaStages; ++k) mbarWait(&full[k % kTmaStages], unsigned(k / kTmaStages) & 1u);
        }
        return;
    }
    __shared__ double ws[kTmaThreads / 32];
    contrib = warpSumD(contrib);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = contrib;
    __syncthreads();
    if (threadIdx.x == 0) {
        double sum = 0.0;
        for (int w = 0; w < kTmaThreads / 32; ++w) sum += ws[w];
        part[blockIdx.x] = sum;
    }
}


}  // namespace

namespace launch {

int sdiaHalf(const int* p) { return halfCount(p); }

void sdiaBuild(const SdiaOp& A, const SdiaBand& B, const df32* band, float* d, cudaStream_t s) {
    if (A.n > 0) k_sdia_build<<<unsigned((A.ns + kB - 1) / kB), kB, 0, s>>>(A, B, band, d);
}

int sdiaReach(const SdiaOp& A) { return A.p[0] + A.m[0] * (A.p[1] + A.m[1] * A.p[2]); }

int sdiaPartials(const SdiaOp& A) {
    if (A.tmaps) return std::max(1, std::min((A.n + kTmaT - 1) / kTmaT, 152 * kTmaBlocksPerSm));
    if (A.group == kG) return std::max(1, std::min((A.n + kG * kBG - 1) / (kG * kBG), 152 * kG4BlocksPerSm));
    const int nb = (A.n + kB - 1) / kB;
    return std::max(1, std::min(nb, kMaxSpmvBlocks));
}

// the dynamic shared-memory limit of the TMA product's instantiation (set where the maps are made,
// before any stream capture)
template <int P0>
static cudaError_t tmaAttr() {
    return cudaFuncSetAttribute(k_sdia32_tma<P0>, cudaFuncAttributeMaxDynamicSharedMemorySize, TmaShape<P0>::SMEM);
}

template <int P0>
static void launchTma(const SdiaOp& A, float* t, double* part, const CgState* st, cudaStream_t s) {
    const CUtensorMap* maps = static_cast<const CUtensorMap*>(A.tmaps);
    k_sdia32_tma<P0><<<sdiaPartials(A), kTmaThreads, TmaShape<P0>::SMEM, s>>>(maps[0], maps[1], A, t, part, st,
                                                                               A.err);
}

// tensor maps of the half diagonals (2D: ns x nh floats, boxes of kTmaBox x (2 p0 + 1)) and of the
// vector x (1D: n floats, boxes of kTmaBox); zero fill outside the arrays. On failure *why says what
// refused them.
bool sdiaTensorMaps(const SdiaOp& A, const float* x, void* out2, std::string* why) {
    using Encode = PFN_cuTensorMapEncodeTiled_v12000;
    static Encode encode = nullptr;
    auto fail = [&](const std::string& w) {
        if (why) *why = w;
        return false;
    };
    if (!encode) {
        void* fn = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
            return fail(std::string("cuTensorMapEncodeTiled entry point: ") + cudaGetErrorString(e) + " query " +
                        std::to_string(int(q)));
        encode = reinterpret_cast<Encode>(fn);
    }
    if (A.p[0] < 1 || A.p[0] > 4 || A.ns % 4 != 0) return fail("shape outside the TMA product's range");
    if ((reinterpret_cast<uintptr_t>(A.d) & 15) || (reinterpret_cast<uintptr_t>(x) & 15))
        return fail("arrays not 16-byte aligned");
    CUtensorMap* maps = static_cast<CUtensorMap*>(out2);
    const cuuint64_t dimD[2] = {cuuint64_t(A.ns), cuuint64_t(A.nh)};
    const cuuint64_t strideD[1] = {cuuint64_t(A.ns) * 4};
    const cuuint32_t boxD[2] = {cuuint32_t(kTmaBox), cuuint32_t(2 * A.p[0] + 1)};
    const cuuint32_t one[2] = {1, 1};
    CUresult r = encode(&maps[0], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(A.d), dimD, strideD, boxD, one,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail("diagonal tensor map: CUresult " + std::to_string(int(r)));
    const cuuint64_t dimX[1] = {cuuint64_t(A.n)};
    const cuuint64_t strideX[1] = {cuuint64_t(A.ns) * 4};  // unused for rank 1
    const cuuint32_t boxX[1] = {cuuint32_t(kTmaBox)};
    r = encode(&maps[1], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 1, const_cast<float*>(x), dimX, strideX, boxX, one,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail("vector tensor map: CUresult " + std::to_string(int(r)));
    const cudaError_t ea = A.p[0] == 1 ? tmaAttr<1>() : A.p[0] == 2 ? tmaAttr<2>() : A.p[0] == 3 ? tmaAttr<3>() : tmaAttr<4>();
    if (ea != cudaSuccess) return fail(std::string("shared-memory attribute: ") + cudaGetErrorString(ea));
    return true;
}

void sdiaSpmv(const SdiaOp& A, const float* x, float* t, double* part, const CgState* st, cudaStream_t s) {
    if (A.tmaps) {
        switch (A.p[0]) {
            case 1: launchTma<1>(A, t, part, st, s); break;
            case 2: launchTma<2>(A, t, part, st, s); break;
            case 3: launchTma<3>(A, t, part, st, s); break;
            default: launchTma<4>(A, t, part, st, s); break;
        }
        return;
    }
    const int nb = sdiaPartials(A);
    if (A.group == kG) {
        switch (A.p[0]) {
            case 1: launchMaybePdl(k_sdia32_g4<1>, dim3(nb), dim3(kBG), s, A.pdl, A, x, t, part, st); break;
            case 2: launchMaybePdl(k_sdia32_g4<2>, dim3(nb), dim3(kBG), s, A.pdl, A, x, t, part, st); break;
            case 3: launchMaybePdl(k_sdia32_g4<3>, dim3(nb), dim3(kBG), s, A.pdl, A, x, t, part, st); break;
            default: launchMaybePdl(k_sdia32_g4<4>, dim3(nb), dim3(kBG), s, A.pdl, A, x, t, part, st); break;
        }
        return;
    }
    switch (A.p[0]) {
        case 1: k_sdia32_dot<1><<<nb, kB, 0, s>>>(A, x, t, part, st); break;
        case 2: k_sdia32_dot<2><<<nb, kB, 0, s>>>(A, x, t, part, st); break;
        case 3: k_sdia32_dot<3><<<nb, kB, 0, s>>>(A, x, t, part, st); break;
        default: k_sdia32_dot<4><<<nb, kB, 0, s>>>(A, x, t, part, st); break;
    }
}

}  // namespace launch
}  // namespace gsgpu

