// sm_103a assembly kernels: basis tables (K1), geometry map and coefficient fields (K2),
// sum-factorised stiffness / load contractions (K3) and the atomic-free CSR gather with the
// Dirichlet lift (K4). Thread -> item mapping only; the arithmetic lives in device_funcs.cuh.
#include <cstdlib>
#include <cstring>

#include "device_funcs.cuh"
#include "kernels.h"

namespace gsgpu {
namespace {

using launch::kBlock;

// K1: one lane per (direction, abscissa): the Cox-de Boor triangle runs in registers
__global__ void __launch_bounds__(kBlock) k_basis(const TabJob* __restrict__ jobs, long long njobs,
                                                  const double* __restrict__ knots, double* __restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= njobs) return;
    const TabJob j = jobs[i];
    double buf[32];
    dev::basis1d(knots + j.koff, j.p, j.span, j.u, buf);
    for (int r = 0; r < 2 * (j.p + 1); ++r) out[j.out + r] = buf[r];
}

// K1, warp-cooperative: the Cox-de Boor triangle of each abscissa by a group of kBasisGroup
// lanes, lane r holding N_r; level k forms N_0..N_k from the lane's own N_r and its neighbour's
// quotient N_{r-1} / (t_{r-1+s+1} - t_{..}) (a shuffle), so the triangle takes p steps of one
// division each instead of p(p+1)/2 on one lane, in registers (one lane per abscissa keeps the
// triangle in a local array). Every value is the same expression, with the same roundings fixed
// (dev::bMul, fma), as in basis1d: the same bits.
// Degrees above kBasisGroup - 1 (wider than the group) take basis1d on the group's first lane.
constexpr int kBasisGroup = 8;
__global__ void __launch_bounds__(kBlock) k_basis_warp(const TabJob* __restrict__ jobs, long long njobs,
                                                       const double* __restrict__ knots, double* __restrict__ out) {
    const long long g = ((long long)blockIdx.x * blockDim.x + threadIdx.x) / kBasisGroup;
    const int r = int(threadIdx.x % kBasisGroup);
    const bool valid = g < njobs;
    TabJob j{};
    if (valid) j = jobs[g];
    const int p = j.p;
    const int pw = p < kBasisGroup ? p : 0;  // the degree the group's shuffle triangle handles
    const double* t = knots + j.koff;
    const int s = j.span;
    const double u = j.u;
    double N = r == 0 ? 1.0 : 0.0, Nm1 = 0.0;
    for (int k = 1; k < kBasisGroup; ++k) {  // uniform trip count: every lane takes part in the shuffles
        const bool act = valid && k <= pw;
        if (act && k == pw) Nm1 = N;  // the degree p-1 values, for the derivatives
        double tmp = 0.0, tr = 0.0;
        if (act && r < k) {
            tr = t[s + 1 + r];
            tmp = N / (tr - t[s + 1 + r - k]);
        }
        const double prev = __shfl_up_sync(0xffffffffu, tmp, 1, kBasisGroup);
        if (act && r <= k) {
            const double saved = r >= 1 ? dev::bMul(u - t[s + r - k], prev) : 0.0;
            N = r < k ? fma(tr - u, tmp, saved) : saved;
        }
    }
    const double prevNm1 = __shfl_up_sync(0xffffffffu, Nm1, 1, kBasisGroup);
    if (!valid) return;
    if (p >= kBasisGroup) {
        if (r == 0) {
            double buf[32];
            dev::basis1d(knots + j.koff, j.p, j.span, j.u, buf);
            for (int q = 0; q < 2 * (j.p + 1); ++q) out[j.out + q] = buf[q];
        }
        return;
    }
    if (r > p) return;
    if (p == 0) {
        out[j.out] = 1.0;
        out[j.out + 1] = 0.0;
        return;
    }
    const int a = s - p;
    double d = 0.0;
    if (r >= 1) d += dev::bMul(double(p), prevNm1) / (t[a + r + p] - t[a + r]);
    if (r <= p - 1) d -= dev::bMul(double(p), Nm1) / (t[a + r + p + 1] - t[a + r + 1]);
    out[j.out + r] = N;
    out[j.out + p + 1 + r] = d;
}

template <typename T>
__global__ void __launch_bounds__(kBlock) k_pair(const PfJob* __restrict__ jobs, const BlkEnt* __restrict__ tab,
                                                 const double* __restrict__ basis, T* __restrict__ pf) {
    const BlkEnt be = tab[blockIdx.x];
    const PfJob j = jobs[be.patch];
    const long long item = be.base + threadIdx.x;
    if (item >= j.count) return;
    pf[j.pf + item] = dev::pairFactor<T>(basis + j.tab, j.p, j.q, j.E, item);
}

template <typename R>
__global__ void __launch_bounds__(kBlock) k_geo1(const DevPatch* __restrict__ P, const BlkEnt* __restrict__ tab,
                                                 const R* __restrict__ coefs, const R* __restrict__ gtab,
                                                 const int* __restrict__ ibuf, R* __restrict__ Y1) {
    const BlkEnt be = tab[blockIdx.x];
    const DevPatch& D = P[be.patch];
    const long long item = be.base + threadIdx.x;
    const long long work = D.dim == 3 ? (long long)D.dim * 2 * D.gn[2] * D.gn[1] * D.Q[0]
                                      : (long long)D.dim * 2 * D.gn[1] * D.Q[0];
    if (item >= work) return;
    Y1[D.y1_off + item] = work < (1LL << 31) ? dev::geoStage1<R, unsigned>(D, item, coefs, gtab, ibuf)
                                             : dev::geoStage1<R>(D, item, coefs, gtab, ibuf);
}

template <typename R>
__global__ void __launch_bounds__(kBlock) k_geo2(const DevPatch* __restrict__ P, const BlkEnt* __restrict__ tab,
                                                 const R* __restrict__ Y1, const R* __restrict__ gtab,
                                                 const int* __restrict__ ibuf, R* __restrict__ Y2) {
    const BlkEnt be = tab[blockIdx.x];
    const DevPatch& D = P[be.patch];
    const long long item = be.base + threadIdx.x;
    const long long work = (long long)D.dim * 3 * D.gn[2] * D.Q[1] * D.Q[0];
    if (item >= work) return;
    Y2[D.y2_off + item] = work < (1LL << 31) ? dev::geoStage2<R, unsigned>(D, item, Y1, gtab, ibuf)
                                             : dev::geoStage2<R>(D, item, Y1, gtab, ibuf);
}

__device__ __forceinline__ unsigned long long detKey(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b & 0x8000000000000000ULL) ? ~b : (b | 0x8000000000000000ULL);
}

// the mass field M = w |det J| at every quadrature point, into the load field's slot (FP64)
__global__ void __launch_bounds__(kBlock) k_mass_field(const DevPatch* __restrict__ P, const BlkEnt* __restrict__ tab,
                                                       const double* __restrict__ Y1, const double* __restrict__ Y2,
                                                       const double* __restrict__ gtab, const int* __restrict__ ibuf,
                                                       const double* __restrict__ wq, double* __restrict__ M) {
    const BlkEnt be = tab[blockIdx.x];
    const DevPatch& D = P[be.patch];
    const long long item = be.base + threadIdx.x;
    if (item >= D.nq) return;
    const int Q0 = D.Q[0], Q1 = D.Q[1];
    const int g0 = int(item % Q0);
    const long long r = item / Q0;
    const int g1 = int(r % Q1), g2 = int(r / Q1);
    double x[3], J[3][3];
    dev::pointMap<double>(D, item, Y1, Y2, gtab, ibuf, x, J);
    double w = wq[D.qoff[0] + g0] * wq[D.qoff[1] + g1];
    double det;
    if (D.dim == 3) {
        w *= wq[D.qoff[2] + g2];
        det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) + J[0][1] * (J[1][2] * J[2][0] - J[1][0] * J[2][2]) +
              J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    } else {
        det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    }
    M[D.lfield_off + item] = w * fabs(det);
}

// the double-float instance is held to 64 registers (4 blocks per SM; measured faster than the 78
// it takes unbounded), the FP64 one is left to the compiler; KW sizes the powers table of the
// Fourier coefficient (the problem's largest wave number, 4 or 8)
template <typename R>
constexpr int kPointBlocks = std::is_same<R, df32>::value ? 4 : 1;
template <typename R, int KW>
__global__ void __launch_bounds__(kBlock, kPointBlocks<R>) k_point(const DevPatch* __restrict__ P, const BlkEnt* __restrict__ tab,
                                                  const dev::FieldConst<R>* __restrict__ F, const R* __restrict__ Y1,
                                                  const R* __restrict__ Y2, const R* __restrict__ gtab,
                                                  const int* __restrict__ ibuf, const R* __restrict__ wq,
                                                  R* __restrict__ C, R* __restrict__ Lf,
                                                  unsigned long long* __restrict__ detkey) {
    __shared__ dev::FieldConst<R> sF;
    const BlkEnt be = tab[blockIdx.x];
    const DevPatch& D = P[be.patch];
    // stage the patch's coefficient parameters in shared memory (uniform across the block)
    {
        const int nw = int(sizeof(dev::FieldConst<R>) / sizeof(int));
        const int* src = reinterpret_cast<const int*>(F + D.field_id);
        int* dst = reinterpret_cast<int*>(&sF);
        for (int k = threadIdx.x; k < nw; k += blockDim.x) dst[k] = src[k];
    }
    __syncthreads();
    const long long item = be.base + threadIdx.x;
    unsigned long long key = ~0ULL;
    if (item < D.nq) key = detKey(dev::pointStep<R, KW>(D, sF, item, Y1, Y2, gtab, ibuf, wq, C, Lf));
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long other = __shfl_xor_sync(0xffffffffu, key, o);
        key = other < key ? other : key;
    }
    __shared__ unsigned long long wmin[kBlock / 32];
    if ((threadIdx.x & 31) == 0) wmin[threadIdx.x >> 5] = key;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m = wmin[0];
        for (int w = 1; w < kBlock / 32; ++w) m = wmin[w] < m ? wmin[w] : m;
        atomicMin(detkey, m);
    }
}

template <typename T, int KIND>
__global__ void __launch_bounds__(kBlock) k_contract(const DevPatch* __restrict__ P, const BlkEnt* __restrict__ tab,
                                                     const T* __restrict__ in, T* __restrict__ out,
                                                     const int* __restrict__ ibuf, const T* __restrict__ pf) {
    const BlkEnt be = tab[blockIdx.x];
    const DevPatch& D = P[be.patch];
    const long long item = be.base + threadIdx.x;
    if (item >= dev::stageWork<KIND>(D)) return;
    dev::contractItem<T, KIND>(D, item, in, out, ibuf, pf);
}

template <int KIND>
__global__ void __launch_bounds__(kBlock) k_contract_df(const DevPatch* __restrict__ P, const BlkEnt* __restrict__ tab,
                                                        const df32* __restrict__ in, df32* __restrict__ out,
                                                        const int* __restrict__ ibuf, const df32* __restrict__ pf) {
    const BlkEnt be = tab[blockIdx.x];
    const DevPatch& D = P[be.patch];
    const long long item = be.base + threadIdx.x;
    if (item >= dev::stageWork<KIND>(D)) return;
    dev::contractItemDF<KIND>(D, item, in, out, ibuf, pf);
}

// interior rows of simple axes (fixed support shape, unrolled); two CTAs per SM
template <int KIND, int DEG, int H0, int NH>
__global__ void __launch_bounds__(kBlock, 2) k_contract_row_df_int(const DevPatch* __restrict__ P,
                                                                   const BlkEnt* __restrict__ tab,
                                                                   const df32* __restrict__ in,
                                                                   df32* __restrict__ out,
                                                                   const df32* __restrict__ pf) {
    const BlkEnt be = tab[blockIdx.x];
    const DevPatch& D = P[be.patch];
    const long long item = be.base + threadIdx.x;
    if (item >= dev::stageInteriorWork<KIND>(D)) return;
    dev::contractRowDFInterior<KIND, DEG, H0, NH>(D, item, in, out, pf);
}

// 3D stage 1 (axis 0) interior rows, tiled (dev::stage31Tiles), outputs H0..H0+3: the block
// stages the pair factors of its elements and the coefficient fields of its lines that those
// outputs use in shared memory, laid out so that the 32 rows of a warp read consecutive words,
// then each thread forms the outputs of its row. The products and the Dot2 order per output are
// those of contractRowDFInterior<31>, so the results are the same bit for bit; what changes is
// where the operands come from (shared memory instead of strided L1 traffic).
template <int P, int H0>
__global__ void __launch_bounds__(dev::kTileLines * dev::kTileRows, 2)
    k_stage31_tile(const DevPatch* __restrict__ Pd, const BlkEnt* __restrict__ tab, const df32* __restrict__ in,
                   df32* __restrict__ out, const df32* __restrict__ pf) {
    using S = dev::Stage<31>;
    constexpr int P1 = P + 1, Q = P + 1, W = 2 * P + 1, LB = dev::kTileLines, RB = dev::kTileRows;
    constexpr int NE = dev::tileElems(P);
    constexpr int F0 = dev::tileField0(H0), NF = dev::tileNField(H0);
    constexpr int T0 = dev::tileTau0(H0), NTAU = dev::tileNTau(H0);
    extern __shared__ df32 smem[];
    df32* sPF = smem;
    df32* sX = smem + dev::tilePfCount(P, H0);
    const BlkEnt be = tab[blockIdx.x];
    const DevPatch& D = Pd[be.patch];
    const dev::StageGeom G = dev::stageGeom<31>(D);
    const int n = D.n[0], E = D.E[0], Qa = D.Q[0];
    const int m = n - 2 * P;
    const int nseg = (m + RB - 1) / RB;
    const long long tile = be.base / kBlock;
    const long long o0 = tile / nseg * LB;
    const int seg = int(tile % nseg);
    const int i0 = P + seg * RB;
    const int e0 = i0 - P;
    const int ne = min(NE, E - e0);
    const int nl = int(min((long long)LB, G.outer - o0));
    // pair factors of elements e0 .. e0+ne-1, types T0 .. T0+NTAU-1 (contiguous per type)
    const long long tstride = (long long)E * Q * P1 * P1;
    const df32* pfa = pf + D.pfoff[0] + T0 * tstride + (long long)e0 * Q * P1 * P1;
    const int per = ne * Q * P1 * P1;
    for (int idx = threadIdx.x; idx < NTAU * per; idx += blockDim.x) {
        const int tau = idx / per;
        const int j = idx - tau * per;
        int r = j;
        const int t = r % P1;
        r /= P1;
        const int si = r % P1;
        r /= P1;
        const int rr = r % Q;
        const int ee = r / Q;
        sPF[(((si * Q + rr) * P1 + t) * NTAU + tau) * NE + ee] = pfa[tau * tstride + j];
    }
    // fields F0 .. F0+NF-1 of the tile's lines at the points of those elements
    const int perl = ne * Q;
    for (int idx = threadIdx.x; idx < NF * nl * perl; idx += blockDim.x) {
        const int f = idx / (nl * perl);
        int r = idx - f * nl * perl;
        const int l = r / perl;
        r -= l * perl;
        const int rr = r % Q;
        const int ee = r / Q;
        sX[((f * Q + rr) * LB + l) * NE + ee] =
            in[G.in_base + (F0 + f) * G.in_fs + (o0 + l) * Qa + (long long)e0 * Q + r];
    }
    __syncthreads();
    const int l = threadIdx.x / RB, rw = threadIdx.x % RB;
    const int i = i0 + rw;
    if (l >= nl || i >= n - P) return;
    const df32* sx = sX + l * NE + rw;
    const df32* spf = sPF + rw;
    Dot2 acc[W][4];
#pragma unroll
    for (int k = 0; k <= P; ++k) {
#pragma unroll
        for (int rr = 0; rr < Q; ++rr) {
            df32 x[NF];
#pragma unroll
            for (int f = 0; f < NF; ++f) x[f] = sx[(f * Q + rr) * LB * NE + k];
            const df32* prow = spf + ((P - k) * Q + rr) * P1 * NTAU * NE + k;
#pragma unroll
            for (int t = 0; t < P1; ++t) {
#pragma unroll
                for (int kk = 0; kk < S::NT; ++kk) {
                    const dev::Term tm = S::term(kk);
                    if (tm.h >= H0 && tm.h < H0 + 4)
                        acc[k + t][tm.h - H0].mac(prow[(t * NTAU + tm.tau - T0) * NE], x[tm.f - F0]);
                }
            }
        }
    }
    df32* op = out + G.out_base + ((o0 + l) * n + i) * W;
#pragma unroll
    for (int w = 0; w < W; ++w)
#pragma unroll
        for (int h = 0; h < 4; ++h) op[(H0 + h) * G.out_fs + w] = acc[w][h].result();
}

// 8-byte asynchronous copy global -> shared (no register round trip; completes with the group)
__device__ __forceinline__ void cpAsync8(void* dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(static_cast<unsigned>(__cvta_generic_to_shared(dst))),
                 "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cpAsyncCommit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cpAsyncWait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// k_stage31_tile as a persistent kernel: each block walks the tiles blockIdx.x, blockIdx.x + G, ...
// (G = gridDim.x, a multiple of the row segments per line of a single patch, so that a block's
// tiles share their elements and pair factors, which it stages once), and double-buffers the
// coefficient fields: while it forms the outputs of one tile, the fields of its next tile arrive
// by asynchronous copies into the other buffer. Same products and Dot2 order per output as
// k_stage31_tile (the same bits); the staging overlaps the arithmetic instead of preceding it.
template <int P, int H0>
__global__ void __launch_bounds__(dev::kTileLines * dev::kTileRows, 2)
    k_stage31_tilep(const DevPatch* __restrict__ Pd, const BlkEnt* __restrict__ tab, long long ntiles,
                    const df32* __restrict__ in, df32* __restrict__ out, const df32* __restrict__ pf) {
    using S = dev::Stage<31>;
    constexpr int P1 = P + 1, Q = P + 1, W = 2 * P + 1, LB = dev::kTileLines, RB = dev::kTileRows;
    constexpr int NE = dev::tileElems(P);
    constexpr int F0 = dev::tileField0(H0), NF = dev::tileNField(H0);
    constexpr int T0 = dev::tileTau0(H0), NTAU = dev::tileNTau(H0);
    constexpr int NX = dev::tileFieldCount(P, H0);
    extern __shared__ df32 smem[];
    df32* sPF = smem;
    df32* sXb = smem + dev::tilePfCount(P, H0);  // two field buffers of NX values
    struct TileInfo {
        int patch, seg, i0, e0, ne, nl, n;
        long long o0;
    };
    auto info = [&](long long j) {
        const BlkEnt be = tab[j];
        const DevPatch& D = Pd[be.patch];
        const int n = D.n[0], E = D.E[0];
        const int m = n - 2 * P;
        const int nseg = (m + RB - 1) / RB;
        const long long tile = be.base / kBlock;
        TileInfo t;
        t.patch = be.patch;
        t.n = n;
        t.o0 = tile / nseg * LB;
        t.seg = int(tile % nseg);
        t.i0 = P + t.seg * RB;
        t.e0 = t.i0 - P;
        t.ne = min(NE, E - t.e0);
        t.nl = int(min((long long)LB, dev::stageGeom<31>(D).outer - t.o0));
        return t;
    };
    auto issueFields = [&](const TileInfo& t, df32* sX) {
        const DevPatch& D = Pd[t.patch];
        const dev::StageGeom G = dev::stageGeom<31>(D);
        const int Qa = D.Q[0];
        const int perl = t.ne * Q;
        for (int idx = threadIdx.x; idx < NF * t.nl * perl; idx += blockDim.x) {
            const int f = idx / (t.nl * perl);
            int r = idx - f * t.nl * perl;
            const int l = r / perl;
            r -= l * perl;
            const int rr = r % Q;
            const int ee = r / Q;
            cpAsync8(&sX[((f * Q + rr) * LB + l) * NE + ee],
                     &in[G.in_base + (F0 + f) * G.in_fs + (t.o0 + l) * Qa + (long long)t.e0 * Q + r]);
        }
    };
    const long long stride = gridDim.x;
    long long j = blockIdx.x;
    if (j >= ntiles) return;
    TileInfo cur = info(j);
    issueFields(cur, sXb);
    cpAsyncCommit();
    int pfPatch = -1, pfSeg = -1;
    for (int it = 0; j < ntiles; j += stride, ++it) {
        df32* sX = sXb + (it & 1) * NX;
        // the next tile's fields into the other buffer (every thread passed the previous tile's
        // closing barrier, so nobody reads that buffer any more)
        TileInfo nxt{};
        const bool more = j + stride < ntiles;
        if (more) {
            nxt = info(j + stride);
            issueFields(nxt, sXb + ((it + 1) & 1) * NX);
        }
        cpAsyncCommit();
        if (cur.patch != pfPatch || cur.seg != pfSeg) {
            // pair factors of elements e0 .. e0+ne-1, types T0 .. T0+NTAU-1
            const DevPatch& D = Pd[cur.patch];
            const int E = D.E[0];
            const long long tstride = (long long)E * Q * P1 * P1;
            const df32* pfa = pf + D.pfoff[0] + T0 * tstride + (long long)cur.e0 * Q * P1 * P1;
            const int per = cur.ne * Q * P1 * P1;
            for (int idx = threadIdx.x; idx < NTAU * per; idx += blockDim.x) {
                const int tau = idx / per;
                const int jj = idx - tau * per;
                int r = jj;
                const int t = r % P1;
                r /= P1;
                const int si = r % P1;
                r /= P1;
                const int rr = r % Q;
                const int ee = r / Q;
                sPF[(((si * Q + rr) * P1 + t) * NTAU + tau) * NE + ee] = pfa[tau * tstride + jj];
            }
            pfPatch = cur.patch;
            pfSeg = cur.seg;
        }
        cpAsyncWait<1>();  // this thread's copies of the current tile have landed
        __syncthreads();   // everyone's, and the pair factors
        const int l = threadIdx.x / RB, rw = threadIdx.x % RB;
        const int i = cur.i0 + rw;
        if (l < cur.nl && i < cur.n - P) {
            const df32* sx = sX + l * NE + rw;
            const df32* spf = sPF + rw;
            Dot2 acc[W][4];
#pragma unroll
            for (int k = 0; k <= P; ++k) {
#pragma unroll
                for (int rr = 0; rr < Q; ++rr) {
                    df32 x[NF];
#pragma unroll
                    for (int f = 0; f < NF; ++f) x[f] = sx[(f * Q + rr) * LB * NE + k];
                    const df32* prow = spf + ((P - k) * Q + rr) * P1 * NTAU * NE + k;
#pragma unroll
                    for (int t = 0; t < P1; ++t) {
#pragma unroll
                        for (int kk = 0; kk < S::NT; ++kk) {
                            const dev::Term tm = S::term(kk);
                            if (tm.h >= H0 && tm.h < H0 + 4)
                                acc[k + t][tm.h - H0].mac(prow[(t * NTAU + tm.tau - T0) * NE], x[tm.f - F0]);
                        }
                    }
                }
            }
            const DevPatch& D = Pd[cur.patch];
            const dev::StageGeom G = dev::stageGeom<31>(D);
            df32* op = out + G.out_base + ((cur.o0 + l) * cur.n + i) * W;
#pragma unroll
            for (int w = 0; w < W; ++w)
#pragma unroll
                for (int h = 0; h < 4; ++h) op[(H0 + h) * G.out_fs + w] = acc[w][h].result();
        }
        __syncthreads();  // the current buffer (and the pair factors) are free again
        if (more) cur = nxt;
    }
    cpAsyncWait<0>();
}

// the remaining (boundary) rows with the general element loop
template <int KIND, int DEG, int H0, int NH>
__global__ void __launch_bounds__(kBlock) k_contract_row_df_bnd(const DevPatch* __restrict__ P,
                                                                const BlkEnt* __restrict__ tab,
                                                                const df32* __restrict__ in, df32* __restrict__ out,
                                                                const int* __restrict__ ibuf,
                                                                const df32* __restrict__ pf) {
    const BlkEnt be = tab[blockIdx.x];
    const DevPatch& D = P[be.patch];
    const long long bitem = be.base + threadIdx.x;
    if (bitem >= dev::stageBoundaryWork<KIND>(D)) return;
    const long long item = dev::boundaryItem<KIND>(D, bitem);
    if (D.q[dev::Stage<KIND>::AX] == DEG + 1)
        dev::contractRowDF<KIND, DEG, H0, NH, DEG + 1>(D, item, in, out, ibuf, pf);
    else
        dev::contractRowDF<KIND, DEG, H0, NH, 0>(D, item, in, out, ibuf, pf);
}

template <int KIND, typename Tin>
__global__ void __launch_bounds__(kBlock) k_load(const DevPatch* __restrict__ P, const BlkEnt* __restrict__ tab,
                                                 const Tin* __restrict__ in, double* __restrict__ out,
                                                 const double* __restrict__ basis, const int* __restrict__ ibuf) {
    const BlkEnt be = tab[blockIdx.x];
    const DevPatch& D = P[be.patch];
    const long long item = be.base + threadIdx.x;
    if (item >= dev::loadWork<KIND>(D)) return;
    out[dev::loadGeom<KIND>(D).out_base + item] = dev::loadItem<KIND, Tin>(D, item, in, basis, ibuf);
}

template <int KIND>
__global__ void __launch_bounds__(kBlock) k_load_df(const DevPatch* __restrict__ P, const BlkEnt* __restrict__ tab,
                                                    const df32* __restrict__ in, double* __restrict__ out,
                                                    const df32* __restrict__ basis, const int* __restrict__ ibuf) {
    const BlkEnt be = tab[blockIdx.x];
    const DevPatch& D = P[be.patch];
    const long long item = be.base + threadIdx.x;
    if (item >= dev::loadWork<KIND>(D)) return;
    out[dev::loadGeom<KIND>(D).out_base + item] = dev::loadItemDF<KIND>(D, item, in, basis, ibuf);
}

template <typename T>
__global__ void __launch_bounds__(kBlock) k_gather(long long nnz, const uint32_t* __restrict__ src,
                                                   const T* __restrict__ band, const uint32_t* __restrict__ ovf_ptr,
                                                   const uint32_t* __restrict__ ovf_idx, T* __restrict__ val) {
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nnz) return;
    val[s] = dev::gatherSlot<T>(src[s], band, ovf_ptr, ovf_idx);
}

__global__ void __launch_bounds__(kBlock) k_gather_df(long long nnz, const uint32_t* __restrict__ src,
                                                      const df32* __restrict__ band, const uint32_t* __restrict__ ovf_ptr,
                                                      const uint32_t* __restrict__ ovf_idx, float* __restrict__ hi,
                                                      float* __restrict__ lo) {
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nnz) return;
    const df32 v = dev::gatherSlotDF(src[s], band, ovf_ptr, ovf_idx);
    hi[s] = v.hi;
    lo[s] = v.lo;
}

__global__ void __launch_bounds__(kBlock) k_to_df(long long n, const double* __restrict__ in, df32* __restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = df32(in[i]);
}

// the FP32 rounding of double-float values (hi + lo rounded to nearest)
__global__ void __launch_bounds__(kBlock) k_df_to_f32(long long n, const df32* __restrict__ in, float* __restrict__ out) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = __fadd_rn(in[i].hi, in[i].lo);
}

template <typename TB>
__global__ void __launch_bounds__(kBlock) k_rhs(int n, const double* __restrict__ lvec, const uint32_t* __restrict__ lptr,
                                                const uint32_t* __restrict__ lidx, const TB* __restrict__ band,
                                                const uint32_t* __restrict__ fptr, const uint32_t* __restrict__ fband,
                                                const uint32_t* __restrict__ fbidx, const double* __restrict__ ddof,
                                                double* __restrict__ rhs) {
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= n) return;
    rhs[I] = dev::rhsRow<TB>(I, lvec, lptr, lidx, band, fptr, fband, fbidx, ddof);
}

__global__ void __launch_bounds__(kBlock) k_coef_soa(const DevPatch* __restrict__ P, const BlkEnt* __restrict__ tab,
                                                     const double* __restrict__ raw, double* __restrict__ soa) {
    const BlkEnt be = tab[blockIdx.x];
    const DevPatch& D = P[be.patch];
    const long long item = be.base + threadIdx.x;
    if (item >= D.ngeo * D.dim) return;
    const long long gi = item / D.dim;
    const int m = int(item % D.dim);
    soa[D.coef_off + m * D.ngeo + gi] = raw[D.coef_off + item];
}

inline unsigned grid1(long long n) { return unsigned((n + kBlock - 1) / kBlock); }

}  // namespace

namespace launch {

void basisTables(const TabJob* jobs, long long njobs, const double* knots, double* out, cudaStream_t s) {
    if (njobs <= 0) return;
    if (std::getenv("GSGPU_BASIS_LANE")) {  // one lane per abscissa (the same values)
        k_basis<<<grid1(njobs), kBlock, 0, s>>>(jobs, njobs, knots, out);
        return;
    }
    k_basis_warp<<<grid1(njobs * kBasisGroup), kBlock, 0, s>>>(jobs, njobs, knots, out);
}
template <typename T>
void pairFactors(const PfJob* jobs, const BlkEnt* tab, long long nblk, const double* basis, T* pf, cudaStream_t s) {
    if (nblk > 0) k_pair<T><<<unsigned(nblk), kBlock, 0, s>>>(jobs, tab, basis, pf);
}
template void pairFactors<double>(const PfJob*, const BlkEnt*, long long, const double*, double*, cudaStream_t);
template void pairFactors<df32>(const PfJob*, const BlkEnt*, long long, const double*, df32*, cudaStream_t);
template void pairFactors<float>(const PfJob*, const BlkEnt*, long long, const double*, float*, cudaStream_t);

template <typename R>
void geoStage1(const DevPatch* P, const BlkEnt* tab, long long nblk, const R* coefs, const R* gtab, const int* ibuf,
               R* Y1, cudaStream_t s) {
    if (nblk > 0) k_geo1<R><<<unsigned(nblk), kBlock, 0, s>>>(P, tab, coefs, gtab, ibuf, Y1);
}
template <typename R>
void geoStage2(const DevPatch* P, const BlkEnt* tab, long long nblk, const R* Y1, const R* gtab, const int* ibuf,
               R* Y2, cudaStream_t s) {
    if (nblk > 0) k_geo2<R><<<unsigned(nblk), kBlock, 0, s>>>(P, tab, Y1, gtab, ibuf, Y2);
}
template <typename R>
void pointStep(const DevPatch* P, const BlkEnt* tab, long long nblk, const dev::FieldConst<R>* F, const R* Y1,
               const R* Y2, const R* gtab, const int* ibuf, const R* wq, R* C, R* Lf, unsigned long long* detkey,
               int kmax, cudaStream_t s) {
    if (nblk <= 0) return;
    if (kmax <= 4) k_point<R, 4><<<unsigned(nblk), kBlock, 0, s>>>(P, tab, F, Y1, Y2, gtab, ibuf, wq, C, Lf, detkey);
    else k_point<R, dev::kMaxKappaWave><<<unsigned(nblk), kBlock, 0, s>>>(P, tab, F, Y1, Y2, gtab, ibuf, wq, C, Lf, detkey);
}
#define INST_GEO(R)                                                                                                \
    template void geoStage1<R>(const DevPatch*, const BlkEnt*, long long, const R*, const R*, const int*, R*,       \
                               cudaStream_t);                                                                      \
    template void geoStage2<R>(const DevPatch*, const BlkEnt*, long long, const R*, const R*, const int*, R*,       \
                               cudaStream_t);                                                                      \
    template void pointStep<R>(const DevPatch*, const BlkEnt*, long long, const dev::FieldConst<R>*, const R*,      \
                               const R*, const R*, const int*, const R*, R*, R*, unsigned long long*, int,          \
                               cudaStream_t);
INST_GEO(double)
INST_GEO(df32)

template <int KIND>
void contractDF(const DevPatch* P, const BlkEnt* tab, long long nblk, const df32* in, df32* out, const int* ibuf,
                const df32* pf, cudaStream_t s) {
    if (nblk > 0) k_contract_df<KIND><<<unsigned(nblk), kBlock, 0, s>>>(P, tab, in, out, ibuf, pf);
}
template void contractDF<31>(const DevPatch*, const BlkEnt*, long long, const df32*, df32*, const int*, const df32*, cudaStream_t);
template void contractDF<32>(const DevPatch*, const BlkEnt*, long long, const df32*, df32*, const int*, const df32*, cudaStream_t);
template void contractDF<33>(const DevPatch*, const BlkEnt*, long long, const df32*, df32*, const int*, const df32*, cudaStream_t);
template void contractDF<21>(const DevPatch*, const BlkEnt*, long long, const df32*, df32*, const int*, const df32*, cudaStream_t);
template void contractDF<22>(const DevPatch*, const BlkEnt*, long long, const df32*, df32*, const int*, const df32*, cudaStream_t);

template <int KIND, int H0, int NH>
void contractRowDF(int P, const DevPatch* Pd, const BlkEnt* tabInt, long long nInt, const BlkEnt* tabBnd,
                   long long nBnd, const df32* in, df32* out, const int* ibuf, const df32* pf, cudaStream_t s) {
#define ROW_CASE(DEG)                                                                                              \
    case DEG:                                                                                                      \
        if (nInt > 0) k_contract_row_df_int<KIND, DEG, H0, NH><<<unsigned(nInt), kBlock, 0, s>>>(Pd, tabInt, in, out, pf); \
        if (nBnd > 0) k_contract_row_df_bnd<KIND, DEG, H0, NH><<<unsigned(nBnd), kBlock, 0, s>>>(Pd, tabBnd, in, out, ibuf, pf); \
        break;
    switch (P) {
        ROW_CASE(1)
        ROW_CASE(2)
        ROW_CASE(3)
        ROW_CASE(4)
        default: break;
    }
#undef ROW_CASE
}
template <int P, int H0>
void stage31TileLaunch(const DevPatch* Pd, const BlkEnt* tab, long long ntiles, const df32* in, df32* out,
                       const df32* pf, int nseg, cudaStream_t s) {
    constexpr int threads = dev::kTileLines * dev::kTileRows;
    if (nseg > 0 && !std::getenv("GSGPU_TILE31_ONESHOT")) {
        // persistent: two blocks per SM, the grid a multiple of the row segments per line
        constexpr size_t bytes = size_t(dev::tilePfCount(P, H0) + 2 * dev::tileFieldCount(P, H0)) * sizeof(df32);
        cudaFuncSetAttribute(k_stage31_tilep<P, H0>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
        long long g = 2 * 152;
        g = g / nseg * nseg;
        if (g < nseg) g = nseg;
        if (g > ntiles) g = ntiles;
        k_stage31_tilep<P, H0><<<unsigned(g), threads, bytes, s>>>(Pd, tab, ntiles, in, out, pf);
        return;
    }
    constexpr size_t bytes = size_t(dev::tilePfCount(P, H0) + dev::tileFieldCount(P, H0)) * sizeof(df32);
    // a failure here shows as the launch error the caller checks
    cudaFuncSetAttribute(k_stage31_tile<P, H0>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
    k_stage31_tile<P, H0><<<unsigned(ntiles), threads, bytes, s>>>(Pd, tab, in, out, pf);
}

void stage31Tile(int P, const DevPatch* Pd, const BlkEnt* tab, long long ntiles, const df32* in, df32* out,
                 const df32* pf, int nseg, cudaStream_t s) {
    if (ntiles <= 0) return;
    if (P == 2) {
        stage31TileLaunch<2, 0>(Pd, tab, ntiles, in, out, pf, nseg, s);
        stage31TileLaunch<2, 4>(Pd, tab, ntiles, in, out, pf, nseg, s);
    } else if (P == 3) {
        stage31TileLaunch<3, 0>(Pd, tab, ntiles, in, out, pf, nseg, s);
        stage31TileLaunch<3, 4>(Pd, tab, ntiles, in, out, pf, nseg, s);
    }
}

#define INST_ROW(K, H0, NH)                                                                                      \
    template void contractRowDF<K, H0, NH>(int, const DevPatch*, const BlkEnt*, long long, const BlkEnt*, long long, \
                                           const df32*, df32*, const int*, const df32*, cudaStream_t);
INST_ROW(31, 0, 4)
INST_ROW(31, 4, 4)
INST_ROW(32, 0, 4)
INST_ROW(31, 0, 2)
INST_ROW(31, 2, 2)
INST_ROW(31, 4, 2)
INST_ROW(31, 6, 2)
INST_ROW(32, 0, 2)
INST_ROW(32, 2, 2)
INST_ROW(33, 0, 1)
INST_ROW(21, 0, 4)
INST_ROW(22, 0, 1)

void gatherCsrDF(long long nnz, const uint32_t* src, const df32* band, const uint32_t* ovf_ptr, const uint32_t* ovf_idx,
                 float* hi, float* lo, cudaStream_t s) {
    if (nnz > 0) k_gather_df<<<grid1(nnz), kBlock, 0, s>>>(nnz, src, band, ovf_ptr, ovf_idx, hi, lo);
}
void toDF(long long n, const double* in, df32* out, cudaStream_t s) {
    if (n > 0) k_to_df<<<grid1(n), kBlock, 0, s>>>(n, in, out);
}

void dfToFloat(long long n, const df32* in, float* out, cudaStream_t s) {
    if (n > 0) k_df_to_f32<<<grid1(n), kBlock, 0, s>>>(n, in, out);
}

template <typename T, int KIND>
void contract(const DevPatch* P, const BlkEnt* tab, long long nblk, const T* in, T* out, const int* ibuf, const T* pf,
              cudaStream_t s) {
    if (nblk > 0) k_contract<T, KIND><<<unsigned(nblk), kBlock, 0, s>>>(P, tab, in, out, ibuf, pf);
}
#define INST_CONTRACT(T, K) \
    template void contract<T, K>(const DevPatch*, const BlkEnt*, long long, const T*, T*, const int*, const T*, cudaStream_t);
INST_CONTRACT(double, 41)
INST_CONTRACT(double, 42)
INST_CONTRACT(double, 43)
INST_CONTRACT(double, 51)
INST_CONTRACT(double, 52)
INST_CONTRACT(double, 31)
INST_CONTRACT(double, 32)
INST_CONTRACT(double, 33)
INST_CONTRACT(double, 21)
INST_CONTRACT(double, 22)
// FP32: the coarse operators of the FP32 multigrid cycle
INST_CONTRACT(float, 31)
INST_CONTRACT(float, 32)
INST_CONTRACT(float, 33)
INST_CONTRACT(float, 21)
INST_CONTRACT(float, 22)

template <int KIND, typename Tin>
void loadContract(const DevPatch* P, const BlkEnt* tab, long long nblk, const Tin* in, double* out,
                  const double* basis, const int* ibuf, cudaStream_t s) {
    if (nblk > 0) k_load<KIND, Tin><<<unsigned(nblk), kBlock, 0, s>>>(P, tab, in, out, basis, ibuf);
}
#define INST_LOAD(K, Tin) \
    template void loadContract<K, Tin>(const DevPatch*, const BlkEnt*, long long, const Tin*, double*, const double*, const int*, cudaStream_t);
INST_LOAD(31, double)
INST_LOAD(32, double)
INST_LOAD(33, double)
INST_LOAD(21, double)
INST_LOAD(22, double)

template <int KIND>
void loadContractDF(const DevPatch* P, const BlkEnt* tab, long long nblk, const df32* in, double* out,
                    const df32* basis, const int* ibuf, cudaStream_t s) {
    if (nblk > 0) k_load_df<KIND><<<unsigned(nblk), kBlock, 0, s>>>(P, tab, in, out, basis, ibuf);
}
template void loadContractDF<31>(const DevPatch*, const BlkEnt*, long long, const df32*, double*, const df32*, const int*,
                                 cudaStream_t);
template void loadContractDF<21>(const DevPatch*, const BlkEnt*, long long, const df32*, double*, const df32*, const int*,
                                 cudaStream_t);

template <typename T>
void gatherCsr(long long nnz, const uint32_t* src, const T* band, const uint32_t* ovf_ptr, const uint32_t* ovf_idx,
               T* val, cudaStream_t s) {
    if (nnz > 0) k_gather<T><<<grid1(nnz), kBlock, 0, s>>>(nnz, src, band, ovf_ptr, ovf_idx, val);
}
template void gatherCsr<double>(long long, const uint32_t*, const double*, const uint32_t*, const uint32_t*, double*, cudaStream_t);
template void gatherCsr<float>(long long, const uint32_t*, const float*, const uint32_t*, const uint32_t*, float*, cudaStream_t);

template <typename TB>
void rhsRows(int n, const double* lvec, const uint32_t* lptr, const uint32_t* lidx, const TB* band,
             const uint32_t* fptr, const uint32_t* fband, const uint32_t* fbidx, const double* ddof, double* rhs,
             cudaStream_t s) {
    if (n > 0) k_rhs<TB><<<grid1(n), kBlock, 0, s>>>(n, lvec, lptr, lidx, band, fptr, fband, fbidx, ddof, rhs);
}
template void rhsRows<double>(int, const double*, const uint32_t*, const uint32_t*, const double*, const uint32_t*,
                              const uint32_t*, const uint32_t*, const double*, double*, cudaStream_t);
template void rhsRows<df32>(int, const double*, const uint32_t*, const uint32_t*, const df32*, const uint32_t*,
                            const uint32_t*, const uint32_t*, const double*, double*, cudaStream_t);

void massField(const DevPatch* P, const BlkEnt* tab, long long nblk, const double* Y1, const double* Y2,
               const double* gtab, const int* ibuf, const double* wq, double* M, cudaStream_t s) {
    if (nblk > 0) k_mass_field<<<unsigned(nblk), kBlock, 0, s>>>(P, tab, Y1, Y2, gtab, ibuf, wq, M);
}

void coefsToSoa(const DevPatch* P, const BlkEnt* tab, long long nblk, const double* raw, double* soa, cudaStream_t s) {
    if (nblk > 0) k_coef_soa<<<unsigned(nblk), kBlock, 0, s>>>(P, tab, raw, soa);
}

double detKeyDecode(unsigned long long key) {
    unsigned long long b = (key & 0x8000000000000000ULL) ? (key & ~0x8000000000000000ULL) : ~key;
    double v;
    std::memcpy(&v, &b, sizeof(v));
    return v;
}

}  // namespace launch
}  // namespace gsgpu
