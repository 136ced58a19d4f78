// Sparsity pattern and gather maps of a problem without interfaces, built on the device from the
// host's row plan (plan.h RowPlan): the same entries, in the same order, as the host builder's
// single-patch path (gsSparseSystem's symbolic pattern for single patches and batches of
// independent patches, src/gsAssembler/gsSparseSystem.h:327-370), without materialising the
// non-zeros on the host. One thread per row walks the row's neighbour box (z, y, x ascending):
// a first pass counts free and eliminated neighbours, a prefix scan gives the row pointers, a
// second pass writes columns, band sources, Dirichlet-lift entries and the diagonal slot.
#include "kernels.h"

namespace gsgpu {
namespace {

using launch::kBlock;
constexpr int kScanBlock = 1024;

struct RowBox {
    int c[3], lo[3], hi[3];
};

__device__ __forceinline__ RowBox rowBox(const DevPatch& D, const launch::RowPlanDev& R, int pi, int loc) {
    RowBox b;
    int r = loc;
    for (int a = 0; a < 3; ++a) {
        if (a < D.dim) {
            b.c[a] = r % D.n[a];
            r /= D.n[a];
            const int* rng = R.rng + R.rngOff[pi * 3 + a];
            b.lo[a] = rng[b.c[a]];
            b.hi[a] = rng[D.n[a] + b.c[a]];
        } else {
            b.c[a] = b.lo[a] = b.hi[a] = 0;
        }
    }
    return b;
}

__global__ void __launch_bounds__(kBlock) k_pat_count(const DevPatch* __restrict__ P, launch::RowPlanDev R,
                                                      long long* __restrict__ nslot, long long* __restrict__ nlift) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row > R.n) return;
    if (row == R.n) {  // the leading zero of the exclusive scans
        nslot[0] = 0;
        nlift[0] = 0;
        return;
    }
    const int pi = R.rowPatch[row];
    const DevPatch& D = P[pi];
    const RowBox b = rowBox(D, R, pi, R.rowLoc[row]);
    const int* idx = R.index + R.poff[pi];
    long long ns = 0, nl = 0;
    for (int z = b.lo[2]; z <= b.hi[2]; ++z)
        for (int y = b.lo[1]; y <= b.hi[1]; ++y)
            for (int x = b.lo[0]; x <= b.hi[0]; ++x) {
                const int lj = x + D.n[0] * (y + (D.dim == 3 ? D.n[1] * z : 0));
                if (idx[lj] < R.nfree) ++ns;
                else ++nl;
            }
    nslot[row + 1] = ns;
    nlift[row + 1] = nl;
}

// inclusive scan of kScanBlock-element chunks; chunk totals to sums
__global__ void __launch_bounds__(kScanBlock) k_scan_chunks(long long* __restrict__ a, long long n,
                                                           long long* __restrict__ sums) {
    __shared__ long long ws[kScanBlock / 32];
    const long long i = (long long)blockIdx.x * kScanBlock + threadIdx.x;
    long long v = i < n ? a[i] : 0;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const long long u = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += u;
    }
    if (lane == 31) ws[w] = v;
    __syncthreads();
    if (w == 0) {
        long long t = ws[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const long long u = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += u;
        }
        ws[lane] = t;
    }
    __syncthreads();
    if (w > 0) v += ws[w - 1];
    if (i < n) a[i] = v;
    if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = v;
}

// exclusive scan of the chunk totals by one block (sequential over groups of kScanBlock)
__global__ void __launch_bounds__(kScanBlock) k_scan_sums(long long* __restrict__ sums, long long nb) {
    __shared__ long long ws[kScanBlock / 32];
    __shared__ long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (long long base = 0; base < nb; base += kScanBlock) {
        const long long i = base + threadIdx.x;
        const long long orig = i < nb ? sums[i] : 0;
        long long v = orig;
        for (int o = 1; o < 32; o <<= 1) {
            const long long u = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += u;
        }
        if (lane == 31) ws[w] = v;
        __syncthreads();
        if (w == 0) {
            long long t = ws[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const long long u = __shfl_up_sync(0xffffffffu, t, o);
                if (lane >= o) t += u;
            }
            ws[lane] = t;
        }
        __syncthreads();
        if (w > 0) v += ws[w - 1];
        if (i < nb) sums[i] = carry + v - orig;  // exclusive
        __syncthreads();
        if (threadIdx.x == kScanBlock - 1) carry += v;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kBlock) k_scan_add(long long* __restrict__ a, long long n,
                                                     const long long* __restrict__ sums) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] += sums[i / kScanBlock];
}

// columns, band sources, lift entries, diagonal slot and load-vector source of each row; flags a
// row whose columns do not ascend (bad) and tracks the largest |column - row|
__global__ void __launch_bounds__(kBlock) k_pat_fill(const DevPatch* __restrict__ P, launch::RowPlanDev R,
                                                     const long long* __restrict__ nslot,
                                                     const long long* __restrict__ nlift, int* __restrict__ col,
                                                     uint32_t* __restrict__ src, uint32_t* __restrict__ fband,
                                                     uint32_t* __restrict__ fbidx, int* __restrict__ diag,
                                                     uint32_t* __restrict__ lidx, int* __restrict__ flags) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= R.n) return;
    const int pi = R.rowPatch[row];
    const DevPatch& D = P[pi];
    const int loc = R.rowLoc[row];
    const RowBox b = rowBox(D, R, pi, loc);
    const int* idx = R.index + R.poff[pi];
    const long long n0W = (long long)D.n[0] * D.W[0], n1W = (long long)D.n[1] * D.W[1];
    long long s = nslot[row], f = nlift[row];
    int prev = -1, dg = -1, far = 0;
    bool ordered = true;
    for (int z = b.lo[2]; z <= b.hi[2]; ++z)
        for (int y = b.lo[1]; y <= b.hi[1]; ++y)
            for (int x = b.lo[0]; x <= b.hi[0]; ++x) {
                const int lj = x + D.n[0] * (y + (D.dim == 3 ? D.n[1] * z : 0));
                const int J = idx[lj];
                long long bi = (long long)b.c[0] * D.W[0] + (x - b.c[0] + D.p[0]);
                bi += ((long long)b.c[1] * D.W[1] + (y - b.c[1] + D.p[1])) * n0W;
                if (D.dim == 3) bi += ((long long)b.c[2] * D.W[2] + (z - b.c[2] + D.p[2])) * n0W * n1W;
                bi += D.band_off;
                if (J < R.nfree) {
                    ordered = ordered && J > prev;
                    prev = J;
                    if (J == row) dg = int(s);
                    const int off = J - row;
                    far = max(far, off < 0 ? -off : off);
                    col[s] = J;
                    src[s] = uint32_t(bi);
                    ++s;
                } else {
                    fband[f] = uint32_t(bi);
                    fbidx[f] = uint32_t(J - R.nfree);
                    ++f;
                }
            }
    diag[row] = dg;
    lidx[row] = uint32_t(D.lvec_off + loc);
    if (!ordered || dg < 0) atomicOr(flags, 1);
    // one atomic per warp for the offset bound
    const unsigned act = __activemask();
    far = __reduce_max_sync(act, far);
    if ((threadIdx.x & 31) == __ffs(act) - 1) atomicMax(flags + 1, far);
}

// row pointers (int32, G+Smo's index_t) and lift pointers from the scans; identity load pointers
__global__ void __launch_bounds__(kBlock) k_pat_ptrs(int n, const long long* __restrict__ nslot,
                                                     const long long* __restrict__ nlift, int* __restrict__ ptr,
                                                     uint32_t* __restrict__ fptr, uint32_t* __restrict__ lptr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > n) return;
    ptr[i] = int(nslot[i]);
    fptr[i] = uint32_t(nlift[i]);
    lptr[i] = uint32_t(i);
}

__global__ void __launch_bounds__(kBlock) k_pat_coff(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                                                     int16_t* __restrict__ coff) {
    const int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= n) return;
    for (int k = ptr[row]; k < ptr[row + 1]; ++k) coff[k] = int16_t(col[k] - row);
}

inline unsigned blocksOf(long long n, int b) { return unsigned((n + b - 1) / b); }

void scanInPlace(long long* a, long long n, long long* sums, cudaStream_t s) {
    const long long nb = (n + kScanBlock - 1) / kScanBlock;
    k_scan_chunks<<<unsigned(nb), kScanBlock, 0, s>>>(a, n, sums);
    k_scan_sums<<<1, kScanBlock, 0, s>>>(sums, nb);
    k_scan_add<<<blocksOf(n, kBlock), kBlock, 0, s>>>(a, n, sums);
}

}  // namespace

namespace launch {

long long scanScratch(long long n) { return (n + kScanBlock - 1) / kScanBlock; }

void patternCount(const DevPatch* P, const RowPlanDev& R, long long* nslot, long long* nlift, long long* sums,
                  cudaStream_t s) {
    k_pat_count<<<blocksOf(R.n + 1LL, kBlock), kBlock, 0, s>>>(P, R, nslot, nlift);
    scanInPlace(nslot, R.n + 1LL, sums, s);
    scanInPlace(nlift, R.n + 1LL, sums, s);
}

void patternFill(const DevPatch* P, const RowPlanDev& R, const long long* nslot, const long long* nlift, int* ptr,
                 int* col, uint32_t* src, uint32_t* fptr, uint32_t* fband, uint32_t* fbidx, int* diag, uint32_t* lptr,
                 uint32_t* lidx, int* flags, cudaStream_t s) {
    k_pat_ptrs<<<blocksOf(R.n + 1LL, kBlock), kBlock, 0, s>>>(R.n, nslot, nlift, ptr, fptr, lptr);
    if (R.n > 0)
        k_pat_fill<<<blocksOf(R.n, kBlock), kBlock, 0, s>>>(P, R, nslot, nlift, col, src, fband, fbidx, diag, lidx,
                                                            flags);
}

void patternColOffsets(int n, const int* ptr, const int* col, int16_t* coff, cudaStream_t s) {
    if (n > 0) k_pat_coff<<<blocksOf(n, kBlock), kBlock, 0, s>>>(n, ptr, col, coff);
}

}  // namespace launch
}  // namespace gsgpu
