// sm_103a assembly kernels: basis tables (K1), geometry map and coefficient fields (K2),
// sum-factorised stiffness / load contractions (K3) and the atomic-free CSR gather with the
// Dirichlet lift (K4). Thread -> item mapping only; the arithmetic lives in device_funcs.cuh.
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

template <typename T>
__global__ void __launch_bounds__(kBlock) k_pair(const PfJob* __restrict__ jobs, const BlkEnt* __restrict__ tab,
                                                 const double* __restrict__ basis, T* __restrict__ pf) {
    const BlkEnt be = tab[blockIdx.x];
    const PfJob j = jobs[be.patch];
    const long long item = be.base + threadIdx.x;
    if (item >= j.count) return;
    pf[j.pf + item] = dev::pairFactor<T>(basis + j.tab, j.p, j.q, j.E, item);
}

__global__ void __launch_bounds__(kBlock) k_geo1(const DevPatch* __restrict__ P, const BlkEnt* __restrict__ tab,
                                                 const double* __restrict__ coefs, const double* __restrict__ gtab,
                                                 const int* __restrict__ ibuf, double* __restrict__ Y1) {
    const BlkEnt be = tab[blockIdx.x];
    const DevPatch& D = P[be.patch];
    const long long item = be.base + threadIdx.x;
    const long long work = D.dim == 3 ? (long long)D.dim * 2 * D.gn[2] * D.gn[1] * D.Q[0]
                                      : (long long)D.dim * 2 * D.gn[1] * D.Q[0];
    if (item >= work) return;
    Y1[D.y1_off + item] = dev::geoStage1(D, item, coefs, gtab, ibuf);
}

__global__ void __launch_bounds__(kBlock) k_geo2(const DevPatch* __restrict__ P, const BlkEnt* __restrict__ tab,
                                                 const double* __restrict__ Y1, const double* __restrict__ gtab,
                                                 const int* __restrict__ ibuf, double* __restrict__ Y2) {
    const BlkEnt be = tab[blockIdx.x];
    const DevPatch& D = P[be.patch];
    const long long item = be.base + threadIdx.x;
    const long long work = (long long)D.dim * 3 * D.gn[2] * D.Q[1] * D.Q[0];
    if (item >= work) return;
    Y2[D.y2_off + item] = dev::geoStage2(D, item, Y1, gtab, ibuf);
}

__device__ __forceinline__ unsigned long long detKey(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    return (b & 0x8000000000000000ULL) ? ~b : (b | 0x8000000000000000ULL);
}

__global__ void __launch_bounds__(kBlock) k_point(const DevPatch* __restrict__ P, const BlkEnt* __restrict__ tab,
                                                  const FieldParams* __restrict__ F, const double* __restrict__ Y1,
                                                  const double* __restrict__ Y2, const double* __restrict__ gtab,
                                                  const int* __restrict__ ibuf, const double* __restrict__ wq,
                                                  double* __restrict__ C, double* __restrict__ Lf,
                                                  unsigned long long* __restrict__ detkey) {
    __shared__ FieldParams sF;
    // stage the coefficient parameters in shared memory (uniform across the block)
    {
        const int nw = int(sizeof(FieldParams) / sizeof(int));
        const int* src = reinterpret_cast<const int*>(F);
        int* dst = reinterpret_cast<int*>(&sF);
        for (int k = threadIdx.x; k < nw; k += blockDim.x) dst[k] = src[k];
    }
    __syncthreads();
    const BlkEnt be = tab[blockIdx.x];
    const DevPatch& D = P[be.patch];
    const long long item = be.base + threadIdx.x;
    unsigned long long key = ~0ULL;
    if (item < D.nq) key = detKey(dev::pointStep(D, sF, item, Y1, Y2, gtab, ibuf, wq, C, Lf));
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
__global__ void __launch_bounds__(kBlock) k_load(const DevPatch* __restrict__ P, const BlkEnt* __restrict__ tab,
                                                 const double* __restrict__ in, double* __restrict__ out,
                                                 const double* __restrict__ basis, const int* __restrict__ ibuf) {
    const BlkEnt be = tab[blockIdx.x];
    const DevPatch& D = P[be.patch];
    const long long item = be.base + threadIdx.x;
    if (item >= dev::loadWork<KIND>(D)) return;
    out[dev::loadGeom<KIND>(D).out_base + item] = dev::loadItem<KIND>(D, item, in, basis, ibuf);
}

template <typename T>
__global__ void __launch_bounds__(kBlock) k_gather(long long nnz, const uint32_t* __restrict__ src,
                                                   const T* __restrict__ band, const uint32_t* __restrict__ ovf_ptr,
                                                   const uint32_t* __restrict__ ovf_idx, T* __restrict__ val) {
    const long long s = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nnz) return;
    val[s] = dev::gatherSlot<T>(src[s], band, ovf_ptr, ovf_idx);
}

__global__ void __launch_bounds__(kBlock) k_rhs(int n, const double* __restrict__ lvec, const uint32_t* __restrict__ lptr,
                                                const uint32_t* __restrict__ lidx, const double* __restrict__ band,
                                                const uint32_t* __restrict__ fptr, const uint32_t* __restrict__ fband,
                                                const uint32_t* __restrict__ fbidx, const double* __restrict__ ddof,
                                                double* __restrict__ rhs) {
    const int I = blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= n) return;
    rhs[I] = dev::rhsRow(I, lvec, lptr, lidx, band, fptr, fband, fbidx, ddof);
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
    if (njobs > 0) k_basis<<<grid1(njobs), kBlock, 0, s>>>(jobs, njobs, knots, out);
}
template <typename T>
void pairFactors(const PfJob* jobs, const BlkEnt* tab, long long nblk, const double* basis, T* pf, cudaStream_t s) {
    if (nblk > 0) k_pair<T><<<unsigned(nblk), kBlock, 0, s>>>(jobs, tab, basis, pf);
}
template void pairFactors<double>(const PfJob*, const BlkEnt*, long long, const double*, double*, cudaStream_t);
template void pairFactors<float>(const PfJob*, const BlkEnt*, long long, const double*, float*, cudaStream_t);

void geoStage1(const DevPatch* P, const BlkEnt* tab, long long nblk, const double* coefs, const double* gtab,
               const int* ibuf, double* Y1, cudaStream_t s) {
    if (nblk > 0) k_geo1<<<unsigned(nblk), kBlock, 0, s>>>(P, tab, coefs, gtab, ibuf, Y1);
}
void geoStage2(const DevPatch* P, const BlkEnt* tab, long long nblk, const double* Y1, const double* gtab,
               const int* ibuf, double* Y2, cudaStream_t s) {
    if (nblk > 0) k_geo2<<<unsigned(nblk), kBlock, 0, s>>>(P, tab, Y1, gtab, ibuf, Y2);
}
void pointStep(const DevPatch* P, const BlkEnt* tab, long long nblk, const FieldParams* F, const double* Y1,
               const double* Y2, const double* gtab, const int* ibuf, const double* wq, double* C, double* Lf,
               unsigned long long* detkey, cudaStream_t s) {
    if (nblk > 0) k_point<<<unsigned(nblk), kBlock, 0, s>>>(P, tab, F, Y1, Y2, gtab, ibuf, wq, C, Lf, detkey);
}
template <typename T, int KIND>
void contract(const DevPatch* P, const BlkEnt* tab, long long nblk, const T* in, T* out, const int* ibuf, const T* pf,
              cudaStream_t s) {
    if (nblk > 0) k_contract<T, KIND><<<unsigned(nblk), kBlock, 0, s>>>(P, tab, in, out, ibuf, pf);
}
#define INST_CONTRACT(T, K) \
    template void contract<T, K>(const DevPatch*, const BlkEnt*, long long, const T*, T*, const int*, const T*, cudaStream_t);
INST_CONTRACT(double, 31)
INST_CONTRACT(double, 32)
INST_CONTRACT(double, 33)
INST_CONTRACT(double, 21)
INST_CONTRACT(double, 22)
INST_CONTRACT(float, 31)
INST_CONTRACT(float, 32)
INST_CONTRACT(float, 33)
INST_CONTRACT(float, 21)
INST_CONTRACT(float, 22)

template <int KIND>
void loadContract(const DevPatch* P, const BlkEnt* tab, long long nblk, const double* in, double* out,
                  const double* basis, const int* ibuf, cudaStream_t s) {
    if (nblk > 0) k_load<KIND><<<unsigned(nblk), kBlock, 0, s>>>(P, tab, in, out, basis, ibuf);
}
template void loadContract<31>(const DevPatch*, const BlkEnt*, long long, const double*, double*, const double*, const int*, cudaStream_t);
template void loadContract<32>(const DevPatch*, const BlkEnt*, long long, const double*, double*, const double*, const int*, cudaStream_t);
template void loadContract<33>(const DevPatch*, const BlkEnt*, long long, const double*, double*, const double*, const int*, cudaStream_t);
template void loadContract<21>(const DevPatch*, const BlkEnt*, long long, const double*, double*, const double*, const int*, cudaStream_t);
template void loadContract<22>(const DevPatch*, const BlkEnt*, long long, const double*, double*, const double*, const int*, cudaStream_t);

template <typename T>
void gatherCsr(long long nnz, const uint32_t* src, const T* band, const uint32_t* ovf_ptr, const uint32_t* ovf_idx,
               T* val, cudaStream_t s) {
    if (nnz > 0) k_gather<T><<<grid1(nnz), kBlock, 0, s>>>(nnz, src, band, ovf_ptr, ovf_idx, val);
}
template void gatherCsr<double>(long long, const uint32_t*, const double*, const uint32_t*, const uint32_t*, double*, cudaStream_t);
template void gatherCsr<float>(long long, const uint32_t*, const float*, const uint32_t*, const uint32_t*, float*, cudaStream_t);

void rhsRows(int n, const double* lvec, const uint32_t* lptr, const uint32_t* lidx, const double* band,
             const uint32_t* fptr, const uint32_t* fband, const uint32_t* fbidx, const double* ddof, double* rhs,
             cudaStream_t s) {
    if (n > 0) k_rhs<<<grid1(n), kBlock, 0, s>>>(n, lvec, lptr, lidx, band, fptr, fband, fbidx, ddof, rhs);
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
