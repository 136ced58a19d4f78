// Launch wrappers of the sm_103a kernels (kernels_assemble.cu, kernels_solve.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "gsgpu_internal.h"

namespace gsgpu {
namespace launch {

constexpr int kBlock = 256;

// assembly
void basisTables(const TabJob* jobs, long long njobs, const double* knots, double* out, cudaStream_t s);
template <typename T>
void pairFactors(const PfJob* jobs, const BlkEnt* tab, long long nblk, const double* basis, T* pf, cudaStream_t s);
void geoStage1(const DevPatch* P, const BlkEnt* tab, long long nblk, const double* coefs, const double* gtab,
               const int* ibuf, double* Y1, cudaStream_t s);
void geoStage2(const DevPatch* P, const BlkEnt* tab, long long nblk, const double* Y1, const double* gtab,
               const int* ibuf, double* Y2, cudaStream_t s);
void pointStep(const DevPatch* P, const BlkEnt* tab, long long nblk, const FieldParams* F, const double* Y1,
               const double* Y2, const double* gtab, const int* ibuf, const double* wq, double* C, double* Lf,
               unsigned long long* detkey, cudaStream_t s);
template <typename T, int KIND>
void contract(const DevPatch* P, const BlkEnt* tab, long long nblk, const T* in, T* out, const int* ibuf, const T* pf,
              cudaStream_t s);
template <int KIND>
void loadContract(const DevPatch* P, const BlkEnt* tab, long long nblk, const double* in, double* out,
                  const double* basis, const int* ibuf, cudaStream_t s);
template <typename T>
void gatherCsr(long long nnz, const uint32_t* src, const T* band, const uint32_t* ovf_ptr, const uint32_t* ovf_idx,
               T* val, cudaStream_t s);
void rhsRows(int n, const double* lvec, const uint32_t* lptr, const uint32_t* lidx, const double* band,
             const uint32_t* fptr, const uint32_t* fband, const uint32_t* fbidx, const double* ddof, double* rhs,
             cudaStream_t s);

// order-preserving uint64 key of a double (for atomicMin over signed values)
inline unsigned long long detKeyInit() { return ~0ULL; }
double detKeyDecode(unsigned long long key);

}  // namespace launch
}  // namespace gsgpu
