// Launch wrappers of the sm_103a kernels (kernels_assemble.cu, kernels_solve.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "device_funcs.cuh"
#include "gsgpu_internal.h"

namespace gsgpu {
namespace launch {

constexpr int kBlock = 256;

// assembly
void basisTables(const TabJob* jobs, long long njobs, const double* knots, double* out, cudaStream_t s);
template <typename T>
void pairFactors(const PfJob* jobs, const BlkEnt* tab, long long nblk, const double* basis, T* pf, cudaStream_t s);
template <typename R>
void geoStage1(const DevPatch* P, const BlkEnt* tab, long long nblk, const R* coefs, const R* gtab, const int* ibuf,
               R* Y1, cudaStream_t s);
template <typename R>
void geoStage2(const DevPatch* P, const BlkEnt* tab, long long nblk, const R* Y1, const R* gtab, const int* ibuf,
               R* Y2, cudaStream_t s);
// M = w |det J| per quadrature point into the load field's slot (the mass matrix's field)
void massField(const DevPatch* P, const BlkEnt* tab, long long nblk, const double* Y1, const double* Y2,
               const double* gtab, const int* ibuf, const double* wq, double* M, cudaStream_t s);
// kmax: the largest Fourier wave number of the fields (sizes the point kernel's powers table)
template <typename R>
void pointStep(const DevPatch* P, const BlkEnt* tab, long long nblk, const dev::FieldConst<R>* F, const R* Y1,
               const R* Y2, const R* gtab, const int* ibuf, const R* wq, R* C, R* Lf, unsigned long long* detkey,
               int kmax, cudaStream_t s);
template <typename T, int KIND>
void contract(const DevPatch* P, const BlkEnt* tab, long long nblk, const T* in, T* out, const int* ibuf, const T* pf,
              cudaStream_t s);
template <int KIND>
void contractDF(const DevPatch* P, const BlkEnt* tab, long long nblk, const df32* in, df32* out, const int* ibuf,
                const df32* pf, cudaStream_t s);
// 3D stage 1 interior rows in shared-memory tiles (degrees with dev::tiledStage31)
// nseg: the row segments per line when every tile belongs to one patch (the persistent kernel's
// grid is a multiple of it), else 0 (one block per tile)
void stage31Tile(int P, const DevPatch* Pd, const BlkEnt* tab, long long ntiles, const df32* in, df32* out,
                 const df32* pf, int nseg, cudaStream_t s);
// degree-P specialisation over the patches whose degree along the stage axis is P
// (degrees 1..4; the context checks the range)
// interior rows (unrolled fixed-shape kernel, tabInt) and the remaining rows (tabBnd)
template <int KIND, int H0, int NH>
void contractRowDF(int P, const DevPatch* Pd, const BlkEnt* tabInt, long long nInt, const BlkEnt* tabBnd,
                   long long nBnd, const df32* in, df32* out, const int* ibuf, const df32* pf, cudaStream_t s);
template <int KIND, typename Tin>
void loadContract(const DevPatch* P, const BlkEnt* tab, long long nblk, const Tin* in, double* out,
                  const double* basis, const int* ibuf, cudaStream_t s);
// the first load stage of the double-float path: df32 field and basis table, compensated sums
template <int KIND>
void loadContractDF(const DevPatch* P, const BlkEnt* tab, long long nblk, const df32* in, double* out,
                    const df32* basis, const int* ibuf, cudaStream_t s);
void gatherCsrDF(long long nnz, const uint32_t* src, const df32* band, const uint32_t* ovf_ptr, const uint32_t* ovf_idx,
                 float* hi, float* lo, cudaStream_t s);
void toDF(long long n, const double* in, df32* out, cudaStream_t s);
// FP32 rounding of double-float values
void dfToFloat(long long n, const df32* in, float* out, cudaStream_t s);
template <typename T>
void gatherCsr(long long nnz, const uint32_t* src, const T* band, const uint32_t* ovf_ptr, const uint32_t* ovf_idx,
               T* val, cudaStream_t s);
template <typename TB>
void rhsRows(int n, const double* lvec, const uint32_t* lptr, const uint32_t* lidx, const TB* band,
             const uint32_t* fptr, const uint32_t* fband, const uint32_t* fbidx, const double* ddof, double* rhs,
             cudaStream_t s);

// discrete L2 error: solution coefficients per patch-local dof, then per-block partial sums of
// (u_h - u)^2 w |det J| over the quadrature points (tabPoint blocks); h1: the H1 seminorm
// integrand |grad u_h - grad u|^2 w |det J| instead
void solutionCoefs(long long nlocal, const int* index, int nfree, const double* x, const double* ddof, double* coef,
                   cudaStream_t s);
void l2Partials(const DevPatch* P, const BlkEnt* tab, long long nblk, const dev::FieldConst<double>* F,
                const double* Y1, const double* Y2, const double* gtab, const int* ibuf, const double* wq,
                const double* btab, const double* coef, double* part, bool h1, cudaStream_t s);

// Neumann boundary integrals: w |n| h per face quadrature point (before the geometry table turns
// into double-float values), then per dof on a Neumann side its sums added to the load vector
void neumannFace(const NeuSide* sides, const BlkEnt* tab, long long nblk, const DevPatch* P,
                 const dev::FieldConst<double>* F, const double* coefs, const double* gtab, const int* ibuf,
                 const double* wq, double* vals, cudaStream_t s);
void neumannDofs(const NeuDof* dofs, long long ndofs, const NeuSide* sides, const DevPatch* P, const double* btab,
                 const int* ibuf, const double* vals, double* lvec, cudaStream_t s);

// sparsity pattern of a problem without interfaces on the device (pattern_dev.cu) from the host's
// row plan (plan.h RowPlan): counts and exclusive scans (nslot, nlift: n+1 entries), then the fill
struct RowPlanDev {
    int n = 0, nfree = 0;
    const int* rowPatch = nullptr;
    const int* rowLoc = nullptr;
    const int* rng = nullptr;
    const long long* rngOff = nullptr;
    const int* index = nullptr;  // dof map (patch-local -> global)
    const int* poff = nullptr;   // first patch-local dof of each patch
};
long long scanScratch(long long n);
void patternCount(const DevPatch* P, const RowPlanDev& R, long long* nslot, long long* nlift, long long* sums,
                  cudaStream_t s);
// flags[0]: a row without its diagonal or with unordered columns; flags[1]: largest |column - row|
void patternFill(const DevPatch* P, const RowPlanDev& R, const long long* nslot, const long long* nlift, int* ptr,
                 int* col, uint32_t* src, uint32_t* fptr, uint32_t* fband, uint32_t* fbidx, int* diag, uint32_t* lptr,
                 uint32_t* lidx, int* flags, cudaStream_t s);
void patternColOffsets(int n, const int* ptr, const int* col, int16_t* coff, cudaStream_t s);

// order-preserving uint64 key of a double (for atomicMin over signed values)
inline unsigned long long detKeyInit() { return ~0ULL; }
double detKeyDecode(unsigned long long key);

}  // namespace launch
}  // namespace gsgpu
