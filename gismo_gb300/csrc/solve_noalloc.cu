// Jacobi-preconditioned CG on a caller-provided device CSR system, allocating no device memory.
//
// The solver's working vectors, partial sums and scalar state live in one file-scope device
// array (kNoAllocScratchDoubles doubles = 8 MiB), which every GPU that loads the library keeps
// until the process exits. The iteration is the one of gsgpu_solve (the same kernels, launched
// one chunk at a time without a CUDA graph, so nothing is instantiated or allocated); only the
// Jacobi diagonal is found on the device by a binary search in each sorted CSR row. Each call
// reads the row-pointer end and the solver state back to the host and synchronises its stream.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/gsgpu.h"
#include "kernels_solve.h"

namespace gsgpu {
namespace {

constexpr long long kNoAllocScratchDoubles = 1LL << 20;  // 8 MiB
constexpr int kMaxDevices = 64;
constexpr int kStateDoubles = 64;  // CgState + error flag, padded

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

std::mutex g_setup_mutex;
double* g_scratch_addr[kMaxDevices] = {};

// scratch doubles needed for n unknowns: state, dinv r z p t, CG partials x2, SpMV partials
long long scratchNeeded(long long n) {
    const long long np = (n + 255) / 256;
    const long long nb = (n + 7) / 8;  // 32 lanes per row: 8 rows per 256-thread block
    return kStateDoubles + 5 * n + 2 * np + nb;
}

// dinv[i] = 1 / A(i,i), the diagonal found by binary search in the sorted columns of row i;
// a missing or zero diagonal sets the error flag and leaves dinv[i] = 0
__global__ void k_dinv_search(int n, const int* __restrict__ ptr, const int* __restrict__ col,
                              const double* __restrict__ val, double* __restrict__ dinv, int* __restrict__ flag) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int lo = ptr[i], hi = ptr[i + 1] - 1;
    double d = 0.0;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        const int c = col[mid];
        if (c == i) {
            d = val[mid];
            break;
        }
        if (c < i) lo = mid + 1;
        else hi = mid - 1;
    }
    if (d == 0.0) {
        *flag = 1;
        dinv[i] = 0.0;
    } else {
        dinv[i] = 1.0 / d;
    }
}

}  // namespace
}  // namespace gsgpu

extern "C" int gsgpu_cg_jacobi_noalloc(int n, const int* ptr, const int* col, const double* val, const double* b,
                                       double* x, double tol, int max_iters, void* stream, int* iterations,
                                       double* relres) {
    using namespace gsgpu;
    if (iterations) *iterations = 0;
    if (relres) *relres = 0.0;
    if (n < 1 || !ptr || !col || !val || !b || !x) return GSGPU_ERR_INVALID;
    if (scratchNeeded(n) > kNoAllocScratchDoubles) return GSGPU_ERR_INVALID;  // n above the fixed maximum
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GSGPU_ERR_CUDA;
    double* scratch = nullptr;
    {
        // once per device, with that device current: the device address of the scratch array
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        if (!g_scratch_addr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return GSGPU_ERR_CUDA;
            g_scratch_addr[dev] = static_cast<double*>(p);
        }
        scratch = g_scratch_addr[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // an error the caller already had pending is reported as such and left pending, not taken
    // for this call's
    if (cudaPeekAtLastError() != cudaSuccess) return GSGPU_ERR_CUDA;
    const long long np = (n + 255) / 256;
    CgState* st = reinterpret_cast<CgState*>(scratch);
    int* flag = reinterpret_cast<int*>(scratch + kStateDoubles - 1);
    double* w = scratch + kStateDoubles;
    double* dinv = w;
    // the array keeps the previous call's contents: clear the error flag before use
    if (cudaMemsetAsync(flag, 0, sizeof(int), s) != cudaSuccess) return GSGPU_ERR_CUDA;
    k_dinv_search<<<unsigned((n + 255) / 256), 256, 0, s>>>(n, ptr, col, val, dinv, flag);
    if (cudaGetLastError() != cudaSuccess) return GSGPU_ERR_CUDA;
    // the row-pointer end (the average row length picks the lanes per row) and the diagonal flag in
    // one round trip; a row without a non-zero diagonal is rejected before any iteration
    int nnz_end = 0, hflag = 0;
    if (cudaMemcpyAsync(&nnz_end, ptr + n, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return GSGPU_ERR_CUDA;
    if (hflag) return GSGPU_ERR_INVALID;
    const double avg = double(nnz_end) / n;
    CgBuffers B;
    B.n = n;
    B.lanes_per_row = avg > 48 ? 32 : (avg > 20 ? 16 : (avg > 10 ? 8 : 4));
    B.ptr = ptr;
    B.col = col;
    B.val = val;
    B.b = b;
    B.x = x;
    B.dinv = dinv;
    B.r = w + n;
    B.z = w + 2LL * n;
    B.p = w + 3LL * n;
    B.t = w + 4LL * n;
    B.part0 = w + 5LL * n;
    B.part1 = B.part0 + np;
    B.part2 = B.part1 + np;  // (n + 7) / 8 doubles: at least the SpMV blocks of every lanes-per-row choice
    B.st = st;
    const int maxit = max_iters > 0 ? max_iters : 1000;
    launch::cgInit(B, tol > 0 ? tol : 1e-10, maxit, s);
    if (cudaGetLastError() != cudaSuccess) return GSGPU_ERR_CUDA;
    CgState hs{};
    const int chunk = 16;
    for (int it = 0; it < maxit + chunk; it += chunk) {
        for (int k = 0; k < chunk; ++k) launch::cgIteration(B, s);
        if (cudaMemcpyAsync(&hs, st, sizeof(CgState), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return GSGPU_ERR_CUDA;
        if (hs.done) break;
    }
    if (cudaGetLastError() != cudaSuccess) return GSGPU_ERR_CUDA;
    if (iterations) *iterations = hs.iters;
    if (relres) *relres = hs.relres;
    return hs.done == 1 ? GSGPU_OK : GSGPU_ERR_NOT_CONVERGED;
}
