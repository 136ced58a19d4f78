// libgsgpu C ABI (include/gsgpu.h): context, refresh (host set-up + upload), assemble (K1-K4 on
// the device) and the CG solvers.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gsgpu.h"
#include "context.h"
#include "device_funcs.cuh"
#include "kernels.h"
#include "kernels_solve.h"
#include "plan.h"

namespace gsgpu {

CudaError::CudaError(cudaError_t e, const char* expr, const char* file, int line)
    : std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e) + " in " + expr + " (" + file + ":" +
                         std::to_string(line) + ")"),
      code(e) {}

void* DeviceArena::alloc(size_t bytes) {
    if (bytes == 0) return nullptr;
    if (budget > 0 && used + bytes > budget) throw BudgetError("device-memory budget exceeded");
    void* p = nullptr;
    if (stream) GSGPU_CUDA_TRY(cudaMallocAsync(&p, bytes, stream));
    else GSGPU_CUDA_TRY(cudaMalloc(&p, bytes));
    used += bytes;
    sizes.push_back({p, bytes});
    return p;
}
void DeviceArena::release(void* p) {
    if (!p) return;
    for (size_t i = 0; i < sizes.size(); ++i)
        if (sizes[i].first == p) {
            used -= sizes[i].second;
            sizes.erase(sizes.begin() + long(i));
            if (stream) cudaFreeAsync(p, stream);
            else cudaFree(p);
            return;
        }
}
void DeviceArena::releaseAll() {
    for (auto& s : sizes) {
        if (stream) cudaFreeAsync(s.first, stream);
        else cudaFree(s.first);
    }
    sizes.clear();
    used = 0;
}


}  // namespace gsgpu

using namespace gsgpu;

// ---------------------------------------------------------------------------------------------
// assembly-time helpers

namespace gsgpu {

void Context::buildTables() {
    auto mk = [&](Tab& T, auto workfn) {
        std::vector<long long> w;
        for (const DevPatch& D : L.dev) w.push_back(workfn(D));
        blockTable(w, launch::kBlock, T.h);
        upload(arena, T.d, T.h, stream);
    };
    {
        std::vector<long long> w;
        for (const PfJob& j : L.pfjobs) w.push_back(j.count);
        blockTable(w, launch::kBlock, tabPf.h);
        upload(arena, tabPf.d, tabPf.h, stream);
    }
    mk(tabCoef, [](const DevPatch& D) { return D.ngeo * D.dim; });
    mk(tabGeo1, [](const DevPatch& D) {
        return D.dim == 3 ? (long long)D.dim * 2 * D.gn[2] * D.gn[1] * D.Q[0] : (long long)D.dim * 2 * D.gn[1] * D.Q[0];
    });
    mk(tabGeo2, [](const DevPatch& D) { return D.dim == 3 ? (long long)D.dim * 3 * D.gn[2] * D.Q[1] * D.Q[0] : 0LL; });
    mk(tabPoint, [](const DevPatch& D) { return D.nq; });
    if (pd.dim == 3) {
        mk(tabSt[0], [](const DevPatch& D) { return dev::stageWork<31>(D); });
        mk(tabSt[1], [](const DevPatch& D) { return dev::stageWork<32>(D); });
        mk(tabSt[2], [](const DevPatch& D) { return dev::stageWork<33>(D); });
        for (int P = 1; P <= 4; ++P) {
            mk(tabRow[0][P], [P](const DevPatch& D) { return D.p[0] == P ? dev::stageInteriorWork<31>(D) : 0LL; });
            mk(tabTile31[P],
               [P](const DevPatch& D) { return D.p[0] == P ? dev::stage31Tiles(D) * launch::kBlock : 0LL; });
            mk(tabRow[1][P], [P](const DevPatch& D) { return D.p[1] == P ? dev::stageInteriorWork<32>(D) : 0LL; });
            mk(tabRow[2][P], [P](const DevPatch& D) { return D.p[2] == P ? dev::stageInteriorWork<33>(D) : 0LL; });
            mk(tabRowB[0][P], [P](const DevPatch& D) { return D.p[0] == P ? dev::stageBoundaryWork<31>(D) : 0LL; });
            mk(tabRowB[1][P], [P](const DevPatch& D) { return D.p[1] == P ? dev::stageBoundaryWork<32>(D) : 0LL; });
            mk(tabRowB[2][P], [P](const DevPatch& D) { return D.p[2] == P ? dev::stageBoundaryWork<33>(D) : 0LL; });
        }
        mk(tabLd[0], [](const DevPatch& D) { return dev::loadWork<31>(D); });
        mk(tabLd[1], [](const DevPatch& D) { return dev::loadWork<32>(D); });
        mk(tabLd[2], [](const DevPatch& D) { return dev::loadWork<33>(D); });
    } else {
        mk(tabSt[0], [](const DevPatch& D) { return dev::stageWork<21>(D); });
        mk(tabSt[1], [](const DevPatch& D) { return dev::stageWork<22>(D); });
        for (int P = 1; P <= 4; ++P) {
            mk(tabRow[0][P], [P](const DevPatch& D) { return D.p[0] == P ? dev::stageInteriorWork<21>(D) : 0LL; });
            mk(tabRow[1][P], [P](const DevPatch& D) { return D.p[1] == P ? dev::stageInteriorWork<22>(D) : 0LL; });
            mk(tabRowB[0][P], [P](const DevPatch& D) { return D.p[0] == P ? dev::stageBoundaryWork<21>(D) : 0LL; });
            mk(tabRowB[1][P], [P](const DevPatch& D) { return D.p[1] == P ? dev::stageBoundaryWork<22>(D) : 0LL; });
        }
        mk(tabLd[0], [](const DevPatch& D) { return dev::loadWork<21>(D); });
        mk(tabLd[1], [](const DevPatch& D) { return dev::loadWork<22>(D); });
    }
    buildNeumann(pd, L, launch::kBlock, neu);
    if (!neu.sides.empty()) {
        upload(arena, dNeuSides, neu.sides, stream);
        upload(arena, dNeuDofs, neu.dofs, stream);
        upload(arena, dNeuBlocks, neu.blocks, stream);
        allocN(arena, dNeuVals, neu.nvals);
    }
}

void Context::refresh() {
    if (!hasProblem) throw StateError("refresh() before set_problem()");
    if (device >= 0) freeAssembly();
    buildDofMap(pd, map);
    buildLayout(pd, L);
    // problems without interfaces get their pattern built on the device (no host non-zeros)
    RowPlan rp;
    devPattern = device >= 0 && std::getenv("GSGPU_HOST_PATTERN") == nullptr && rowPlanSingle(pd, map, L, rp);
    if (devPattern) {
        pat = Pattern();
        pat.n = map.freeSize;
    } else {
        buildPattern(pd, map, L, pat, 0);
        nnz = (long long)pat.col.size();
    }
    if (batch) segRow = segmentRows(pd, map);
    setupSdia();
    setupSegSdia();
    applyTuning();
    if (device < 0) {  // host-only context: the plan, no device buffers
        refreshed = true;
        return;
    }
    refreshUploads();
    if (devPattern) patternOnDevice(rp);
    else patternFromHost();
    findBoxRows();
    if (batch) batchSetup();
    allocN(arena, dVal, nnz);
    allocN(arena, dRhs, pat.n);
    allocN(arena, dDdof, std::max(1, map.boundarySize));
    allocN(arena, dDetKey, 1);
    buildTables();
    // the control points of the problem
    std::vector<double> raw;
    for (const HostPatch& P : pd.patches) raw.insert(raw.end(), P.coefs.begin(), P.coefs.end());
    GSGPU_CUDA_TRY(cudaMemcpyAsync(dCoefRaw, raw.data(), raw.size() * sizeof(double), cudaMemcpyHostToDevice, stream));
    launch::coefsToSoa(dPatches, tabCoef.d, (long long)tabCoef.h.size(), dCoefRaw, dCoefs, stream);
    GSGPU_CUDA_TRY(cudaStreamSynchronize(stream));
    refreshed = true;
    assembled = false;
    solved = false;
}

// sparsity pattern, gather maps and diagonal slots on the device from the row plan
void Context::patternOnDevice(const RowPlan& rp) {
    cudaStream_t s = stream;
    const int n = pat.n;
    int *dRowPatch = nullptr, *dRowLoc = nullptr, *dRng = nullptr, *dPoff = nullptr, *dFlags = nullptr;
    long long *dRngOff = nullptr, *cnt0 = nullptr, *cnt1 = nullptr, *sums = nullptr;
    std::vector<int> poff;
    for (const HostPatch& P : pd.patches) poff.push_back(P.offset);
    upload(arena, dRowPatch, rp.rowPatch, s);
    upload(arena, dRowLoc, rp.rowLoc, s);
    upload(arena, dRng, rp.rng.empty() ? std::vector<int>(1, 0) : rp.rng, s);
    upload(arena, dRngOff, rp.rngOff, s);
    upload(arena, dPoff, poff, s);
    allocN(arena, cnt0, n + 1LL);
    allocN(arena, cnt1, n + 1LL);
    allocN(arena, sums, std::max(1LL, launch::scanScratch(n + 1LL)));
    allocN(arena, dFlags, 2);
    GSGPU_CUDA_TRY(cudaMemsetAsync(dFlags, 0, 2 * sizeof(int), s));
    launch::RowPlanDev R;
    R.n = n;
    R.nfree = map.freeSize;
    R.rowPatch = dRowPatch;
    R.rowLoc = dRowLoc;
    R.rng = dRng;
    R.rngOff = dRngOff;
    R.index = dIndex;
    R.poff = dPoff;
    launch::patternCount(dPatches, R, cnt0, cnt1, sums, s);
    long long tot[2] = {0, 0};
    GSGPU_CUDA_TRY(cudaMemcpyAsync(&tot[0], cnt0 + n, sizeof(long long), cudaMemcpyDeviceToHost, s));
    GSGPU_CUDA_TRY(cudaMemcpyAsync(&tot[1], cnt1 + n, sizeof(long long), cudaMemcpyDeviceToHost, s));
    GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
    if (tot[0] >= (1LL << 31)) throw std::invalid_argument("more than 2^31 non-zeros");
    if (L.band >= (long long)Pattern::kMulti) throw std::invalid_argument("band too large for 31-bit band indexing");
    nnz = tot[0];
    allocN(arena, dPtr, n + 1LL);
    allocN(arena, dCol, std::max(1LL, nnz));
    allocN(arena, dSrc, std::max(1LL, nnz));
    allocN(arena, dFptr, n + 1LL);
    allocN(arena, dFband, std::max(1LL, tot[1]));
    allocN(arena, dFbidx, std::max(1LL, tot[1]));
    allocN(arena, dDiag, std::max(1, n));
    allocN(arena, dLptr, n + 1LL);
    allocN(arena, dLidx, std::max(1, n));
    upload(arena, dOvfPtr, std::vector<uint32_t>(1, 0), s);
    upload(arena, dOvfIdx, std::vector<uint32_t>(1, 0), s);
    launch::patternFill(dPatches, R, cnt0, cnt1, dPtr, dCol, dSrc, dFptr, dFband, dFbidx, dDiag, dLptr, dLidx, dFlags,
                        s);
    int flags[2] = {0, 0};
    GSGPU_CUDA_TRY(cudaMemcpyAsync(flags, dFlags, sizeof(flags), cudaMemcpyDeviceToHost, s));
    GSGPU_CUDA_TRY(cudaGetLastError());
    GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
    if (flags[0]) throw std::runtime_error("device pattern: a row without its diagonal or with unordered columns");
    arena.release(dColOff);
    dColOff = nullptr;
    if (flags[1] <= 32767 && nnz > 0) {  // banded patterns: 16-bit column offsets from the row
        allocN(arena, dColOff, nnz);
        launch::patternColOffsets(n, dPtr, dCol, dColOff, s);
    }
    GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
    for (void* p : {(void*)dRowPatch, (void*)dRowLoc, (void*)dRng, (void*)dRngOff, (void*)dPoff, (void*)cnt0,
                    (void*)cnt1, (void*)sums, (void*)dFlags})
        arena.release(p);
}

// the host pattern: diagonal slots, uploads and 16-bit column offsets when they fit
void Context::patternFromHost() {
    // diagonal slot of every row (Jacobi)
    diag.assign(pat.n, -1);
    int nodiag = 0;
#pragma omp parallel for schedule(static) reduction(+ : nodiag)
    for (int r = 0; r < pat.n; ++r) {
        const int* b = pat.col.data() + pat.ptr[r];
        const int* e = pat.col.data() + pat.ptr[r + 1];
        const int* f = std::lower_bound(b, e, r);
        if (f == e || *f != r) ++nodiag;
        else diag[r] = pat.ptr[r] + int(f - b);
    }
    if (nodiag) throw std::runtime_error("pattern has no diagonal entry");
    upload(arena, dPtr, pat.ptr, stream);
    upload(arena, dCol, pat.col, stream);
    upload(arena, dSrc, pat.src, stream);
    upload(arena, dOvfPtr, pat.ovf_ptr.empty() ? std::vector<uint32_t>(1, 0) : pat.ovf_ptr, stream);
    upload(arena, dOvfIdx, pat.ovf_idx.empty() ? std::vector<uint32_t>(1, 0) : pat.ovf_idx, stream);
    upload(arena, dLptr, pat.lptr, stream);
    upload(arena, dLidx, pat.lidx, stream);
    upload(arena, dFptr, pat.fptr, stream);
    upload(arena, dFband, pat.fband.empty() ? std::vector<uint32_t>(1, 0) : pat.fband, stream);
    upload(arena, dFbidx, pat.fbidx.empty() ? std::vector<uint32_t>(1, 0) : pat.fbidx, stream);
    upload(arena, dDiag, diag, stream);
    {
        // banded patterns (single patches) store columns as 16-bit offsets from the row
        int far = 0;
#pragma omp parallel for schedule(static) reduction(+ : far)
        for (int r = 0; r < pat.n; ++r)
            for (int k = pat.ptr[r]; k < pat.ptr[r + 1]; ++k)
                if (pat.col[k] - r > 32767 || pat.col[k] - r < -32768) ++far;
        arena.release(dColOff);
        dColOff = nullptr;
        if (far == 0 && !pat.col.empty()) {
            bigvec<int16_t> off(pat.col.size());
#pragma omp parallel for schedule(static)
            for (int r = 0; r < pat.n; ++r)
                for (int k = pat.ptr[r]; k < pat.ptr[r + 1]; ++k) off[k] = int16_t(pat.col[k] - r);
            upload(arena, dColOff, off, stream);
        }
    }
}

// box rows: rows whose columns are the row plus the column offsets of one reference row, a row of
// the most frequent length nearest the middle (in a patch's lexicographic numbering: the full
// neighbour box of every basis function away from the boundary). The FP32 SpMVs take their column
// offsets from a shared table there; kept when they are at least a quarter of the rows of a
// large system.
void Context::findBoxRows() {
    arena.release(dBoxFlag);
    dBoxFlag = nullptr;
    arena.release(dBoxOff);
    dBoxOff = nullptr;
    nBox = 0;
    nBoxRows = 0;
    const int n = pat.n;
    if (n < (1 << 14) || nnz == 0 || std::getenv("GSGPU_NO_BOX_ROWS")) return;
    cudaStream_t s = stream;
    std::vector<int> hptr;
    const int* P = pat.ptr.data();
    if (devPattern) {
        hptr.resize(size_t(n) + 1);
        GSGPU_CUDA_TRY(cudaMemcpyAsync(hptr.data(), dPtr, hptr.size() * sizeof(int), cudaMemcpyDeviceToHost, s));
        GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
        P = hptr.data();
    }
    std::vector<int> hist(launch::kMaxBox + 1, 0);
    for (int r = 0; r < n; ++r) {
        const int len = P[r + 1] - P[r];
        if (len <= launch::kMaxBox) ++hist[len];
    }
    const int boxLen = int(std::max_element(hist.begin() + 2, hist.end()) - hist.begin());
    if (hist[boxLen] * 4LL < n) return;
    int r0 = -1;
    for (int d = 0; d <= n / 2 && r0 < 0; ++d)
        for (int r : {n / 2 + d, n / 2 - d})
            if (r0 < 0 && r >= 0 && r < n && P[r + 1] - P[r] == boxLen) r0 = r;
    if (r0 < 0) return;
    std::vector<int> off(boxLen);
    if (devPattern) {
        GSGPU_CUDA_TRY(cudaMemcpyAsync(off.data(), dCol + P[r0], boxLen * sizeof(int), cudaMemcpyDeviceToHost, s));
        GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
    } else {
        std::copy(pat.col.data() + P[r0], pat.col.data() + P[r0] + boxLen, off.begin());
    }
    for (int& v : off) v -= r0;
    upload(arena, dBoxOff, off, s);
    allocN(arena, dBoxFlag, n);
    unsigned long long* dCount = nullptr;
    allocN(arena, dCount, 1);
    GSGPU_CUDA_TRY(cudaMemsetAsync(dCount, 0, sizeof(unsigned long long), s));
    launch::boxFlags(n, dPtr, dCol, dBoxOff, boxLen, dBoxFlag, dCount, s);
    unsigned long long cnt = 0;
    GSGPU_CUDA_TRY(cudaMemcpyAsync(&cnt, dCount, sizeof(cnt), cudaMemcpyDeviceToHost, s));
    GSGPU_CUDA_TRY(cudaGetLastError());
    GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
    arena.release(dCount);
    if (cnt * 4 < (unsigned long long)n) {
        arena.release(dBoxFlag);
        dBoxFlag = nullptr;
        arena.release(dBoxOff);
        dBoxOff = nullptr;
        return;
    }
    nBox = boxLen;
    nBoxRows = (long long)cnt;
}

// The half-diagonal FP32 inner operator applies to a patch with simple knots along every axis and
// degrees 1..4 whose free dofs (global indices idx[0..ndofs) of its functions, free below freeSize)
// are one box of m0 x m1 x m2 patch-local functions numbered lexicographically from row0, at least
// 2p + 1 wide along every axis; lo is the box's lower corner. Checked on the dof map itself.
static bool patchBox(const DevPatch& D, const int* idx, int freeSize, int row0, int m[3], int lo[3]) {
    const int dim = D.dim;
    for (int k = 0; k < dim; ++k)
        if (!D.simple[k] || D.p[k] < 1 || D.p[k] > 4) return false;
    int hi[3] = {1, 1, 1}, nd[3] = {1, 1, 1};
    for (int k = 0; k < 3; ++k) lo[k] = 0, m[k] = 1;
    for (int k = 0; k < dim; ++k) nd[k] = D.n[k], lo[k] = nd[k], hi[k] = -1;
    long long cnt = 0;
    for (int i2 = 0; i2 < nd[2]; ++i2)
        for (int i1 = 0; i1 < nd[1]; ++i1)
            for (int i0 = 0; i0 < nd[0]; ++i0)
                if (idx[(size_t(i2) * nd[1] + i1) * nd[0] + i0] < freeSize) {
                    const int c[3] = {i0, i1, i2};
                    ++cnt;
                    for (int k = 0; k < dim; ++k) lo[k] = std::min(lo[k], c[k]), hi[k] = std::max(hi[k], c[k] + 1);
                }
    if (cnt == 0) return false;
    long long nbox = 1;
    for (int k = 0; k < dim; ++k) {
        m[k] = hi[k] - lo[k];
        if (m[k] < 2 * D.p[k] + 1) return false;
        nbox *= m[k];
    }
    if (nbox != cnt) return false;
    for (int i2 = 0; i2 < nd[2]; ++i2)
        for (int i1 = 0; i1 < nd[1]; ++i1)
            for (int i0 = 0; i0 < nd[0]; ++i0) {
                const int c[3] = {i0, i1, i2};
                bool in = true;
                for (int k = 0; k < dim; ++k) in = in && c[k] >= lo[k] && c[k] < hi[k];
                const int J = idx[(size_t(i2) * nd[1] + i1) * nd[0] + i0];
                const long long want = in ? row0 + (long long)(c[0] - lo[0]) +
                                                (long long)m[0] * ((c[1] - lo[1]) + (long long)m[1] * (c[2] - lo[2]))
                                          : -1;
                if (in ? J != want : J < freeSize) return false;
            }
    return true;
}

// The single-patch form (sdia.cu) for a problem of one patch (not a batch); GSGPU_NO_SDIA=1 keeps
// the CSR form (the tests compare the two).
void Context::setupSdia() {
    sdiaOk = false;
    sdiaOp = SdiaOp();
    sdiaBand = SdiaBand();
    if (batch || pd.patches.size() != 1 || std::getenv("GSGPU_NO_SDIA")) return;
    const DevPatch& D = L.dev[0];
    const int dim = D.dim;
    int m[3], lo[3];
    if (!patchBox(D, map.index.data(), map.freeSize, 0, m, lo)) return;
    const int nfree = map.freeSize;
    if ((long long)m[0] * m[1] * m[2] != nfree) return;
    sdiaOp.n = nfree;
    for (int k = 0; k < 3; ++k) {
        sdiaOp.m[k] = m[k];
        sdiaOp.p[k] = k < dim ? D.p[k] : 0;
        sdiaBand.n[k] = k < dim ? D.n[k] : 1;
        sdiaBand.W[k] = k < dim ? D.W[k] : 1;
        sdiaBand.lo[k] = k < dim ? lo[k] : 0;
    }
    sdiaOp.nh = launch::sdiaHalf(sdiaOp.p);
    sdiaOp.ns = (nfree + 255) / 256 * 256;
    sdiaOk = true;
}

// The batched form (kernels_batch.cu) for the problems of a batch that are such patches: per problem
// its half diagonals, unpadded, one after the other (the other problems keep their CSR rows).
// GSGPU_NO_SDIA=1 keeps the CSR form for all.
void Context::setupSegSdia() {
    segSdiaOk = false;
    segSdiaHost.clear();
    segSdiaSize = 0;
    if (!batch || std::getenv("GSGPU_NO_SDIA")) return;
    long long doff = 0;
    int count = 0;
    std::vector<SegSdiaDesc> descs;
    for (size_t q = 0; q < pd.patches.size(); ++q) {
        const HostPatch& P = pd.patches[q];
        const DevPatch& D = L.dev[q];
        SegSdiaDesc S;
        S.row0 = segRow[q];
        S.n = segRow[q + 1] - segRow[q];
        int m[3], lo[3];
        if (S.n == 0 || !patchBox(D, map.index.data() + P.offset, map.freeSize, S.row0, m, lo)) {
            S.doff = doff;  // nh = 0: CSR rows
            descs.push_back(S);
            continue;
        }
        ++count;
        for (int k = 0; k < 3; ++k) {
            S.m[k] = m[k];
            S.p[k] = k < D.dim ? D.p[k] : 0;
            S.bn[k] = k < D.dim ? D.n[k] : 1;
            S.W[k] = k < D.dim ? D.W[k] : 1;
            S.lo[k] = k < D.dim ? lo[k] : 0;
        }
        S.band_off = D.band_off;
        S.nh = launch::sdiaHalf(S.p);
        S.doff = doff;
        doff += (long long)S.nh * S.n;
        descs.push_back(S);
    }
    if (std::getenv("GSGPU_BATCH_DEBUG"))
        fprintf(stderr, "[batch] half-diagonal inner operator: %d of %zu problems, %lld values\n", count,
                pd.patches.size(), doff);
    if (count == 0) return;
    segSdiaHost.swap(descs);
    segSdiaSize = doff;
    segSdiaOk = true;
}

// patch data, tables and the assembly buffers (everything but the pattern)
void Context::refreshUploads() {
    upload(arena, dPatches, L.dev, stream);
    {
        std::vector<dev::FieldConst<double>> fc64;
        std::vector<dev::FieldConst<df32>> fcdf;
        fieldKmax = 0;
        for (const FieldParams& F : pd.fieldTable()) {
            fc64.push_back(dev::fieldConst<double>(F));
            fcdf.push_back(dev::fieldConst<df32>(F));
            fieldKmax = std::max(fieldKmax, F.kmax);
        }
        upload(arena, dFields, fc64, stream);
        upload(arena, dFieldsDf, fcdf, stream);
    }
    {
        std::vector<df32> w(L.wq.size());
        for (size_t i = 0; i < w.size(); ++i) w[i] = df32(L.wq[i]);
        upload(arena, dWqDf, w, stream);
    }
    upload(arena, dKnots, L.knots, stream);
    upload(arena, dGknots, L.gknots, stream);
    upload(arena, dTabJobs, L.tabjobs, stream);
    upload(arena, dGtabJobs, L.gtabjobs, stream);
    upload(arena, dPfJobs, L.pfjobs, stream);
    upload(arena, dIbuf, L.ibuf, stream);
    upload(arena, dWq, L.wq, stream);
    allocN(arena, dTab, L.ntab);
    allocN(arena, dTabDf, L.ntab);
    allocN(arena, dGtab, L.ngtab);
    allocN(arena, dPf, L.npf);
    allocN(arena, dCoefRaw, L.coefs);
    allocN(arena, dCoefs, L.coefs);
    allocN(arena, dFieldC, L.fields);
    allocN(arena, dFieldL, L.lfield);
    allocN(arena, dY1, L.y1);
    allocN(arena, dY2, std::max(1LL, L.y2));
    allocN(arena, dS, L.s);
    allocN(arena, dU, std::max(1LL, L.u));
    allocN(arena, dBand, L.band);
    allocN(arena, dLv1, L.lv1);
    allocN(arena, dLv2, std::max(1LL, L.lv2));
    allocN(arena, dLvec, L.lvec);
    upload(arena, dIndex, map.index, stream);
}

void Context::setCoefs(const double* coefs) {
    if (!refreshed) throw StateError("set_coefs() before refresh()");
    if (device < 0) throw StateError("set_coefs() needs a CUDA device (host-only context)");
    // keep the host copy (Dirichlet values are computed on the host)
    const double* c = coefs;
    for (HostPatch& P : pd.patches) {
        std::copy(c, c + P.coefs.size(), P.coefs.begin());
        c += P.coefs.size();
    }
    GSGPU_CUDA_TRY(cudaMemcpyAsync(dCoefRaw, coefs, size_t(L.coefs) * sizeof(double), cudaMemcpyHostToDevice, stream));
    launch::coefsToSoa(dPatches, tabCoef.d, (long long)tabCoef.h.size(), dCoefRaw, dCoefs, stream);
    assembled = false;
}

void Context::assemble(int precision) {
    if (!refreshed) throw StateError("assemble() before refresh()");
    if (device < 0) throw StateError("assemble() needs a CUDA device (host-only context)");
    cudaStream_t s = stream;
    for (int i = 0; i < 8; ++i)
        if (!ev[i]) GSGPU_CUDA_TRY(cudaEventCreate(&ev[i]));
    GSGPU_CUDA_TRY(cudaEventRecord(ev[0], s));
    // Dirichlet values (gsAssembler::computeDirichletDofsIntpl) are computed on the host while the
    // device runs K1-K3; they are only needed by the rhs lift at the end
    struct HostTask {
        std::thread th;
        std::exception_ptr err;
        ~HostTask() {
            if (th.joinable()) th.join();
        }
    } dir;
    std::vector<double> ddofNew;
    double dirMs = 0.0;
    dir.th = std::thread([&] {
        try {
            auto t0 = std::chrono::steady_clock::now();
            if (ddofFromUser) ddofNew = ddofUser;
            else dirichletValues(pd, map, ddofNew);
            dirMs = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        } catch (...) {
            dir.err = std::current_exception();
        }
    });
    GSGPU_CUDA_TRY(cudaEventRecord(ev[1], s));
    // K1: basis tables and pair factors
    const bool mixed = precision == kMixed;
    if (mixed) ensureMixedBuffers();
    launch::basisTables(dTabJobs, (long long)L.tabjobs.size(), dKnots, dTab, s);
    launch::basisTables(dGtabJobs, (long long)L.gtabjobs.size(), dGknots, dGtab, s);
    // Neumann face values in FP64, from the FP64 geometry table (both precisions)
    launch::neumannFace(dNeuSides, dNeuBlocks, (long long)neu.blocks.size(), dPatches, dFields, dCoefs, dGtab, dIbuf,
                        dWq, dNeuVals, s);
    // the df32 path reuses the FP64 intermediate buffers (same 8-byte element size)
    df32* gtabDf = reinterpret_cast<df32*>(dGtab);
    df32* pfDf = reinterpret_cast<df32*>(dPf);
    if (mixed) {
        launch::toDF(L.ngtab, dGtab, gtabDf, s);  // element-wise in place
        launch::toDF(L.ntab, dTab, dTabDf, s);    // the load contraction's table (dTab stays FP64)
        launch::pairFactors<df32>(dPfJobs, tabPf.d, (long long)tabPf.h.size(), dTab, pfDf, s);
        launch::toDF(L.coefs, dCoefs, dCoefsDf, s);
    } else {
        launch::pairFactors<double>(dPfJobs, tabPf.d, (long long)tabPf.h.size(), dTab, dPf, s);
    }
    GSGPU_CUDA_TRY(cudaEventRecord(ev[2], s));
    // K2: geometry map, Jacobians, coefficient and load fields
    const unsigned long long init = launch::detKeyInit();
    GSGPU_CUDA_TRY(cudaMemcpyAsync(dDetKey, &init, sizeof(init), cudaMemcpyHostToDevice, s));
    df32* y1Df = reinterpret_cast<df32*>(dY1);
    df32* y2Df = reinterpret_cast<df32*>(dY2);
    df32* cDf = reinterpret_cast<df32*>(dFieldC);
    df32* lDf = reinterpret_cast<df32*>(dFieldL);
    df32* sDf = reinterpret_cast<df32*>(dS);
    df32* uDf = reinterpret_cast<df32*>(dU);
    df32* bandDf = reinterpret_cast<df32*>(dBand);
    if (mixed) {
        launch::geoStage1<df32>(dPatches, tabGeo1.d, (long long)tabGeo1.h.size(), dCoefsDf, gtabDf, dIbuf, y1Df, s);
        if (pd.dim == 3)
            launch::geoStage2<df32>(dPatches, tabGeo2.d, (long long)tabGeo2.h.size(), y1Df, gtabDf, dIbuf, y2Df, s);
        launch::pointStep<df32>(dPatches, tabPoint.d, (long long)tabPoint.h.size(), dFieldsDf, y1Df, y2Df, gtabDf,
                                dIbuf, dWqDf, cDf, lDf, dDetKey, fieldKmax, s);
    } else {
        launch::geoStage1<double>(dPatches, tabGeo1.d, (long long)tabGeo1.h.size(), dCoefs, dGtab, dIbuf, dY1, s);
        if (pd.dim == 3)
            launch::geoStage2<double>(dPatches, tabGeo2.d, (long long)tabGeo2.h.size(), dY1, dGtab, dIbuf, dY2, s);
        launch::pointStep<double>(dPatches, tabPoint.d, (long long)tabPoint.h.size(), dFields, dY1, dY2, dGtab, dIbuf,
                                  dWq, dFieldC, dFieldL, dDetKey, fieldKmax, s);
    }
    GSGPU_CUDA_TRY(cudaEventRecord(ev[3], s));
    // K3: sum-factorised stiffness contraction into the band
    if (mixed) {
        // row-blocked df32 contractions (all band offsets of a row function per work item), one
        // launch per degree class along each stage axis. Per degree the variant comes from the
        // tuning table (autotune.cu): 3D stage 1 in shared-memory tiles or rows with 4 or 2 output
        // fields per launch (4: fewer input re-reads, 2: fewer registers, more warps); 3D stage 2
        // rows with 4 or 2 output fields. Every variant forms the same sums in the same order.
        for (int P = 1; P <= 4; ++P) {
            auto nb = [&](int st) { return (long long)tabRow[st][P].h.size(); };
            auto nbB = [&](int st) { return (long long)tabRowB[st][P].h.size(); };
            const int v31 = tuned31[P];
            if (pd.dim == 3 && v31 == kStage31RowsNh2) {
                launch::contractRowDF<31, 0, 2>(P, dPatches, tabRow[0][P].d, nb(0), tabRowB[0][P].d, nbB(0), cDf, sDf, dIbuf, pfDf, s);
                launch::contractRowDF<31, 2, 2>(P, dPatches, tabRow[0][P].d, nb(0), tabRowB[0][P].d, nbB(0), cDf, sDf, dIbuf, pfDf, s);
                launch::contractRowDF<31, 4, 2>(P, dPatches, tabRow[0][P].d, nb(0), tabRowB[0][P].d, nbB(0), cDf, sDf, dIbuf, pfDf, s);
                launch::contractRowDF<31, 6, 2>(P, dPatches, tabRow[0][P].d, nb(0), tabRowB[0][P].d, nbB(0), cDf, sDf, dIbuf, pfDf, s);
            } else if (pd.dim == 3) {
                // interior rows in shared-memory tiles (they cover the same patches as tabRow[0][P]) or
                // the unrolled row kernel; boundary rows always by rows
                const bool tiled = v31 == kStage31Tiles && dev::tiledStage31(P);
                const long long ni = tiled ? 0 : nb(0);
                if (tiled) {
                    // one patch: its row segments per line (the persistent tile kernel's grid stride)
                    int nseg = 0;
                    if (L.dev.size() == 1)
                        nseg = (L.dev[0].n[0] - 2 * P + dev::kTileRows - 1) / dev::kTileRows;
                    launch::stage31Tile(P, dPatches, tabTile31[P].d, (long long)tabTile31[P].h.size(), cDf, sDf, pfDf,
                                        nseg, s);
                }
                if (tiled) {
                    // only the boundary rows remain: two output fields per launch (half the
                    // registers of four, twice the resident warps)
                    launch::contractRowDF<31, 0, 2>(P, dPatches, tabRow[0][P].d, 0, tabRowB[0][P].d, nbB(0), cDf, sDf, dIbuf, pfDf, s);
                    launch::contractRowDF<31, 2, 2>(P, dPatches, tabRow[0][P].d, 0, tabRowB[0][P].d, nbB(0), cDf, sDf, dIbuf, pfDf, s);
                    launch::contractRowDF<31, 4, 2>(P, dPatches, tabRow[0][P].d, 0, tabRowB[0][P].d, nbB(0), cDf, sDf, dIbuf, pfDf, s);
                    launch::contractRowDF<31, 6, 2>(P, dPatches, tabRow[0][P].d, 0, tabRowB[0][P].d, nbB(0), cDf, sDf, dIbuf, pfDf, s);
                } else {
                    launch::contractRowDF<31, 0, 4>(P, dPatches, tabRow[0][P].d, ni, tabRowB[0][P].d, nbB(0), cDf, sDf, dIbuf, pfDf, s);
                    launch::contractRowDF<31, 4, 4>(P, dPatches, tabRow[0][P].d, ni, tabRowB[0][P].d, nbB(0), cDf, sDf, dIbuf, pfDf, s);
                }
            } else {
                launch::contractRowDF<21, 0, 4>(P, dPatches, tabRow[0][P].d, nb(0), tabRowB[0][P].d, nbB(0), cDf, sDf, dIbuf, pfDf, s);
            }
        }
        for (int P = 1; P <= 4; ++P) {
            auto nb = [&](int st) { return (long long)tabRow[st][P].h.size(); };
            auto nbB = [&](int st) { return (long long)tabRowB[st][P].h.size(); };
            if (pd.dim == 3 && tuned32[P] == kStage32RowsNh2) {
                launch::contractRowDF<32, 0, 2>(P, dPatches, tabRow[1][P].d, nb(1), tabRowB[1][P].d, nbB(1), sDf, uDf, dIbuf, pfDf, s);
                launch::contractRowDF<32, 2, 2>(P, dPatches, tabRow[1][P].d, nb(1), tabRowB[1][P].d, nbB(1), sDf, uDf, dIbuf, pfDf, s);
            } else if (pd.dim == 3) {
                launch::contractRowDF<32, 0, 4>(P, dPatches, tabRow[1][P].d, nb(1), tabRowB[1][P].d, nbB(1), sDf, uDf, dIbuf, pfDf, s);
            } else {
                launch::contractRowDF<22, 0, 1>(P, dPatches, tabRow[1][P].d, nb(1), tabRowB[1][P].d, nbB(1), sDf, bandDf, dIbuf, pfDf, s);
            }
        }
        if (pd.dim == 3)
            for (int P = 1; P <= 4; ++P)
                launch::contractRowDF<33, 0, 1>(P, dPatches, tabRow[2][P].d, (long long)tabRow[2][P].h.size(),
                                                tabRowB[2][P].d, (long long)tabRowB[2][P].h.size(), uDf, bandDf, dIbuf,
                                                pfDf, s);
    } else if (pd.dim == 3) {
        launch::contract<double, 31>(dPatches, tabSt[0].d, (long long)tabSt[0].h.size(), dFieldC, dS, dIbuf, dPf, s);
        launch::contract<double, 32>(dPatches, tabSt[1].d, (long long)tabSt[1].h.size(), dS, dU, dIbuf, dPf, s);
        launch::contract<double, 33>(dPatches, tabSt[2].d, (long long)tabSt[2].h.size(), dU, dBand, dIbuf, dPf, s);
    } else {
        launch::contract<double, 21>(dPatches, tabSt[0].d, (long long)tabSt[0].h.size(), dFieldC, dS, dIbuf, dPf, s);
        launch::contract<double, 22>(dPatches, tabSt[1].d, (long long)tabSt[1].h.size(), dS, dBand, dIbuf, dPf, s);
    }
    GSGPU_CUDA_TRY(cudaEventRecord(ev[4], s));
    // load vector (first stage: compensated df32 sums of the df32 load field on the mixed path;
    // FP64 contraction otherwise and for the later stages)
    if (pd.dim == 3) {
        if (mixed)
            launch::loadContractDF<31>(dPatches, tabLd[0].d, (long long)tabLd[0].h.size(), lDf, dLv1, dTabDf, dIbuf, s);
        else
            launch::loadContract<31, double>(dPatches, tabLd[0].d, (long long)tabLd[0].h.size(), dFieldL, dLv1, dTab, dIbuf, s);
        launch::loadContract<32, double>(dPatches, tabLd[1].d, (long long)tabLd[1].h.size(), dLv1, dLv2, dTab, dIbuf, s);
        launch::loadContract<33, double>(dPatches, tabLd[2].d, (long long)tabLd[2].h.size(), dLv2, dLvec, dTab, dIbuf, s);
    } else {
        if (mixed)
            launch::loadContractDF<21>(dPatches, tabLd[0].d, (long long)tabLd[0].h.size(), lDf, dLv1, dTabDf, dIbuf, s);
        else
            launch::loadContract<21, double>(dPatches, tabLd[0].d, (long long)tabLd[0].h.size(), dFieldL, dLv1, dTab, dIbuf, s);
        launch::loadContract<22, double>(dPatches, tabLd[1].d, (long long)tabLd[1].h.size(), dLv1, dLvec, dTab, dIbuf, s);
    }
    // Neumann integrals into the load vector of the dofs on Neumann sides
    launch::neumannDofs(dNeuDofs, (long long)neu.dofs.size(), dNeuSides, dPatches, dTab, dIbuf, dNeuVals, dLvec, s);
    GSGPU_CUDA_TRY(cudaEventRecord(ev[5], s));
    // K4: CSR values (segmented gather) and rhs with the Dirichlet lift
    dir.th.join();
    if (dir.err) std::rethrow_exception(dir.err);
    ddof.swap(ddofNew);
    hostDirichletMs = dirMs;
    if (!ddof.empty())
        GSGPU_CUDA_TRY(cudaMemcpyAsync(dDdof, ddof.data(), ddof.size() * sizeof(double), cudaMemcpyHostToDevice, s));
    if (mixed) {
        launch::gatherCsrDF(nnz, dSrc, bandDf, dOvfPtr, dOvfIdx, dValHi, dValLo, s);
        if (sdiaOk) launch::sdiaBuild(sdiaOp, sdiaBand, bandDf, dSdia, s);
        if (segSdiaOk) {
            if (!dSegSdia) allocN(arena, dSegSdia, segSdiaSize);
            launch::segSdiaBuild(pat.n, dRowSeg, dSegSdiaDesc, bandDf, dSegSdia, s);
        }
        launch::rhsRows<df32>(pat.n, dLvec, dLptr, dLidx, bandDf, dFptr, dFband, dFbidx, dDdof, dRhs, s);
    } else {
        launch::gatherCsr<double>(nnz, dSrc, dBand, dOvfPtr, dOvfIdx, dVal, s);
        launch::rhsRows<double>(pat.n, dLvec, dLptr, dLidx, dBand, dFptr, dFband, dFbidx, dDdof, dRhs, s);
    }
    GSGPU_CUDA_TRY(cudaEventRecord(ev[6], s));
    GSGPU_CUDA_TRY(cudaGetLastError());
    GSGPU_CUDA_TRY(cudaEventSynchronize(ev[6]));
    unsigned long long key = 0;
    GSGPU_CUDA_TRY(cudaMemcpyAsync(&key, dDetKey, sizeof(key), cudaMemcpyDeviceToHost, s));
    GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
    detMin = launch::detKeyDecode(key);
    assembled = true;
    solved = false;
    assembledPrecision = precision;
    ++assembleSerial;
    if (!(detMin > 0.0)) throw JacobianError("geometry map has det J <= 0 at a quadrature point");
}

// gsGenericAssembler::assembleMass (gsGenericAssembler.h:103): M_ij = int phi_i phi_j |det J| on
// the free dofs, in FP64, by the stiffness path's kernels with one field (w |det J|) and the
// value-value pair factors: basis tables, geometry stages, the field, three (two) sum-factorised
// contractions into the band and the gather over the same slot -> band map into the CSR pattern
// of matrix(). It reuses the assembly's intermediate buffers (the stiffness CSR values, rhs and
// solver state are untouched); the next assemble() recomputes them.
void Context::assembleMass() {
    if (!refreshed) throw StateError("mass() before refresh()");
    if (device < 0) throw StateError("mass() needs a CUDA device (host-only context)");
    cudaStream_t s = stream;
    if (!dMass) allocN(arena, dMass, nnz);
    launch::basisTables(dTabJobs, (long long)L.tabjobs.size(), dKnots, dTab, s);
    launch::basisTables(dGtabJobs, (long long)L.gtabjobs.size(), dGknots, dGtab, s);
    launch::pairFactors<double>(dPfJobs, tabPf.d, (long long)tabPf.h.size(), dTab, dPf, s);
    launch::geoStage1<double>(dPatches, tabGeo1.d, (long long)tabGeo1.h.size(), dCoefs, dGtab, dIbuf, dY1, s);
    if (pd.dim == 3) launch::geoStage2<double>(dPatches, tabGeo2.d, (long long)tabGeo2.h.size(), dY1, dGtab, dIbuf, dY2, s);
    launch::massField(dPatches, tabPoint.d, (long long)tabPoint.h.size(), dY1, dY2, dGtab, dIbuf, dWq, dFieldL, s);
    if (pd.dim == 3) {
        launch::contract<double, 41>(dPatches, tabSt[0].d, (long long)tabSt[0].h.size(), dFieldL, dS, dIbuf, dPf, s);
        launch::contract<double, 42>(dPatches, tabSt[1].d, (long long)tabSt[1].h.size(), dS, dU, dIbuf, dPf, s);
        launch::contract<double, 43>(dPatches, tabSt[2].d, (long long)tabSt[2].h.size(), dU, dBand, dIbuf, dPf, s);
    } else {
        launch::contract<double, 51>(dPatches, tabSt[0].d, (long long)tabSt[0].h.size(), dFieldL, dS, dIbuf, dPf, s);
        launch::contract<double, 52>(dPatches, tabSt[1].d, (long long)tabSt[1].h.size(), dS, dBand, dIbuf, dPf, s);
    }
    launch::gatherCsr<double>(nnz, dSrc, dBand, dOvfPtr, dOvfIdx, dMass, s);
    GSGPU_CUDA_TRY(cudaGetLastError());
    GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
    assembled = false;  // the intermediate buffers now hold the mass matrix's
    solved = false;
}

// y = K x with the assembled FP64 matrix (the CG SpMV kernel); x, y on the host
void Context::applyMatrix(const double* x, double* y) {
    if (!assembled || assembledPrecision != kFP64) throw StateError("apply() needs assemble(GSGPU_PREC_FP64)");
    ensureSolveBuffers();
    cudaStream_t s = stream;
    GSGPU_CUDA_TRY(cudaMemcpyAsync(dP, x, sizeof(double) * size_t(pat.n), cudaMemcpyHostToDevice, s));
    GSGPU_CUDA_TRY(cudaMemsetAsync(dCg, 0, sizeof(CgState), s));  // a running state: the kernel is not skipped
    CgBuffers B;
    B.n = pat.n;
    B.lanes_per_row = lanesPerRow(true);
    B.ptr = dPtr;
    B.col = dCol;
    B.coff = dColOff;
    B.val = dVal;
    B.p = dP;
    B.t = dT;
    B.part2 = dPart2;
    B.st = dCg;
    launch::cgSpmv(B, s);
    GSGPU_CUDA_TRY(cudaMemcpyAsync(y, dT, sizeof(double) * size_t(pat.n), cudaMemcpyDeviceToHost, s));
    GSGPU_CUDA_TRY(cudaGetLastError());
    GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
    solved = false;  // the CG state was overwritten
}

// gsField::distanceL2 of the last solution: the geometry stages are re-run in FP64 (after a
// mixed-precision assembly their buffers hold double-float values), then one quadrature kernel
// gsField::distanceL2 / distanceH1 integrate with their evaluator's default rule, p + 1 Gauss points
// per direction, whatever rule the assembler uses (gsNorm.h, the visitor's default quadrature).
// With the default assembly rule (quA = 1, quB = 1) that is the assembly grid, whose tables and
// geometry buffers are reused; otherwise the norm grid gets its own layout and temporary buffers.
std::vector<double> Context::l2PerPatch(bool h1) {
    if (!solved) throw StateError("l2_error() before solve()");
    cudaStream_t s = stream;
    const bool own = !(pd.quA == 1.0 && pd.quB == 1);
    Layout Ln;
    if (own) {
        ProblemDesc pn = pd;
        pn.quA = 1.0;
        pn.quB = 1;
        buildLayout(pn, Ln);
    }
    const Layout& N = own ? Ln : L;
    // the norm grid's device data: the assembly's when the rules agree, else temporaries
    DevPatch* dP = dPatches;
    TabJob *dTJ = dTabJobs, *dGJ = dGtabJobs;
    int* dIb = dIbuf;
    double *dW = dWq, *dT = dTab, *dG = dGtab, *dYa = dY1, *dYb = dY2, *dKn = dKnots, *dGk = dGknots;
    Tab tG1, tG2, tP;
    const Tab *pG1 = &tabGeo1, *pG2 = &tabGeo2, *pP = &tabPoint;
    if (own) {
        dP = nullptr, dTJ = dGJ = nullptr, dIb = nullptr, dW = dT = dG = dYa = dYb = dKn = dGk = nullptr;
        upload(arena, dP, N.dev, s);
        upload(arena, dTJ, N.tabjobs, s);
        upload(arena, dGJ, N.gtabjobs, s);
        upload(arena, dIb, N.ibuf, s);
        upload(arena, dW, N.wq, s);
        upload(arena, dKn, N.knots, s);
        upload(arena, dGk, N.gknots, s);
        allocN(arena, dT, N.ntab);
        allocN(arena, dG, N.ngtab);
        allocN(arena, dYa, N.y1);
        allocN(arena, dYb, std::max(1LL, N.y2));
        auto mk = [&](Tab& T, auto workfn) {
            std::vector<long long> w;
            for (const DevPatch& D : N.dev) w.push_back(workfn(D));
            blockTable(w, launch::kBlock, T.h);
            upload(arena, T.d, T.h, s);
        };
        mk(tG1, [](const DevPatch& D) {
            return D.dim == 3 ? (long long)D.dim * 2 * D.gn[2] * D.gn[1] * D.Q[0] : (long long)D.dim * 2 * D.gn[1] * D.Q[0];
        });
        mk(tG2, [](const DevPatch& D) { return D.dim == 3 ? (long long)D.dim * 3 * D.gn[2] * D.Q[1] * D.Q[0] : 0LL; });
        mk(tP, [](const DevPatch& D) { return D.nq; });
        pG1 = &tG1, pG2 = &tG2, pP = &tP;
    }
    // (after a mixed assembly the assembly's geometry table holds double-float values: rebuilt in FP64)
    launch::basisTables(dGJ, (long long)N.gtabjobs.size(), dGk, dG, s);
    launch::basisTables(dTJ, (long long)N.tabjobs.size(), dKn, dT, s);
    launch::geoStage1<double>(dP, pG1->d, (long long)pG1->h.size(), dCoefs, dG, dIb, dYa, s);
    if (pd.dim == 3) launch::geoStage2<double>(dP, pG2->d, (long long)pG2->h.size(), dYa, dG, dIb, dYb, s);
    const long long nlocal = (long long)map.index.size();
    const long long nblk = (long long)pP->h.size();
    double* coef = nullptr;
    double* part = nullptr;
    allocN(arena, coef, nlocal);
    allocN(arena, part, nblk);
    launch::solutionCoefs(nlocal, dIndex, map.freeSize, dX, dDdof, coef, s);
    launch::l2Partials(dP, pP->d, nblk, dFields, dYa, dYb, dG, dIb, dW, dT, coef, part, h1, s);
    std::vector<double> h(nblk);
    GSGPU_CUDA_TRY(cudaGetLastError());
    GSGPU_CUDA_TRY(cudaMemcpyAsync(h.data(), part, nblk * sizeof(double), cudaMemcpyDeviceToHost, s));
    GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
    arena.release(coef);
    arena.release(part);
    if (own) {
        for (void* p : {(void*)dP, (void*)dTJ, (void*)dGJ, (void*)dIb, (void*)dW, (void*)dKn, (void*)dGk, (void*)dT,
                        (void*)dG, (void*)dYa, (void*)dYb, (void*)tG1.d, (void*)tG2.d, (void*)tP.d})
            arena.release(p);
    }
    // per patch, in block order (the blocks of a patch are contiguous in the table)
    std::vector<double> acc(pd.patches.size(), 0.0);
    for (long long b = 0; b < nblk; ++b) acc[size_t(pP->h[size_t(b)].patch)] += h[size_t(b)];
    return acc;
}

double Context::l2Error(bool h1) {
    double acc = 0.0;
    for (double v : l2PerPatch(h1)) acc += v;
    return std::sqrt(acc);
}

void Context::times(double* ms) {
    float t[6];
    for (int i = 0; i < 6; ++i) GSGPU_CUDA_TRY(cudaEventElapsedTime(&t[i], ev[i], ev[i + 1]));
    ms[0] = hostDirichletMs;
    for (int i = 1; i < 6; ++i) ms[i] = t[i];
    float tot;
    GSGPU_CUDA_TRY(cudaEventElapsedTime(&tot, ev[0], ev[6]));
    ms[6] = tot;
}

void Context::dropGraphs() {
    if (gexecFp64) cudaGraphExecDestroy(gexecFp64);
    if (gexecMixed) cudaGraphExecDestroy(gexecMixed);
    if (gexecMg) cudaGraphExecDestroy(gexecMg);
    for (cudaGraphExec_t& g : gexecSeg)
        if (g) cudaGraphExecDestroy(g), g = nullptr;
    gexecFp64 = gexecMixed = gexecMg = nullptr;
    gexecMgKey = MgGraphKey();
}

void Context::freeAssembly() {
    dropGraphs();
    arena.releaseAll();
    *this = Context::reset(std::move(*this));
}

Context Context::reset(Context&& c) {
    Context n;
    n.device = c.device;
    n.stream = c.stream;
    for (int i = 0; i < 8; ++i) n.ev[i] = c.ev[i];
    n.pd = std::move(c.pd);
    n.hasProblem = c.hasProblem;
    n.batch = c.batch;
    n.arena.budget = c.arena.budget;
    n.arena.stream = n.stream;
    c.stream = nullptr;
    for (int i = 0; i < 8; ++i) c.ev[i] = nullptr;
    return n;
}

// ---------------------------------------------------------------------------------------------
void Context::ensureSolveBuffers() {
    const int n = pat.n;
    if (solveN == n && dX) return;
    dropGraphs();
    for (double** b : {&dX, &dR, &dZ, &dP, &dT, &dDinv, &dPart0, &dPart1, &dPart2}) arena.release(*b), *b = nullptr;
    arena.release(dCg);
    dCg = nullptr;
    allocN(arena, dX, n);
    allocN(arena, dR, n);
    allocN(arena, dZ, n);
    allocN(arena, dP, n);
    allocN(arena, dT, n);
    allocN(arena, dDinv, n);
    // partials: one per block of the widest grid that writes them (the persistent inner iteration
    // runs up to kMaxSpmvBlocks blocks)
    allocN(arena, dPart0, std::max(launch::cgPartials(n), launch::kMaxSpmvBlocks));
    allocN(arena, dPart1, std::max(launch::cgPartials(n), launch::kMaxSpmvBlocks));
    // SpMV partials: one per SpMV block; the most blocks are launched with 32 lanes per row
    allocN(arena, dPart2, std::max({launch::cgPartials(n), launch::spmvPartials(n, 32), launch::kMaxSpmvBlocks,
                                    sdiaOk ? launch::sdiaPartials(sdiaOp) : 0}));
    dCg = static_cast<CgState*>(arena.alloc(sizeof(CgState)));
    solveN = n;
}

// lanes per CSR row of the SpMV kernels: long rows use 16 lanes for FP32 values (the load rate
// limits) and 8 for FP64 values (fewer FP64 shuffle-adds: the FP64 pipe limits); measured on GB300
int Context::lanesPerRow(bool fp64) const {
    if (const char* e = std::getenv("GSGPU_LANES_PER_ROW")) {  // tuning override: 4, 8, 16 or 32
        const int v = std::atoi(e);
        if (v == 4 || v == 8 || v == 16 || v == 32) return v;
    }
    const double avg = pat.n ? double(nnz) / pat.n : 1.0;
    if (avg > 48) return fp64 ? 8 : 16;
    if (avg > 20) return fp64 ? 8 : 16;
    if (avg > 10) return 8;
    return 4;
}

void Context::solve(const gsgpu_solver_opts& o, gsgpu_solve_info& info) {
    if (!assembled) throw StateError("solve() before assemble()");
    if (batch) {
        solveBatch(o, info);
        return;
    }
    if (o.method == GSGPU_SOLVER_CG_MG) {
        if (o.precision == GSGPU_PREC_MIXED && assembledPrecision != kMixed)
            throw StateError("mixed-precision solve needs assemble(GSGPU_PREC_MIXED)");
        if (o.precision == GSGPU_PREC_FP64 && assembledPrecision != kFP64)
            throw StateError("FP64 solve needs assemble(GSGPU_PREC_FP64)");
        if (o.precision != GSGPU_PREC_MIXED && o.precision != GSGPU_PREC_FP64)
            throw std::invalid_argument("unknown precision mode");
        solveMG(o, info);
        return;
    }
    if (o.method != GSGPU_SOLVER_CG_JACOBI) throw std::invalid_argument("unknown solver method");
    if (o.precision == GSGPU_PREC_MIXED) {
        if (assembledPrecision != kMixed) throw StateError("mixed-precision solve needs assemble(GSGPU_PREC_MIXED)");
        solveMixed(o, info);
        return;
    }
    if (o.precision != GSGPU_PREC_FP64) throw std::invalid_argument("unknown precision mode");
    if (assembledPrecision != kFP64) throw StateError("FP64 solve needs assemble(GSGPU_PREC_FP64)");
    ensureSolveBuffers();
    cudaStream_t s = stream;
    cudaEvent_t e0, e1;
    GSGPU_CUDA_TRY(cudaEventCreate(&e0));
    GSGPU_CUDA_TRY(cudaEventCreate(&e1));
    GSGPU_CUDA_TRY(cudaEventRecord(e0, s));
    launch::jacobiDiag(pat.n, dDiag, dVal, 1.0, dDinv, s);
    CgBuffers B;
    B.n = pat.n;
    B.lanes_per_row = lanesPerRow(true);
    B.ptr = dPtr;
    B.col = dCol;
    B.coff = dColOff;
    // no box rows for FP64 values: measured slower on GB300 (C2: 73.6 vs 70.1 ms per step), the
    // FP64 SpMV is not limited by its column-offset bytes
    B.val = dVal;
    B.b = dRhs;
    B.dinv = dDinv;
    B.x = dX; B.r = dR; B.z = dZ; B.p = dP; B.t = dT;
    B.part0 = dPart0; B.part1 = dPart1; B.part2 = dPart2;
    B.st = dCg;
    const double tol = o.tol > 0 ? o.tol : 1e-10;
    const int maxit = o.max_iters > 0 ? o.max_iters : 1000;
    launch::cgInit(B, tol, maxit, s);
    CgState hs{};
    spmvBytes = double(nnz) * (8 + (dColOff ? 2 : 4)) + double(pat.n + 1) * 4 + 2.0 * pat.n * 8;
    if (profiling) {
        // one iteration at a time, every SpMV bracketed by events (no graph)
        cudaEvent_t a, b;
        GSGPU_CUDA_TRY(cudaEventCreate(&a));
        GSGPU_CUDA_TRY(cudaEventCreate(&b));
        GSGPU_CUDA_TRY(cudaMemcpyAsync(&hs, dCg, sizeof(CgState), cudaMemcpyDeviceToHost, s));
        GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
        for (int it = 0; it < maxit && !hs.done; ++it) {
            GSGPU_CUDA_TRY(cudaEventRecord(a, s));
            launch::cgSpmv(B, s);
            GSGPU_CUDA_TRY(cudaEventRecord(b, s));
            launch::cgRest(B, s);
            GSGPU_CUDA_TRY(cudaMemcpyAsync(&hs, dCg, sizeof(CgState), cudaMemcpyDeviceToHost, s));
            GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
            float m = 0;
            GSGPU_CUDA_TRY(cudaEventElapsedTime(&m, a, b));
            spmvMs += m;
            ++spmvLaunches;
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    } else {
        // iterations in chunks captured as a CUDA graph (once per context); kernels become no-ops
        // once converged
        const int chunk = 16;
        if (!gexecFp64 || gexecLpr[0] != B.lanes_per_row) {
            if (gexecFp64) cudaGraphExecDestroy(gexecFp64);
            gexecFp64 = nullptr;
            cudaGraph_t g;
            GSGPU_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            for (int k = 0; k < chunk; ++k) launch::cgIteration(B, s);
            GSGPU_CUDA_TRY(cudaStreamEndCapture(s, &g));
            GSGPU_CUDA_TRY(cudaGraphInstantiate(&gexecFp64, g, 0));
            cudaGraphDestroy(g);
            gexecLpr[0] = B.lanes_per_row;
        }
        cudaGraphExec_t exec = gexecFp64;
        for (int done_it = 0; done_it < maxit + chunk; done_it += chunk) {
            GSGPU_CUDA_TRY(cudaGraphLaunch(exec, s));
            GSGPU_CUDA_TRY(cudaMemcpyAsync(&hs, dCg, sizeof(CgState), cudaMemcpyDeviceToHost, s));
            GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
            if (hs.done) break;
        }
    }
    GSGPU_CUDA_TRY(cudaEventRecord(e1, s));
    GSGPU_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    info.iterations = hs.iters;
    info.relres = hs.relres;
    info.refinements = 0;
    info.t_solve_ms = ms;
    solved = true;
    lastConverged = hs.done == 1;
}

void Context::ensureMixedBuffers() {
    if (dValHi) return;
    dropGraphs();
    const int n = pat.n;
    allocN(arena, dCoefsDf, L.coefs);
    allocN(arena, dValHi, nnz);
    allocN(arena, dValLo, nnz);
    allocN(arena, dDinv32, n);
    allocN(arena, dR32, n);
    allocN(arena, dZ32, n);
    if (sdiaOk) {
        // the half-diagonal product reads x up to sdiaReach entries (plus the 16-float windows of the
        // four-row product) before and after the vector: the direction carries that many zeros on
        // both sides (written once, never overwritten)
        const int pad = (launch::sdiaReach(sdiaOp) + 16 + 63) / 64 * 64;
        allocN(arena, dP32pad, (long long)n + 2LL * pad);
        GSGPU_CUDA_TRY(cudaMemsetAsync(dP32pad, 0, (size_t(n) + 2 * size_t(pad)) * sizeof(float), stream));
        dP32 = dP32pad + pad;
        sdiaOp.xpad = pad;
    } else {
        allocN(arena, dP32, n);
    }
    allocN(arena, dT32, n);
    allocN(arena, dDx32, n);
    allocN(arena, dXhi, n);
    allocN(arena, dXlo, n);
    if (sdiaOk) {
        allocN(arena, dSdia, (long long)sdiaOp.nh * sdiaOp.ns);
        sdiaOp.d = dSdia;
        allocN(arena, dSdiaErr, 1);
        GSGPU_CUDA_TRY(cudaMemsetAsync(dSdiaErr, 0, sizeof(int), stream));
        sdiaOp.err = dSdiaErr;
        setInnerVariant();
    }
}

// the half-diagonal inner product of the tuned variant: TMA-fed (tensor maps of the diagonals and of
// the direction vector), or load-based with one or four rows per thread. False when the variant
// cannot run on these buffers (the one-row load-based product stays; GSGPU_REQUIRE_TMA=1 makes a
// refused TMA map an error, for the tests). The captured solver graph holds the product's launch
// and is dropped.
bool Context::setInnerVariant() {
    if (!sdiaOk || !dSdia) return false;
    if (gexecMixed) cudaGraphExecDestroy(gexecMixed), gexecMixed = nullptr;
    sdiaOp.tmaps = nullptr;
    sdiaOp.group = 1;
    if (tunedInner == kInnerSdiaRows4) {
        // 16-byte loads of the diagonals and of x, 16-byte stores of t
        auto a16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
        if (!a16(dSdia) || !a16(dP32) || !a16(dT32) || sdiaOp.ns % 4 != 0) return false;
        sdiaOp.group = 4;
        return true;
    }
    if (tunedInner != kInnerSdiaTma) return true;
    std::string why;
    if (launch::sdiaTensorMaps(sdiaOp, dP32, sdiaMaps, &why)) {
        sdiaOp.tmaps = sdiaMaps;
        return true;
    }
    if (std::getenv("GSGPU_REQUIRE_TMA")) throw std::runtime_error("TMA half-diagonal product unavailable: " + why);
    return false;
}

void Context::solveMixed(const gsgpu_solver_opts& o, gsgpu_solve_info& info) {
    ensureSolveBuffers();
    ensureMixedBuffers();
    cudaStream_t s = stream;
    cudaEvent_t e0, e1;
    GSGPU_CUDA_TRY(cudaEventCreate(&e0));
    GSGPU_CUDA_TRY(cudaEventCreate(&e1));
    GSGPU_CUDA_TRY(cudaEventRecord(e0, s));
    launch::jacobiDiag32(pat.n, dDiag, dValHi, dDinv32, s);
    CgBuffers B;
    B.n = pat.n;
    B.lanes_per_row = lanesPerRow(false);
    B.ptr = dPtr;
    B.col = dCol;
    B.coff = dColOff;
    B.box = dBoxFlag;
    B.box_off = dBoxOff;
    B.nbox = nBox;
    B.b = dRhs;
    B.x = dX;
    B.r = dR;
    B.part0 = dPart0; B.part1 = dPart1; B.part2 = dPart2;
    B.st = dCg;
    B.val_hi = dValHi; B.val_lo = dValLo; B.dinv32 = dDinv32;
    if (const char* e = std::getenv("GSGPU_MIXED_DELTA")) B.delta = std::atof(e);  // tuning override
    B.r32 = dR32; B.z32 = dZ32; B.p32 = dP32; B.t32 = dT32; B.dx32 = dDx32; B.xhi = dXhi; B.xlo = dXlo;
    if (sdiaOk) B.sdia = sdiaOp;
    {
        auto a16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
        B.vec4 = a16(dDx32) && a16(dR32) && a16(dZ32) && a16(dP32) && a16(dT32) && a16(dDinv32);
        // programmatic dependent launch of the half-diagonal iteration kernels (GSGPU_NO_PDL=1 off)
        B.pdl = B.vec4 && B.sdia.d && B.sdia.group == 4 && !std::getenv("GSGPU_NO_PDL");
        B.sdia.pdl = B.pdl;
    }
    const double tol = o.tol > 0 ? o.tol : 1e-10;
    const int maxit = o.max_iters > 0 ? o.max_iters : 1000;
    launch::mixedInit(B, tol, maxit, s);
    CgState hs{};
    // algorithmic bytes of one inner product: the operator once, x read, t written
    if (sdiaOk) spmvBytes = double(sdiaOp.nh) * pat.n * 4 + 2.0 * pat.n * 4;
    else spmvBytes = double(nnz) * (4 + (dColOff ? 2 : 4)) + double(pat.n + 1) * 4 + 2.0 * pat.n * 4 - boxSavedBytes();
    const int chunk = 16;
    if (profiling) {
        cudaEvent_t a, b;
        GSGPU_CUDA_TRY(cudaEventCreate(&a));
        GSGPU_CUDA_TRY(cudaEventCreate(&b));
        for (int c = 0; c < maxit / chunk + 2; ++c) {
            for (int k = 0; k < chunk; ++k) {
                GSGPU_CUDA_TRY(cudaMemcpyAsync(&hs, dCg, sizeof(CgState), cudaMemcpyDeviceToHost, s));
                GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
                if (hs.done || hs.pause) break;
                GSGPU_CUDA_TRY(cudaEventRecord(a, s));
                launch::mixedSpmv(B, s);
                GSGPU_CUDA_TRY(cudaEventRecord(b, s));
                launch::mixedRest(B, s);
                GSGPU_CUDA_TRY(cudaEventSynchronize(b));
                float m = 0;
                GSGPU_CUDA_TRY(cudaEventElapsedTime(&m, a, b));
                spmvMs += m;
                ++spmvLaunches;
            }
            launch::mixedReplace(B, s);
            GSGPU_CUDA_TRY(cudaMemcpyAsync(&hs, dCg, sizeof(CgState), cudaMemcpyDeviceToHost, s));
            GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
            if (hs.done) break;
        }
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    } else {
        // chunks of FP32 iterations followed by one residual replacement, captured as a graph
        // (once per context)
        const int graphKey = B.lanes_per_row;
        if (!gexecMixed || gexecLpr[1] != graphKey) {
            if (gexecMixed) cudaGraphExecDestroy(gexecMixed);
            gexecMixed = nullptr;
            cudaGraph_t g;
            GSGPU_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
            for (int k = 0; k < chunk; ++k) launch::mixedIteration(B, s);
            launch::mixedReplace(B, s);
            GSGPU_CUDA_TRY(cudaStreamEndCapture(s, &g));
            GSGPU_CUDA_TRY(cudaGraphInstantiate(&gexecMixed, g, 0));
            cudaGraphDestroy(g);
            gexecLpr[1] = graphKey;
        }
        cudaGraphExec_t exec = gexecMixed;
        for (int c = 0; c < maxit / chunk + 2; ++c) {
            GSGPU_CUDA_TRY(cudaGraphLaunch(exec, s));
            GSGPU_CUDA_TRY(cudaMemcpyAsync(&hs, dCg, sizeof(CgState), cudaMemcpyDeviceToHost, s));
            GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
            if (hs.done) break;
        }
    }
    GSGPU_CUDA_TRY(cudaEventRecord(e1, s));
    GSGPU_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    info.iterations = hs.iters;
    info.relres = hs.relres;
    info.refinements = hs.replacements;
    info.t_solve_ms = ms;
    if (B.sdia.err) {
        int e = 0;
        GSGPU_CUDA_TRY(cudaMemcpy(&e, B.sdia.err, sizeof(int), cudaMemcpyDeviceToHost));
        if (e) {
            GSGPU_CUDA_TRY(cudaMemset(B.sdia.err, 0, sizeof(int)));
            throw TimeoutError("a bounded wait of the half-diagonal product expired (TMA copies did not complete)");
        }
    }
    solved = true;
    lastConverged = hs.done == 1;
}

}  // namespace gsgpu

// ---------------------------------------------------------------------------------------------
// C ABI

struct gsgpu_context {
    gsgpu::Context c;
    std::string err;
};

namespace {
template <class F>
int guarded(gsgpu_context* ctx, F&& f) {
    if (!ctx) return GSGPU_ERR_INVALID;
    try {
        if (ctx->c.device >= 0) GSGPU_CUDA_TRY(cudaSetDevice(ctx->c.device));
        f();
        ctx->err.clear();
        return GSGPU_OK;
    } catch (const gsgpu::CudaError& e) {
        ctx->err = e.what();
        return GSGPU_ERR_CUDA;
    } catch (const gsgpu::BudgetError& e) {
        ctx->err = e.what();
        return GSGPU_ERR_BUDGET;
    } catch (const gsgpu::StateError& e) {
        ctx->err = e.what();
        return GSGPU_ERR_STATE;
    } catch (const gsgpu::JacobianError& e) {
        ctx->err = e.what();
        return GSGPU_ERR_JACOBIAN;
    } catch (const gsgpu::TimeoutError& e) {
        ctx->err = e.what();
        return GSGPU_ERR_TIMEOUT;
    } catch (const std::invalid_argument& e) {
        ctx->err = e.what();
        return GSGPU_ERR_INVALID;
    } catch (const std::exception& e) {
        ctx->err = e.what();
        return GSGPU_ERR_INVALID;
    }
}
}  // namespace

extern "C" {

int gsgpu_create(gsgpu_context** out, int device) {
    if (!out) return GSGPU_ERR_INVALID;
    *out = nullptr;
    if (device == -1) {  // host-only context: dof map and sparsity pattern, no device work
        gsgpu_context* c = new gsgpu_context();
        c->c.device = -1;
        *out = c;
        return GSGPU_OK;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) return GSGPU_ERR_CUDA;
    if (cudaSetDevice(device) != cudaSuccess) return GSGPU_ERR_CUDA;
    gsgpu_context* c = new gsgpu_context();
    c->c.device = device;
    if (cudaStreamCreateWithFlags(&c->c.stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return GSGPU_ERR_CUDA;
    }
    c->c.arena.stream = c->c.stream;
    // keep freed blocks in the device's pool for the next batch instead of returning them at
    // every synchronisation (a property of this process's pool, not of the GPU)
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = ~0ULL;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    *out = c;
    return GSGPU_OK;
}

int gsgpu_destroy(gsgpu_context* ctx) {
    if (!ctx) return GSGPU_ERR_INVALID;
    if (ctx->c.device < 0) {
        delete ctx;
        return GSGPU_OK;
    }
    cudaSetDevice(ctx->c.device);
    if (ctx->c.stream) cudaStreamSynchronize(ctx->c.stream);
    ctx->c.dropGraphs();
    ctx->c.arena.releaseAll();
    for (int i = 0; i < 8; ++i)
        if (ctx->c.ev[i]) cudaEventDestroy(ctx->c.ev[i]);
    if (ctx->c.stream) cudaStreamDestroy(ctx->c.stream);
    delete ctx;
    return GSGPU_OK;
}

const char* gsgpu_last_error(const gsgpu_context* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int gsgpu_set_problem(gsgpu_context* ctx, const gsgpu_problem* prob) {
    return guarded(ctx, [&] {
        gsgpu::ProblemDesc pd;
        gsgpu::problemFromC(prob, pd);
        if (ctx->c.device >= 0) {
            ctx->c.dropGraphs();
            ctx->c.arena.releaseAll();
        }
        ctx->c = gsgpu::Context::reset(std::move(ctx->c));
        ctx->c.pd = std::move(pd);
        ctx->c.hasProblem = true;
        ctx->c.batch = false;
    });
}

int gsgpu_set_batch(gsgpu_context* ctx, int count, const gsgpu_problem* problems) {
    return guarded(ctx, [&] {
        gsgpu::ProblemDesc pd;
        gsgpu::batchFromC(count, problems, pd);
        if (ctx->c.device >= 0) {
            ctx->c.dropGraphs();
            ctx->c.arena.releaseAll();
        }
        ctx->c = gsgpu::Context::reset(std::move(ctx->c));
        ctx->c.pd = std::move(pd);
        ctx->c.hasProblem = true;
        ctx->c.batch = true;
    });
}

}  // extern "C"

int gsgpu::setBatchDescs(gsgpu_context* ctx, std::vector<gsgpu::ProblemDesc>& items) {
    return guarded(ctx, [&] {
        gsgpu::ProblemDesc pd;
        gsgpu::batchFromDescs(items, pd);
        if (ctx->c.device >= 0) {
            ctx->c.dropGraphs();
            ctx->c.arena.releaseAll();
        }
        ctx->c = gsgpu::Context::reset(std::move(ctx->c));
        ctx->c.pd = std::move(pd);
        ctx->c.hasProblem = true;
        ctx->c.batch = true;
    });
}

// the structure of a batch (what refresh() derives its plan from): per problem the dimension,
// quadrature rule, Dirichlet strategy, degrees and knot vectors of both bases, the control-point
// count and the boundary sides; not the control points or the closed-form field constants
std::string gsgpu::batchSignature(const std::vector<gsgpu::ProblemDesc>& items) {
    std::string sig;
    auto put = [&](const void* p, size_t n) { sig.append(static_cast<const char*>(p), n); };
    for (const gsgpu::ProblemDesc& pd : items) {
        put(&pd.dim, sizeof(int));
        put(&pd.quA, sizeof(double));
        put(&pd.quB, sizeof(int));
        put(&pd.dirL2, sizeof(int));
        for (const gsgpu::HostPatch& P : pd.patches) {
            for (int k = 0; k < pd.dim; ++k)
                for (const gsgpu::Basis1D* B : {&P.b[k], &P.g[k]}) {
                    put(&B->p, sizeof(int));
                    const size_t nt = B->t.size();
                    put(&nt, sizeof(nt));
                    put(B->t.data(), nt * sizeof(double));
                }
            const size_t nc = P.coefs.size();
            put(&nc, sizeof(nc));
        }
        for (const std::vector<int>* v : {&pd.dsides, &pd.nsides, &pd.ifaces}) {
            const size_t n = v->size();
            put(&n, sizeof(n));
            put(v->data(), n * sizeof(int));
        }
        put("|", 1);
    }
    return sig;
}

// new control points and field constants for a refreshed batch context whose batch has the
// signature of `items` (the plan, pattern and device buffers stay resident): the next assemble()
// uses them
int gsgpu::updateBatchData(gsgpu_context* ctx, std::vector<gsgpu::ProblemDesc>& items) {
    return guarded(ctx, [&] {
        gsgpu::Context& c = ctx->c;
        if (!c.batch || !c.refreshed || c.device < 0) throw gsgpu::StateError("update of a batch that is not resident");
        if (items.size() != c.pd.patches.size()) throw std::invalid_argument("batch update: problem count differs");
        std::vector<double> raw;
        for (size_t j = 0; j < items.size(); ++j) {
            gsgpu::HostPatch& P = c.pd.patches[j];
            const gsgpu::HostPatch& Q = items[j].patches.at(0);
            if (Q.coefs.size() != P.coefs.size()) throw std::invalid_argument("batch update: control points differ");
            P.coefs = Q.coefs;
            c.pd.pfields.at(j) = items[j].fields;
            raw.insert(raw.end(), P.coefs.begin(), P.coefs.end());
        }
        std::vector<gsgpu::dev::FieldConst<double>> fc64;
        std::vector<gsgpu::dev::FieldConst<gsgpu::df32>> fcdf;
        c.fieldKmax = 0;
        for (const gsgpu::FieldParams& F : c.pd.fieldTable()) {
            fc64.push_back(gsgpu::dev::fieldConst<double>(F));
            fcdf.push_back(gsgpu::dev::fieldConst<gsgpu::df32>(F));
            c.fieldKmax = std::max(c.fieldKmax, F.kmax);
        }
        cudaStream_t s = c.stream;
        GSGPU_CUDA_TRY(cudaMemcpyAsync(c.dFields, fc64.data(), fc64.size() * sizeof(fc64[0]), cudaMemcpyHostToDevice, s));
        GSGPU_CUDA_TRY(cudaMemcpyAsync(c.dFieldsDf, fcdf.data(), fcdf.size() * sizeof(fcdf[0]), cudaMemcpyHostToDevice, s));
        GSGPU_CUDA_TRY(cudaMemcpyAsync(c.dCoefRaw, raw.data(), raw.size() * sizeof(double), cudaMemcpyHostToDevice, s));
        gsgpu::launch::coefsToSoa(c.dPatches, c.tabCoef.d, (long long)c.tabCoef.h.size(), c.dCoefRaw, c.dCoefs, s);
        GSGPU_CUDA_TRY(cudaStreamSynchronize(s));  // the host vectors above go out of scope
        c.assembled = c.solved = false;
    });
}

// device bytes a context holds
double gsgpu::deviceBytes(const gsgpu_context* ctx) { return ctx ? double(ctx->c.arena.used) : 0.0; }

void gsgpu::releaseDevice(gsgpu_context* ctx) {
    if (!ctx || ctx->c.device < 0) return;
    cudaSetDevice(ctx->c.device);
    ctx->c.freeAssembly();
    ctx->c.refreshed = ctx->c.assembled = ctx->c.solved = false;
}

extern "C" {

int gsgpu_batch_info(gsgpu_context* ctx, int* offsets, int* iterations, double* relres) {
    return guarded(ctx, [&] {
        auto& c = ctx->c;
        if (!c.batch) throw gsgpu::StateError("batch_info() on a context without a batch");
        if (!c.refreshed) throw gsgpu::StateError("batch_info() before refresh()");
        if (offsets) std::copy(c.segRow.begin(), c.segRow.end(), offsets);
        if (iterations || relres) {
            if (!c.solved) throw gsgpu::StateError("batch_info() iterations before solve()");
            for (size_t j = 0; j < c.segLast.size(); ++j) {
                if (iterations) iterations[j] = c.segLast[j].total;
                if (relres) relres[j] = c.segLast[j].relres;
            }
        }
    });
}

int gsgpu_batch_l2_error(gsgpu_context* ctx, double* err) {
    if (!err) return GSGPU_ERR_INVALID;
    return guarded(ctx, [&] {
        if (!ctx->c.batch) throw gsgpu::StateError("batch_l2_error() on a context without a batch");
        const std::vector<double> sq = ctx->c.l2PerPatch();
        for (size_t j = 0; j < sq.size(); ++j) err[j] = std::sqrt(sq[j]);
    });
}

int gsgpu_batch_h1_error(gsgpu_context* ctx, double* err) {
    if (!err) return GSGPU_ERR_INVALID;
    return guarded(ctx, [&] {
        if (!ctx->c.batch) throw gsgpu::StateError("batch_h1_error() on a context without a batch");
        const std::vector<double> sq = ctx->c.l2PerPatch(true);
        for (size_t j = 0; j < sq.size(); ++j) err[j] = std::sqrt(sq[j]);
    });
}

int gsgpu_refresh(gsgpu_context* ctx) { return guarded(ctx, [&] { ctx->c.refresh(); }); }

int gsgpu_set_coefs(gsgpu_context* ctx, const double* coefs) {
    return guarded(ctx, [&] {
        if (!coefs) throw std::invalid_argument("null coefs");
        ctx->c.setCoefs(coefs);
    });
}

int gsgpu_assemble(gsgpu_context* ctx, int precision) {
    return guarded(ctx, [&] { ctx->c.assemble(precision); });
}

int gsgpu_sizes(gsgpu_context* ctx, int* nfree, long long* nnz, int* nfixed, int* nlocal) {
    return guarded(ctx, [&] {
        if (!ctx->c.refreshed) throw gsgpu::StateError("sizes() before refresh()");
        if (nfree) *nfree = ctx->c.pat.n;
        if (nnz) *nnz = ctx->c.nnz;
        if (nfixed) *nfixed = ctx->c.map.boundarySize;
        if (nlocal) *nlocal = ctx->c.map.nlocal;
    });
}

int gsgpu_matrix_csr(gsgpu_context* ctx, int* ptr, int* col, double* val) {
    return guarded(ctx, [&] {
        auto& c = ctx->c;
        if (!c.refreshed) throw gsgpu::StateError("matrix() before refresh()");
        if (val && !c.assembled) throw gsgpu::StateError("matrix() values before assemble()");
        if (c.devPattern) {  // the pattern lives on the device only
            if (ptr)
                GSGPU_CUDA_TRY(cudaMemcpyAsync(ptr, c.dPtr, size_t(c.pat.n + 1) * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
            if (col && c.nnz)
                GSGPU_CUDA_TRY(cudaMemcpyAsync(col, c.dCol, size_t(c.nnz) * sizeof(int), cudaMemcpyDeviceToHost, c.stream));
            GSGPU_CUDA_TRY(cudaStreamSynchronize(c.stream));
        } else {
            if (ptr) std::copy(c.pat.ptr.begin(), c.pat.ptr.end(), ptr);
            if (col) std::copy(c.pat.col.begin(), c.pat.col.end(), col);
        }
        if (val && c.assembledPrecision == gsgpu::kMixed) {  // the df32 operator as FP64 values hi + lo
            std::vector<float> hi(size_t(c.nnz)), lo(size_t(c.nnz));
            GSGPU_CUDA_TRY(cudaMemcpyAsync(hi.data(), c.dValHi, hi.size() * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
            GSGPU_CUDA_TRY(cudaMemcpyAsync(lo.data(), c.dValLo, lo.size() * sizeof(float), cudaMemcpyDeviceToHost, c.stream));
            GSGPU_CUDA_TRY(cudaStreamSynchronize(c.stream));
            for (size_t k = 0; k < hi.size(); ++k) val[k] = double(hi[k]) + double(lo[k]);
        } else if (val) {
            GSGPU_CUDA_TRY(cudaMemcpyAsync(val, c.dVal, size_t(c.nnz) * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
            GSGPU_CUDA_TRY(cudaStreamSynchronize(c.stream));
        }
    });
}

int gsgpu_rhs(gsgpu_context* ctx, double* rhs) {
    return guarded(ctx, [&] {
        auto& c = ctx->c;
        if (!c.assembled) throw gsgpu::StateError("rhs() before assemble()");
        GSGPU_CUDA_TRY(cudaMemcpyAsync(rhs, c.dRhs, size_t(c.pat.n) * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        GSGPU_CUDA_TRY(cudaStreamSynchronize(c.stream));
    });
}

int gsgpu_fixed_dofs(gsgpu_context* ctx, double* ddof) {
    return guarded(ctx, [&] {
        auto& c = ctx->c;
        if (c.device < 0 && c.refreshed) {  // host-only context: the values of the problem's strategy
            std::vector<double> v;
            gsgpu::dirichletValues(c.pd, c.map, v);
            std::copy(v.begin(), v.end(), ddof);
            return;
        }
        if (!c.assembled) throw gsgpu::StateError("fixedDofs() before assemble()");
        std::copy(c.ddof.begin(), c.ddof.end(), ddof);
    });
}

int gsgpu_set_fixed_dofs(gsgpu_context* ctx, const double* ddof, int n) {
    return guarded(ctx, [&] {
        auto& c = ctx->c;
        if (!c.refreshed) throw gsgpu::StateError("set_fixed_dofs() before refresh()");
        if (!ddof) {
            c.ddofUser.clear();
            c.ddofFromUser = false;
            return;
        }
        if (n != c.map.boundarySize)
            throw std::invalid_argument("set_fixed_dofs(): " + std::to_string(n) + " values for " +
                                        std::to_string(c.map.boundarySize) + " eliminated dofs");
        c.ddofUser.assign(ddof, ddof + n);
        c.ddofFromUser = true;
    });
}

int gsgpu_dof_map(gsgpu_context* ctx, int* index) {
    return guarded(ctx, [&] {
        auto& c = ctx->c;
        if (!c.refreshed) throw gsgpu::StateError("dof map before refresh()");
        std::copy(c.map.index.begin(), c.map.index.end(), index);
    });
}

int gsgpu_solve(gsgpu_context* ctx, const gsgpu_solver_opts* opts, double* x, gsgpu_solve_info* info) {
    if (!opts) return GSGPU_ERR_INVALID;
    gsgpu_solve_info tmp{};
    const int rc = guarded(ctx, [&] {
        ctx->c.solve(*opts, tmp);
        if (x) {  // on the context's stream, so that caller-side events on it bracket the copy
            GSGPU_CUDA_TRY(cudaMemcpyAsync(x, ctx->c.dX, size_t(ctx->c.pat.n) * sizeof(double), cudaMemcpyDeviceToHost,
                                           ctx->c.stream));
            GSGPU_CUDA_TRY(cudaStreamSynchronize(ctx->c.stream));
        }
    });
    if (info) *info = tmp;
    if (rc == GSGPU_OK && !ctx->c.lastConverged) {
        ctx->err = "maximum number of iterations reached";
        return GSGPU_ERR_NOT_CONVERGED;
    }
    return rc;
}

int gsgpu_apply(gsgpu_context* ctx, const double* x, double* y) {
    if (!x || !y) return GSGPU_ERR_INVALID;
    return guarded(ctx, [&] {
        if (ctx->c.batch) throw std::invalid_argument("apply() is not available for batches");
        ctx->c.applyMatrix(x, y);
    });
}

int gsgpu_mg_apply(gsgpu_context* ctx, const gsgpu_solver_opts* opts, const double* r, double* z) {
    if (!opts || !r || !z) return GSGPU_ERR_INVALID;
    return guarded(ctx, [&] {
        if (ctx->c.batch) throw std::invalid_argument("mg_apply() is not available for batches");
        ctx->c.mgApply(*opts, r, z);
    });
}

int gsgpu_l2_error(gsgpu_context* ctx, double* err) {
    if (!err) return GSGPU_ERR_INVALID;
    return guarded(ctx, [&] { *err = ctx->c.l2Error(false); });
}

int gsgpu_h1_error(gsgpu_context* ctx, double* err) {
    if (!err) return GSGPU_ERR_INVALID;
    return guarded(ctx, [&] { *err = ctx->c.l2Error(true); });
}

int gsgpu_stream(gsgpu_context* ctx, void** stream) {
    return guarded(ctx, [&] { *stream = (void*)ctx->c.stream; });
}

int gsgpu_set_profiling(gsgpu_context* ctx, int on) {
    return guarded(ctx, [&] {
        ctx->c.profiling = on != 0;
        ctx->c.spmvLaunches = 0;
        ctx->c.spmvMs = 0.0;
    });
}

int gsgpu_spmv_stats(gsgpu_context* ctx, long long* launches, double* total_ms, double* bytes_per_launch) {
    return guarded(ctx, [&] {
        if (launches) *launches = ctx->c.spmvLaunches;
        if (total_ms) *total_ms = ctx->c.spmvMs;
        if (bytes_per_launch) *bytes_per_launch = ctx->c.spmvBytes;
    });
}

int gsgpu_mass_csr(gsgpu_context* ctx, double* val) {
    return guarded(ctx, [&] {
        ctx->c.assembleMass();
        if (val && ctx->c.nnz > 0)
            GSGPU_CUDA_TRY(cudaMemcpy(val, ctx->c.dMass, size_t(ctx->c.nnz) * sizeof(double), cudaMemcpyDeviceToHost));
    });
}

int gsgpu_eval_fields(const gsgpu_problem* prob, int npts, const double* x, double* kappa, double* f, double* u) {
    if (!prob || npts < 0 || (npts > 0 && !x)) return GSGPU_ERR_INVALID;
    try {
        gsgpu::ProblemDesc pd;
        gsgpu::problemFromC(prob, pd);
        const int d = pd.dim;
        for (int i = 0; i < npts; ++i) {
            double k = 0, ff = 0, uu = 0;
            gsgpu::evalFields(pd.fields, x + size_t(i) * d, k, ff, uu);
            if (kappa) kappa[i] = k;
            if (f) f[i] = ff;
            if (u) u[i] = uu;
        }
    } catch (...) {
        return GSGPU_ERR_INVALID;
    }
    return GSGPU_OK;
}

int gsgpu_autotune(gsgpu_context* ctx, double* ms9) {
    return guarded(ctx, [&] { ctx->c.autotune(ms9); });
}

int gsgpu_tuned_variants(gsgpu_context* ctx, int* v3) {
    return guarded(ctx, [&] {
        if (!v3) throw std::invalid_argument("tuned_variants: null output");
        if (!ctx->c.refreshed) throw gsgpu::StateError("tuned_variants() before refresh()");
        const gsgpu::DevPatch& D = ctx->c.L.dev.at(0);
        v3[0] = ctx->c.tuned31[std::min(4, std::max(1, D.p[0]))];
        v3[1] = ctx->c.tuned32[std::min(4, std::max(1, D.p[1]))];
        v3[2] = ctx->c.sdiaOk ? ctx->c.tunedInner : -1;
    });
}

int gsgpu_tune_save(const char* path) { return path && gsgpu::tuneSave(path) ? GSGPU_OK : GSGPU_ERR_INVALID; }
int gsgpu_tune_load(const char* path) { return path && gsgpu::tuneLoad(path) ? GSGPU_OK : GSGPU_ERR_INVALID; }
int gsgpu_tune_clear(void) {
    gsgpu::tuneClear();
    return GSGPU_OK;
}

int gsgpu_min_jacobian(gsgpu_context* ctx, double* detmin) {
    return guarded(ctx, [&] {
        if (!ctx->c.assembled) throw gsgpu::StateError("min_jacobian() before assemble()");
        *detmin = ctx->c.detMin;
    });
}

int gsgpu_assemble_times(gsgpu_context* ctx, double* ms7) {
    return guarded(ctx, [&] {
        if (!ctx->c.assembled) throw gsgpu::StateError("assemble_times() before assemble()");
        ctx->c.times(ms7);
    });
}

}  // extern "C"
