// Batches of independent single-patch problems: segment tables and the segmented solver (one
// gsConjugateGradient with gsJacobiOp per problem, src/gsSolver/gsConjugateGradient.hpp:19-84),
// in FP64 or as an FP32 segmented PCG inside an FP64 iterative refinement.
#include <cuda_runtime.h>

#include <algorithm>
#include <stdexcept>
#include <vector>

#include "context.h"
#include "kernels_batch.h"

namespace gsgpu {

// free-dof rows of each problem: the dof mapper numbers the free dofs patch by patch, so the
// problems' rows are contiguous and in problem order
std::vector<int> segmentRows(const ProblemDesc& pd, const DofMap& map) {
    std::vector<int> seg(pd.patches.size() + 1, 0);
    for (size_t j = 0; j < pd.patches.size(); ++j) {
        const HostPatch& P = pd.patches[j];
        int lo = map.freeSize, hi = -1, cnt = 0;
        for (int i = 0; i < P.ndofs; ++i) {
            const int g = map.index[P.offset + i];
            if (g >= map.freeSize) continue;
            lo = std::min(lo, g);
            hi = std::max(hi, g);
            ++cnt;
        }
        if (cnt && (lo != seg[j] || hi - lo + 1 != cnt))
            throw std::runtime_error("batch: the free dofs of a problem are not contiguous");
        seg[j + 1] = seg[j] + cnt;
    }
    if (seg.back() != map.freeSize) throw std::runtime_error("batch: free dof count mismatch");
    return seg;
}

void Context::batchSetup() {
    const int nseg = int(segRow.size()) - 1;
    std::vector<int> rowSeg(pat.n);
    for (int j = 0; j < nseg; ++j)
        for (int r = segRow[j]; r < segRow[j + 1]; ++r) rowSeg[r] = j;
    upload(arena, dSegRow, segRow, stream);
    upload(arena, dRowSeg, rowSeg, stream);
    allocN(arena, dSegRc0, std::max(1, pat.n));
    allocN(arena, dSegRc1, std::max(1, pat.n));
    allocN(arena, dSegSt, nseg);
    allocN(arena, dSegOuter, nseg);
    allocN(arena, dSegDone, 2);  // [inner done, outer done]
    allocN(arena, dSegXdf, std::max(1, pat.n));
    if (segSdiaOk) upload(arena, dSegSdiaDesc, segSdiaHost, stream);
    // pieces of at most kSegPiece rows, aligned to the start of their segment (so a problem's sums
    // do not depend on the other problems of the batch)
    std::vector<int> pieceRow, pieceSeg, segPiece(nseg + 1, 0);
    for (int j = 0; j < nseg; ++j) {
        segPiece[j] = int(pieceSeg.size());
        for (int r = segRow[j]; r < segRow[j + 1]; r += kSegPiece) {
            pieceRow.push_back(r);
            pieceSeg.push_back(j);
        }
    }
    segPiece[nseg] = int(pieceSeg.size());
    pieceRow.push_back(pat.n);
    nPiece = int(pieceSeg.size());
    upload(arena, dPieceRow, pieceRow, stream);
    upload(arena, dPieceSeg, pieceSeg.empty() ? std::vector<int>(1, 0) : pieceSeg, stream);
    upload(arena, dSegPiece, segPiece, stream);
    allocN(arena, dPiecePart, 2LL * std::max(1, nPiece));
}

// one chunk of 16 iterations as a captured graph (per precision, once per context)
template <typename T>
void Context::segChunk(const SegCg<T>& B, cudaGraphExec_t& exec) {
    cudaStream_t s = stream;
    if (!exec) {
        cudaGraph_t g;
        GSGPU_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        for (int k = 0; k < kSegChunk; ++k) launch::segIteration<T>(B, s);
        GSGPU_CUDA_TRY(cudaStreamEndCapture(s, &g));
        GSGPU_CUDA_TRY(cudaGraphInstantiate(&exec, g, 0));
        cudaGraphDestroy(g);
    }
    GSGPU_CUDA_TRY(cudaGraphLaunch(exec, s));
}

// chunks until every segment is done
template <typename T>
void Context::segRun(const SegCg<T>& B, cudaGraphExec_t& exec, int maxit) {
    cudaStream_t s = stream;
    int ndone = 0;
    GSGPU_CUDA_TRY(cudaMemcpyAsync(&ndone, B.ndone, sizeof(int), cudaMemcpyDeviceToHost, s));
    GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
    for (int it = 0; it < maxit + kSegChunk && ndone < B.nseg; it += kSegChunk) {
        segChunk<T>(B, exec);
        GSGPU_CUDA_TRY(cudaMemcpyAsync(&ndone, B.ndone, sizeof(int), cudaMemcpyDeviceToHost, s));
        GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
    }
}

void Context::solveBatch(const gsgpu_solver_opts& o, gsgpu_solve_info& info) {
    if (o.method != GSGPU_SOLVER_CG_JACOBI) throw std::invalid_argument("batches are solved by Jacobi-PCG");
    const bool mixed = o.precision == GSGPU_PREC_MIXED;
    if (!mixed && o.precision != GSGPU_PREC_FP64) throw std::invalid_argument("unknown precision mode");
    if (mixed && assembledPrecision != kMixed) throw StateError("mixed-precision solve needs assemble(GSGPU_PREC_MIXED)");
    if (!mixed && assembledPrecision != kFP64) throw StateError("FP64 solve needs assemble(GSGPU_PREC_FP64)");
    ensureSolveBuffers();
    if (mixed) ensureMixedBuffers();
    cudaStream_t s = stream;
    const int nseg = int(segRow.size()) - 1;
    const double tol = o.tol > 0 ? o.tol : 1e-10;
    const int maxit = o.max_iters > 0 ? o.max_iters : 1000;
    cudaEvent_t e0, e1;
    GSGPU_CUDA_TRY(cudaEventCreate(&e0));
    GSGPU_CUDA_TRY(cudaEventCreate(&e1));
    GSGPU_CUDA_TRY(cudaEventRecord(e0, s));
    auto common = [&](auto& B) {
        B.n = pat.n;
        B.nseg = nseg;
        B.segRow = dSegRow;
        B.rowSeg = dRowSeg;
        B.ptr = dPtr;
        B.col = dCol;
        B.coff = dColOff;
        B.rc0 = dSegRc0;
        B.rc1 = dSegRc1;
        B.npiece = nPiece;
        B.pieceRow = dPieceRow;
        B.pieceSeg = dPieceSeg;
        B.segPiece = dSegPiece;
        B.pp0 = dPiecePart;
        B.pp1 = dPiecePart + std::max(1, nPiece);
        B.st = dSegSt;
        B.ndone = dSegDone;
    };
    segLast.assign(nseg, SegState{});
    if (!mixed) {
        SegCg<double> B;
        common(B);
        B.val = dVal;
        B.dinv = dDinv;
        B.b = dRhs;
        B.x = dX;
        B.r = dR;
        B.z = dZ;
        B.p = dP;
        B.t = dT;
        launch::segDinv<double>(B, dDiag, s);
        launch::segInit<double>(B, tol, maxit, s);
        segRun<double>(B, gexecSeg[0], maxit);
        GSGPU_CUDA_TRY(cudaMemcpyAsync(segLast.data(), dSegSt, sizeof(SegState) * nseg, cudaMemcpyDeviceToHost, s));
        GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
        for (SegState& S : segLast) S.total = S.iters;
    } else {
        // FP32 segmented CG on hi for the correction d (dDx32) from r32 = fl32(b), each
        // segment's recursion running on; every chunk, x += d, the true residual b - (hi + lo) x
        // decides per segment, and the recursion continues from it with its search direction
        // kept (residual replacement, as in the single-problem mixed CG), instead of restarting
        // CG for every refinement
        SegCg<float> B;
        common(B);
        B.val = dValHi;
        B.dinv = dDinv32;
        B.b = dXhi;
        B.x = dDx32;
        B.r = dR32;
        B.z = dZ32;
        B.p = dP32;
        B.t = dT32;
        B.outer = dSegOuter;
        if (segSdiaOk) {
            B.sdia = dSegSdiaDesc;
            B.sd = dSegSdia;
        }
        SegRefine R;
        R.hi = dValHi;
        R.lo = dValLo;
        R.b = dRhs;
        R.x = dX;
        R.xdf = dSegXdf;
        R.r = dR;
        R.r32 = dXhi;
        R.st = dSegOuter;
        R.ndone = dSegDone + 1;
        const int maxref = maxit + 2;  // chunks: each advances every running segment by one iteration at least
        launch::segDinv<float>(B, dDiag, s);
        launch::refineResidual(B, R, tol, maxref, 1, s);
        launch::refineRhs(B, R, s);
        launch::segInit<float>(B, tol, maxit, s);
        for (int ref = 0; ref < maxref; ++ref) {
            int ndone = 0;
            GSGPU_CUDA_TRY(cudaMemcpyAsync(&ndone, R.ndone, sizeof(int), cudaMemcpyDeviceToHost, s));
            GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
            if (ndone >= nseg) break;
            segChunk<float>(B, gexecSeg[1]);
            launch::refineReplace(B, R, tol, maxref, s);
        }
        launch::refineCount(B, R, s);
        GSGPU_CUDA_TRY(cudaMemcpyAsync(segLast.data(), dSegOuter, sizeof(SegState) * nseg, cudaMemcpyDeviceToHost, s));
        GSGPU_CUDA_TRY(cudaStreamSynchronize(s));
    }
    GSGPU_CUDA_TRY(cudaGetLastError());
    GSGPU_CUDA_TRY(cudaEventRecord(e1, s));
    GSGPU_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    int itmax = 0, ref = 0;
    double rmax = 0.0;
    bool all = true;
    for (const SegState& S : segLast) {
        itmax = std::max(itmax, S.total);
        rmax = std::max(rmax, S.relres);
        ref = std::max(ref, mixed ? S.iters : 0);
        all = all && S.done == 1;
    }
    info.iterations = itmax;
    info.relres = rmax;
    info.refinements = ref;
    info.t_solve_ms = ms;
    solved = true;
    lastConverged = all;
}

}  // namespace gsgpu
