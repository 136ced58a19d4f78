// The state behind one gsgpu_context: host plan, device buffers, streams and events.
#pragma once

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../../include/gsgpu.h"
#include "gsgpu_internal.h"
#include "device_funcs.cuh"
#include "kernels_batch.h"
#include "kernels_mg.h"
#include "kernels_solve.h"
#include "mg_plan.h"
#include "plan.h"
#include "autotune.h"

namespace gsgpu {

struct CudaError : std::runtime_error {
    cudaError_t code;
    CudaError(cudaError_t e, const char* expr, const char* file, int line);
};
struct BudgetError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct StateError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct JacobianError : std::runtime_error {
    using std::runtime_error::runtime_error;
};
struct TimeoutError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// every device allocation of a context goes through here (accounting against a budget)
// device buffers of one context, stream-ordered on the context's stream (cudaMallocAsync /
// cudaFreeAsync from the device's default pool): freeing never synchronises the device, so the
// contexts of a server's slots do not stall each other between batches
struct DeviceArena {
    size_t used = 0;
    size_t budget = 0;  // 0 = unlimited
    cudaStream_t stream = nullptr;  // the owning context's stream (nullptr: plain cudaMalloc / cudaFree)
    std::vector<std::pair<void*, size_t>> sizes;
    void* alloc(size_t bytes);
    void release(void* p);
    void releaseAll();
};

struct Tab {
    std::vector<BlkEnt> h;
    BlkEnt* d = nullptr;
};

template <typename T, typename Alloc>
inline void upload(DeviceArena& A, T*& dptr, const std::vector<T, Alloc>& h, cudaStream_t s) {
    A.release(dptr);
    dptr = static_cast<T*>(A.alloc(h.size() * sizeof(T)));
    if (!h.empty()) GSGPU_CUDA_TRY(cudaMemcpyAsync(dptr, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
}
template <typename T>
inline void allocN(DeviceArena& A, T*& dptr, long long n) {
    A.release(dptr);
    dptr = static_cast<T*>(A.alloc(size_t(n > 0 ? n : 0) * sizeof(T)));
}

// one coarse level of the multigrid hierarchy on the device (level 0 is the assembled system)
struct MgLevelBuf {
    MgLevelPlan plan;
    int lpr64 = 8, lpr32 = 16;
    DevPatch* dPatches = nullptr;
    double *dKnots = nullptr, *dTab = nullptr, *dPf = nullptr;
    TabJob* dTabJobs = nullptr;
    PfJob* dPfJobs = nullptr;
    int* dIbuf = nullptr;
    Tab tabPf, tabSt[3];
    int *dPtr = nullptr, *dCol = nullptr, *dDiag = nullptr;
    int16_t* dColOff = nullptr;
    uint32_t *dSrc = nullptr, *dOvfPtr = nullptr, *dOvfIdx = nullptr;
    int *dPptr = nullptr, *dPcol = nullptr, *dRptr = nullptr, *dRcol = nullptr;
    double *dPval = nullptr, *dRval = nullptr, *dVal = nullptr, *dVec = nullptr;  // dVec: dinv b x r z p t
    float *dPval32 = nullptr, *dRval32 = nullptr, *dVal32 = nullptr, *dVec32 = nullptr;
};

// what a captured multigrid solver graph depends on
struct MgGraphKey {
    int mixed = -1, levels = 0, npre = 0, npost = 0, coarse_iters = 0, cycles = 0;
    double damping = 0.0, coarse_tol = 0.0, cgc = 0.0;
    bool operator==(const MgGraphKey& o) const {
        return mixed == o.mixed && levels == o.levels && npre == o.npre && npost == o.npost &&
               coarse_iters == o.coarse_iters && cycles == o.cycles && damping == o.damping &&
               coarse_tol == o.coarse_tol && cgc == o.cgc;
    }
};

namespace launch {
void coefsToSoa(const DevPatch* P, const BlkEnt* tab, long long nblk, const double* raw, double* soa, cudaStream_t s);
}

// free-dof row offsets of the problems of a batch (one patch per problem)
std::vector<int> segmentRows(const ProblemDesc& pd, const DofMap& map);
// gsgpu_set_batch from validated descriptions (consumed); the request server's entry
int setBatchDescs(gsgpu_context* ctx, std::vector<ProblemDesc>& items);
// free every device buffer of the context (it keeps its stream and problem)
void releaseDevice(gsgpu_context* ctx);
// the structure of a batch of problems (all that refresh() derives the plan from)
std::string batchSignature(const std::vector<ProblemDesc>& items);
// new control points and field constants for a resident batch of the same signature (no refresh)
int updateBatchData(gsgpu_context* ctx, std::vector<ProblemDesc>& items);
double deviceBytes(const gsgpu_context* ctx);

struct Context {
    int device = -1;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[8] = {};
    DeviceArena arena;

    ProblemDesc pd;
    bool hasProblem = false, refreshed = false, assembled = false, solved = false, lastConverged = false;
    int assembledPrecision = 0;
    DofMap map;
    Layout L;
    Pattern pat;
    std::vector<int> diag;
    std::vector<double> ddof;
    double detMin = 0.0, hostDirichletMs = 0.0;

    // device buffers (assembly)
    DevPatch* dPatches = nullptr;
    dev::FieldConst<double>* dFields = nullptr;
    dev::FieldConst<df32>* dFieldsDf = nullptr;
    double *dKnots = nullptr, *dGknots = nullptr, *dTab = nullptr, *dGtab = nullptr, *dPf = nullptr, *dWq = nullptr;
    df32* dTabDf = nullptr;  // the basis table as double-float values (the mixed path's load contraction)
    int fieldKmax = 8;       // the largest Fourier wave number of the uploaded fields
    TabJob *dTabJobs = nullptr, *dGtabJobs = nullptr;
    PfJob* dPfJobs = nullptr;
    int* dIbuf = nullptr;
    double *dCoefRaw = nullptr, *dCoefs = nullptr, *dFieldC = nullptr, *dFieldL = nullptr, *dY1 = nullptr,
           *dY2 = nullptr, *dS = nullptr, *dU = nullptr, *dBand = nullptr, *dLv1 = nullptr, *dLv2 = nullptr,
           *dLvec = nullptr;
    int *dPtr = nullptr, *dCol = nullptr, *dDiag = nullptr;
    int16_t* dColOff = nullptr;  // column - row, when every offset fits in 16 bits
    uint8_t* dBoxFlag = nullptr; // box rows of the SpMVs (CgBuffers::box), or none
    int* dBoxOff = nullptr;
    int nBox = 0;
    long long nBoxRows = 0;
    long long nnz = 0;           // non-zeros of the CSR system
    std::vector<double> ddofUser;  // eliminated-dof values given by the caller (gsgpu_set_fixed_dofs)
    bool ddofFromUser = false;
    bool devPattern = false;     // pattern built on the device (no interfaces): no host col/src arrays
    uint32_t *dSrc = nullptr, *dOvfPtr = nullptr, *dOvfIdx = nullptr, *dLptr = nullptr, *dLidx = nullptr,
             *dFptr = nullptr, *dFband = nullptr, *dFbidx = nullptr;
    double *dVal = nullptr, *dRhs = nullptr, *dDdof = nullptr;
    int* dIndex = nullptr;  // dof map (patch-local -> global), for the L2 error
    unsigned long long* dDetKey = nullptr;
    // mixed precision: df32 copies of the small inputs, the split CSR values and FP32 vectors
    df32 *dCoefsDf = nullptr, *dWqDf = nullptr;
    float *dValHi = nullptr, *dValLo = nullptr, *dDinv32 = nullptr;
    float *dR32 = nullptr, *dZ32 = nullptr, *dP32 = nullptr, *dT32 = nullptr, *dDx32 = nullptr, *dXhi = nullptr,
          *dXlo = nullptr;
    // the FP32 inner operator as half diagonals (single patch whose free dofs are one box, sdia.cu)
    bool sdiaOk = false;
    SdiaOp sdiaOp;
    SdiaBand sdiaBand;
    // kernel variants of this problem from the tuning table (autotune.cu), per degree class
    int tuned31[5] = {0, 0, 0, 0, 0}, tuned32[5] = {0, 0, 0, 0, 0}, tunedInner = kInnerSdiaRows4;
    void applyTuning();
    bool setInnerVariant();
    // time every variant on this problem, record the fastest in the table, apply it; ms[k]: the time
    // of each stiffness combination (6) and each inner-product variant (2)
    void autotune(double* ms);
    float* dSdia = nullptr;
    // batches: the half-diagonal inner operator of every problem (kernels_batch.cu), if all qualify
    bool segSdiaOk = false;
    std::vector<SegSdiaDesc> segSdiaHost;
    long long segSdiaSize = 0;  // stored values
    SegSdiaDesc* dSegSdiaDesc = nullptr;
    int nPiece = 0;  // pieces of the batch's segments (SegCg::pieceRow)
    int *dPieceRow = nullptr, *dPieceSeg = nullptr, *dSegPiece = nullptr;
    double* dPiecePart = nullptr;
    float* dSegSdia = nullptr;
    float* dP32pad = nullptr;         // allocation of the inner CG direction with its zero padding
    int* dSdiaErr = nullptr;          // set by the TMA-fed product's bounded waits when they expire
    alignas(64) unsigned char sdiaMaps[256] = {};  // two CUtensorMap (diagonals, x) when TMA is used
    void setupSdia();
    void setupSegSdia();
    Tab tabPf, tabCoef, tabGeo1, tabGeo2, tabPoint, tabSt[3], tabLd[3];
    Tab tabRow[3][5];  // [stage][degree along the stage axis]: interior rows of simple axes
    Tab tabRowB[3][5]; // the remaining rows
    Tab tabTile31[5];  // 3D stage 1 interior rows in shared-memory tiles (degrees 2, 3)
    // Neumann boundary integrals: the host plan, its sides, dofs and face-point blocks on the
    // device, and the face quadrature values
    NeumannPlan neu;
    NeuSide* dNeuSides = nullptr;
    NeuDof* dNeuDofs = nullptr;
    BlkEnt* dNeuBlocks = nullptr;
    double* dNeuVals = nullptr;

    // device buffers (solve)
    int solveN = -1;
    double *dX = nullptr, *dR = nullptr, *dZ = nullptr, *dP = nullptr, *dT = nullptr, *dDinv = nullptr;
    double *dPart0 = nullptr, *dPart1 = nullptr, *dPart2 = nullptr;
    CgState* dCg = nullptr;
    // instantiated solver graphs (16 iterations [+ replacement]); valid while the buffers live
    cudaGraphExec_t gexecFp64 = nullptr, gexecMixed = nullptr;
    int gexecLpr[2] = {0, 0};
    void dropGraphs();
    // h-multigrid: coarse levels, level-0 vectors, coarsest-level state and the solver graph
    std::vector<MgLevelBuf> mgl;
    int mgLevels = 0;
    long long assembleSerial = 0, mgSerial = -1;
    int mgPrecision = -1, mgCoarseIters = 0;
    double mgCoarseTol = 0.0;
    double *dMgVec0 = nullptr, *dMgPart = nullptr, *dRold = nullptr;  // level 0 FP64: dinv b x r z
    float* dFieldC32 = nullptr;  // FP32 copy of the df32 coefficient fields (coarse operators of the FP32 cycle)
    float* dMgPsplit = nullptr;  // outer MG-CG direction as double-float (hi, lo), mixed form
    float* dMgVec0f = nullptr;                                       // level 0 FP32: dinv b x r z
    CgState *dMgCoarseSt = nullptr, *dMgSt = nullptr;
    cudaGraphExec_t gexecMg = nullptr;
    MgGraphKey gexecMgKey;
    void mgSetup(int levels);
    void mgAssemble(bool mixed);
    void solveMG(const gsgpu_solver_opts& o, gsgpu_solve_info& info);
    double l2Error(bool h1);  // sqrt of the summed squared errors (h1: the H1 seminorm)
    std::vector<double> l2PerPatch(bool h1 = false);  // squared L2 (h1: H1 seminorm) error per patch
    // batches of independent problems (one patch each): segment = problem
    bool batch = false;
    std::vector<int> segRow;  // free-dof offsets per problem (nseg + 1)
    int *dSegRow = nullptr, *dRowSeg = nullptr, *dSegDone = nullptr;
    double *dSegRc0 = nullptr, *dSegRc1 = nullptr;
    SegState *dSegSt = nullptr, *dSegOuter = nullptr;
    df32* dSegXdf = nullptr;  // the double-float split of the batch solution (mixed residuals)
    cudaGraphExec_t gexecSeg[2] = {nullptr, nullptr};
    std::vector<SegState> segLast;
    void batchSetup();
    void solveBatch(const gsgpu_solver_opts& o, gsgpu_solve_info& info);
    static constexpr int kSegChunk = 16;  // segmented CG iterations per captured graph
    template <typename T>
    void segChunk(const SegCg<T>& B, cudaGraphExec_t& exec);
    template <typename T>
    void segRun(const SegCg<T>& B, cudaGraphExec_t& exec, int maxit);
    template <typename T>
    void mgRun(const gsgpu_solver_opts& o, gsgpu_solve_info& info, bool mixed);
    template <typename T>
    void mgPrepare(const gsgpu_solver_opts& o, bool mixed, std::vector<MgLevelDev<T>>& lv, MgParams& prm);
    void mgApply(const gsgpu_solver_opts& o, const double* r, double* z);
    void applyMatrix(const double* x, double* y);
    // profiling of the solver's SpMV launches
    bool profiling = false;
    long long spmvLaunches = 0;
    double spmvMs = 0.0, spmvBytes = 0.0;

    void refresh();
    void refreshUploads();
    void patternOnDevice(const RowPlan& rp);
    void patternFromHost();
    void findBoxRows();
    // SpMV bytes the box rows do not read (their column offsets) less the flags they do read
    double boxSavedBytes() const {
        return nBox ? double(nBoxRows) * nBox * (dColOff ? 2 : 4) - double(pat.n) : 0.0;
    }
    void setCoefs(const double* coefs);
    void assemble(int precision);
    double* dMass = nullptr;  // mass matrix values in the CSR pattern (gsgpu_mass_csr)
    void assembleMass();
    void solve(const gsgpu_solver_opts& o, gsgpu_solve_info& info);
    void times(double* ms);
    void freeAssembly();
    void buildTables();
    void ensureSolveBuffers();
    void ensureMixedBuffers();
    void solveMixed(const gsgpu_solver_opts& o, gsgpu_solve_info& info);
    int lanesPerRow(bool fp64) const;
    static Context reset(Context&& c);
};

}  // namespace gsgpu
