// The autotuner of the kernel variants (tuning table in autotune.h): it times each variant of the
// mixed assembly's stiffness contraction (3D stage 1: shared-memory tiles or rows with 4 / 2 output
// fields; stage 2: rows with 4 / 2 output fields) and of the inner FP32 product (load-based or
// TMA-fed half-diagonal operator) on the context's own problem with CUDA events, records the
// fastest per (kernel group, dimension, degree, Gauss points) in the process-wide table and applies
// it. Contexts made afterwards take their variants from the table (Context::applyTuning); the
// table can be saved and loaded, so a tuning run on one GPU serves later processes.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <limits>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/gsgpu.h"
#include "context.h"
#include "device_funcs.cuh"

namespace gsgpu {
namespace {

struct Entry {
    int variant;
    double ms;
};
std::mutex g_mutex;
std::map<std::tuple<int, int, int, int>, Entry> g_table;

std::tuple<int, int, int, int> asTuple(const TuneKey& k) { return std::make_tuple(k.kind, k.dim, k.p, k.q); }

}  // namespace

int tuneLookup(const TuneKey& k) {
    std::lock_guard<std::mutex> lock(g_mutex);
    auto it = g_table.find(asTuple(k));
    return it == g_table.end() ? -1 : it->second.variant;
}

void tuneRecord(const TuneKey& k, int variant, double ms) {
    std::lock_guard<std::mutex> lock(g_mutex);
    g_table[asTuple(k)] = Entry{variant, ms};
}

bool tuneSave(const char* path) {
    std::lock_guard<std::mutex> lock(g_mutex);
    std::ofstream f(path);
    if (!f) return false;
    f << "# gsgpu tuning table: kind dim degree gauss_points variant ms\n";
    for (const auto& kv : g_table)
        f << std::get<0>(kv.first) << ' ' << std::get<1>(kv.first) << ' ' << std::get<2>(kv.first) << ' '
          << std::get<3>(kv.first) << ' ' << kv.second.variant << ' ' << kv.second.ms << '\n';
    return bool(f);
}

bool tuneLoad(const char* path) {
    std::ifstream f(path);
    if (!f) return false;
    std::map<std::tuple<int, int, int, int>, Entry> add;
    std::string line;
    while (std::getline(f, line)) {
        if (line.empty() || line[0] == '#') continue;
        std::istringstream is(line);
        int kind, dim, p, q, v;
        double ms;
        if (!(is >> kind >> dim >> p >> q >> v >> ms)) return false;
        const bool ok = (kind == kTuneStage31 && v >= 0 && v <= 2) || (kind == kTuneStage32 && v >= 0 && v <= 1) ||
                        (kind == kTuneInner && v >= kInnerSdiaLoads && v <= kInnerSdiaRows4);
        if (!ok || dim < 2 || dim > 3 || p < 1 || p > 4 || q < 1) return false;
        add[std::make_tuple(kind, dim, p, q)] = Entry{v, ms};
    }
    std::lock_guard<std::mutex> lock(g_mutex);
    for (const auto& kv : add) g_table[kv.first] = kv.second;
    return true;
}

void tuneClear() {
    std::lock_guard<std::mutex> lock(g_mutex);
    g_table.clear();
}

namespace {
int gaussPoints(const ProblemDesc& pd, int p) { return int(pd.quA * p + pd.quB + 0.5); }
}  // namespace

// variants of this problem: the table, else the defaults (measured on GB300: stage-1 tiles where the
// degree has them, 4 output fields, the load-based inner product with four rows per thread); the
// environment overrides (GSGPU_NO_TILE31, GSGPU_ROW_NH=2|4, GSGPU_SDIA_INNER=0|1|2, GSGPU_SDIA_TMA)
// come last
void Context::applyTuning() {
    const int dim = pd.dim;
    for (int P = 1; P <= 4; ++P) {
        const int q = gaussPoints(pd, P);
        int v31 = tuneLookup({kTuneStage31, dim, P, q});
        if (v31 < 0) v31 = dev::tiledStage31(P) ? kStage31Tiles : kStage31RowsNh4;
        int v32 = tuneLookup({kTuneStage32, dim, P, q});
        if (v32 < 0) v32 = kStage32RowsNh4;
        if (std::getenv("GSGPU_NO_TILE31") && v31 == kStage31Tiles) v31 = kStage31RowsNh4;
        if (const char* e = std::getenv("GSGPU_ROW_NH")) {
            const bool two = std::atoi(e) == 2;
            v31 = two ? kStage31RowsNh2 : (v31 == kStage31RowsNh2 ? kStage31RowsNh4 : v31);
            v32 = two ? kStage32RowsNh2 : kStage32RowsNh4;
        }
        tuned31[P] = v31;
        tuned32[P] = v32;
    }
    tunedInner = kInnerSdiaRows4;
    if (sdiaOk) {
        const int v = tuneLookup({kTuneInner, dim, sdiaOp.p[0], gaussPoints(pd, sdiaOp.p[0])});
        if (v >= 0) tunedInner = v;
    }
    if (const char* e = std::getenv("GSGPU_SDIA_INNER")) {
        const int v = std::atoi(e);
        if (v >= kInnerSdiaLoads && v <= kInnerSdiaRows4) tunedInner = v;
    }
    if (std::getenv("GSGPU_SDIA_TMA")) tunedInner = kInnerSdiaTma;
}

void Context::autotune(double* ms) {
    if (!refreshed) throw StateError("autotune() before refresh()");
    if (device < 0) throw StateError("autotune() needs a CUDA device (host-only context)");
    double out[9];
    std::fill(out, out + 9, -1.0);
    const int dim = pd.dim;
    // degrees present along the stage axes
    std::vector<int> deg0, deg1;
    for (const DevPatch& D : L.dev) {
        if (std::find(deg0.begin(), deg0.end(), D.p[0]) == deg0.end()) deg0.push_back(D.p[0]);
        if (std::find(deg1.begin(), deg1.end(), D.p[1]) == deg1.end()) deg1.push_back(D.p[1]);
    }
    double ts[7];
    auto stiffness = [&]() {  // best of two timed mixed assemblies (after one untimed)
        assemble(kMixed);
        double best = std::numeric_limits<double>::infinity();
        for (int r = 0; r < 2; ++r) {
            assemble(kMixed);
            times(ts);
            best = std::min(best, ts[3]);
        }
        return best;
    };
    if (dim == 3) {
        const int v31s[3] = {kStage31Tiles, kStage31RowsNh4, kStage31RowsNh2};
        const int v32s[2] = {kStage32RowsNh4, kStage32RowsNh2};
        bool anyTiles = false;
        for (int P : deg0) anyTiles = anyTiles || dev::tiledStage31(P);
        double best = std::numeric_limits<double>::infinity();
        int b31 = -1, b32 = -1;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 2; ++b) {
                if (v31s[a] == kStage31Tiles && !anyTiles) continue;
                for (int P = 1; P <= 4; ++P) {
                    tuned31[P] = v31s[a] == kStage31Tiles && !dev::tiledStage31(P) ? kStage31RowsNh4 : v31s[a];
                    tuned32[P] = v32s[b];
                }
                const double t = stiffness();
                out[a * 2 + b] = t;
                if (t < best) best = t, b31 = v31s[a], b32 = v32s[b];
            }
        for (int P : deg0)
            tuneRecord({kTuneStage31, dim, P, gaussPoints(pd, P)},
                       b31 == kStage31Tiles && !dev::tiledStage31(P) ? kStage31RowsNh4 : b31, best);
        for (int P : deg1) tuneRecord({kTuneStage32, dim, P, gaussPoints(pd, P)}, b32, best);
    }
    if (sdiaOk && !batch) {
        // the inner product: each variant on the first iterations of a mixed solve, per-launch events
        ensureSolveBuffers();
        ensureMixedBuffers();
        gsgpu_solver_opts o{};
        o.method = GSGPU_SOLVER_CG_JACOBI;
        o.precision = GSGPU_PREC_MIXED;
        o.tol = 1e-30;  // run the iteration budget
        o.max_iters = 48;
        gsgpu_solve_info info{};
        const bool prof = profiling;
        const long long l0 = spmvLaunches;
        const double m0 = spmvMs;
        double best = std::numeric_limits<double>::infinity();
        int bv = kInnerSdiaLoads;
        for (int v : {kInnerSdiaLoads, kInnerSdiaTma, kInnerSdiaRows4}) {
            tunedInner = v;
            if (!setInnerVariant()) continue;
            profiling = true;
            solveMixed(o, info);  // warm
            spmvLaunches = 0;
            spmvMs = 0.0;
            solveMixed(o, info);
            const double t = spmvLaunches ? spmvMs / double(spmvLaunches) : std::numeric_limits<double>::infinity();
            out[6 + v] = t;
            if (t < best) best = t, bv = v;
        }
        profiling = prof;
        spmvLaunches = l0;
        spmvMs = m0;
        tuneRecord({kTuneInner, dim, sdiaOp.p[0], gaussPoints(pd, sdiaOp.p[0])}, bv, best);
        solved = false;
    }
    applyTuning();
    if (sdiaOk && dValHi) setInnerVariant();
    assemble(kMixed);  // leave the context assembled with the chosen variants
    if (ms) std::copy(out, out + 9, ms);
}

}  // namespace gsgpu
