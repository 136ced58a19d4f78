// Host-side set-up of the GPU assembly: the problem description, the gsDofMapper numbering,
// the symbolic CSR pattern with the slot -> band-entry gather maps, the Dirichlet values and the
// buffer layout of every patch. Plain C++ (no CUDA): this is what refresh() computes once per
// mesh; assemble() then only moves numbers through the kernels.
#pragma once

#include <cstdint>
#include <string>
#include <memory>
#include <utility>
#include <vector>

#include "gsgpu_internal.h"

namespace gsgpu {

// one-dimensional B-spline basis (knot vector with multiplicities)
struct Basis1D {
    int p = 0;
    std::vector<double> t;       // knots
    std::vector<double> breaks;  // distinct knot values
    int n() const { return int(t.size()) - p - 1; }
    int nelem() const { return int(breaks.size()) - 1; }
    void init(int deg, const double* k, int nk);
    int span(double u) const;                       // span index s, t[s] <= u < t[s+1]
    int elementSpan(int e) const;                   // span index of element e
    std::vector<double> greville() const;
    // values (k=0) and first derivatives (k=1) of the p+1 functions s-p..s at u:
    // out[k*(p+1)+r]
    void eval(int s, double u, double* out) const;
};

struct HostPatch {
    int dim = 2;
    int field = 0;  // index into ProblemDesc::pfields (0 when the problem has one field set)
    Basis1D b[3], g[3];
    std::vector<double> coefs;  // ngeo x dim, row-major
    int nd[3] = {1, 1, 1};
    int ndofs = 0;
    int offset = 0;
};

struct ProblemDesc {
    int dim = 2;
    std::vector<HostPatch> patches;
    std::vector<int> ifaces;    // 4 per interface
    std::vector<int> dsides;    // 2 per Dirichlet side
    std::vector<int> nsides;    // 2 per Neumann side
    FieldParams fields{};
    // batches of independent problems: one field set per problem (HostPatch::field indexes it);
    // empty for a single problem, whose patches all use `fields`
    std::vector<FieldParams> pfields;
    double quA = 1.0;
    int quB = 1;
    int dirL2 = 0;  // Dirichlet values by L2 projection (else interpolation)
    const FieldParams& fieldsOf(int patch) const {
        return pfields.empty() ? fields : pfields[size_t(patches[size_t(patch)].field)];
    }
    // the device field table: one entry per field set
    std::vector<FieldParams> fieldTable() const { return pfields.empty() ? std::vector<FieldParams>(1, fields) : pfields; }
};

// gsDofMapper numbering (src/gsCore/gsDofMapper.cpp:99-344) for a list of patches
struct DofMap {
    std::vector<int> index;     // per patch-local dof (concatenated) -> global index
    int freeSize = 0;
    int boundarySize = 0;
    int nlocal = 0;
};

void buildDofMap(const ProblemDesc& pd, DofMap& map);

// copy and validate a C-ABI problem description (include/gsgpu.h)
struct ProblemC;
void problemFromC(const void* gsgpu_problem_ptr, ProblemDesc& pd);
// a batch of independent single-patch problems as one ProblemDesc (patch j = problem j, with its
// own field set); quA/quB and the dimension must agree
void batchFromC(int count, const void* gsgpu_problem_array, ProblemDesc& pd);
// the same from validated descriptions (consumed)
void batchFromDescs(std::vector<ProblemDesc>& items, ProblemDesc& pd);

// allocator whose resize() leaves new elements uninitialised: the large pattern arrays are filled by
// parallel loops, which then also do the first touch of their pages
template <class T>
struct NoInitAlloc : std::allocator<T> {
    template <class U>
    struct rebind {
        using other = NoInitAlloc<U>;
    };
    NoInitAlloc() = default;
    template <class U>
    NoInitAlloc(const NoInitAlloc<U>&) noexcept {}
    template <class U>
    void construct(U* p) noexcept {
        ::new (static_cast<void*>(p)) U;
    }
    template <class U, class... Args>
    void construct(U* p, Args&&... a) {
        ::new (static_cast<void*>(p)) U(std::forward<Args>(a)...);
    }
};
template <class T>
using bigvec = std::vector<T, NoInitAlloc<T>>;

// symbolic CSR + gather maps
struct Pattern {
    int n = 0;
    std::vector<int> ptr;           // n+1 (int32: the reference's index_t)
    bigvec<int> col;                // nnz
    // per CSR slot: band entry (global band offset) or (kMulti | index into the overflow lists)
    bigvec<uint32_t> src;
    std::vector<uint32_t> ovf_ptr;  // overflow list pointers (slots with several sources)
    std::vector<uint32_t> ovf_idx;
    // per free row: load-vector sources (global load-vector offsets)
    std::vector<uint32_t> lptr, lidx;
    // per free row: Dirichlet lift terms (band entry, boundary index)
    std::vector<uint32_t> fptr, fband, fbidx;
    static constexpr uint32_t kMulti = 0x80000000u;
};

struct Layout {
    std::vector<DevPatch> dev;       // one descriptor per patch
    // packed per-direction host data
    std::vector<double> xi, wq;      // quadrature abscissae and weights
    std::vector<double> knots, gknots;
    std::vector<int> qspan, gqspan;  // per abscissa: span in the discretisation / geometry basis
    std::vector<int> ibuf;           // first active per element, elo/ehi per dof, geometry first per abscissa
    long long ntab = 0, ngtab = 0, npf = 0;   // sizes of basis tables and pair-factor tables
    long long coefs = 0, fields = 0, lfield = 0, y1 = 0, y2 = 0, s = 0, u = 0, band = 0, lv1 = 0, lv2 = 0, lvec = 0;
    // for the basis kernels: one entry per abscissa, and one pair-factor job per (patch, dir)
    std::vector<TabJob> tabjobs, gtabjobs;
    std::vector<PfJob> pfjobs;
};

void buildLayout(const ProblemDesc& pd, Layout& L);
void buildPattern(const ProblemDesc& pd, const DofMap& map, const Layout& L, Pattern& pat, int nthreads);
// Dirichlet values by interpolation at the boundary anchors
// (gsAssembler::computeDirichletDofsIntpl, src/gsAssembler/gsAssembler.hpp:314-390)
void dirichletValues(const ProblemDesc& pd, const DofMap& map, std::vector<double>& ddof);
// closed-form fields on the host (same formulas as the device)
void evalFields(const FieldParams& F, const double* x, double& kappa, double& f, double& u);
void gaussLegendre(int n, std::vector<double>& x, std::vector<double>& w);

// Neumann boundary integrals (gsVisitorNeumann): per Neumann side, its face quadrature grid (the
// volume rule's abscissae in the side directions, the boundary parameter in the fixed one) and the
// normal-direction basis values at the boundary; per patch-local dof on a Neumann side, the sides
// whose integrals it collects (in side order, so the sum is deterministic)
struct NeumannPlan {
    std::vector<NeuSide> sides;
    std::vector<NeuDof> dofs;
    std::vector<BlkEnt> blocks;  // face quadrature points, kBlock per entry (patch = side index)
    long long nvals = 0;         // face quadrature points over all sides
};
void buildNeumann(const ProblemDesc& pd, const Layout& L, int block, NeumannPlan& np);

// block -> (patch, base) tables for batched kernels
void blockTable(const std::vector<long long>& work, int block, std::vector<BlkEnt>& tab);

// Rows of a problem without interfaces: the patch and patch-local index of each free row, and per
// patch and direction the support-sharing neighbour range [jlo(i), jhi(i)] of every function
// (jlo at rng[rngOff[3 patch + a] + i], jhi n_a entries later)
struct RowPlan {
    std::vector<int> rowPatch, rowLoc;
    std::vector<int> rng;
    std::vector<long long> rngOff;
};
bool rowPlanSingle(const ProblemDesc& pd, const DofMap& map, const Layout& L, RowPlan& rp);

}  // namespace gsgpu
