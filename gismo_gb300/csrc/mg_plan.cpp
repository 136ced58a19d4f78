// Host set-up of the h-multigrid hierarchy (see mg_plan.h).
#include "mg_plan.h"

#include <algorithm>
#include <stdexcept>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace gsgpu {

Basis1D coarsenBasis(const Basis1D& B) {
    // keep the end breaks and every second interior break, with their multiplicities
    std::vector<double> t;
    const std::vector<double>& br = B.breaks;
    const int m = int(br.size()) - 1;
    for (int i = 0; i <= m; ++i) {
        if (!(i == 0 || i == m || i % 2 == 0)) continue;
        const int mult = int(std::count(B.t.begin(), B.t.end(), br[i]));
        for (int r = 0; r < mult; ++r) t.push_back(br[i]);
    }
    Basis1D C;
    C.init(B.p, t.data(), int(t.size()));
    return C;
}

// knot-insertion matrix T (nf x nc, row-major): fine function values of the coarse functions,
// built by inserting the missing knots one at a time (Boehm's algorithm)
static std::vector<double> insertionMatrix(const Basis1D& C, const Basis1D& F) {
    const int p = C.p;
    std::vector<double> t = C.t;
    int n = C.n();
    const int nc = n;
    std::vector<double> T(size_t(n) * nc, 0.0);
    for (int i = 0; i < n; ++i) T[size_t(i) * nc + i] = 1.0;
    std::vector<double> extra;
    {
        size_t a = 0;
        for (double u : F.t) {
            if (a < t.size() && t[a] == u) ++a;
            else extra.push_back(u);
        }
    }
    for (double u : extra) {
        const int s = int(std::upper_bound(t.begin(), t.end(), u) - t.begin()) - 1;
        std::vector<double> Tn(size_t(n + 1) * nc, 0.0);
        for (int i = 0; i <= n; ++i) {
            const double a = (i <= s - p) ? 1.0 : (i > s ? 0.0 : (u - t[i]) / (t[i + p] - t[i]));
            for (int c = 0; c < nc; ++c) {
                double v = 0.0;
                if (i < n) v += a * T[size_t(i) * nc + c];
                if (i >= 1) v += (1.0 - a) * T[size_t(i - 1) * nc + c];
                Tn[size_t(i) * nc + c] = v;
            }
        }
        t.insert(t.begin() + s + 1, u);
        ++n;
        T.swap(Tn);
    }
    if (n != F.n()) throw std::runtime_error("multigrid: coarse knots are not nested in the fine knots");
    return T;
}

// layout of a coarse level on the finest quadrature grid
static void layoutOnGrid(const ProblemDesc& pdl, const ProblemDesc& fine, const Layout& FL, Layout& L) {
    L = Layout();
    const int d = pdl.dim;
    long long xo = 0, ko = 0, io = 0, to = 0, pfo = 0;
    for (size_t pi = 0; pi < pdl.patches.size(); ++pi) {
        const HostPatch& P = pdl.patches[pi];
        const HostPatch& PF = fine.patches[pi];
        const DevPatch& FD = FL.dev[pi];
        DevPatch D = FD;  // quadrature grid, fields and geometry extents of the finest level
        for (int k = 0; k < 3; ++k) D.simple[k] = 0;  // coarse functions on fine elements: general shape
        D.ndof = 1;
        D.bandsize = 1;
        for (int k = 0; k < 3; ++k) {
            if (k >= d) continue;
            const Basis1D& B = P.b[k];
            const Basis1D& Bf = PF.b[k];
            D.p[k] = B.p;
            D.n[k] = B.n();
            D.W[k] = 2 * B.p + 1;
            D.ndof *= D.n[k];
            D.bandsize *= (long long)D.n[k] * D.W[k];
            // abscissae of the finest level
            D.qoff[k] = xo;
            for (int g = 0; g < FD.Q[k]; ++g) {
                L.xi.push_back(FL.xi[FD.qoff[k] + g]);
                L.wq.push_back(FL.wq[FD.qoff[k] + g]);
            }
            xo += FD.Q[k];
            const long long kofs = ko;
            L.knots.insert(L.knots.end(), B.t.begin(), B.t.end());
            ko += (long long)B.t.size();
            D.toff[k] = to;
            for (int g = 0; g < FD.Q[k]; ++g) {
                const double u = L.xi[D.qoff[k] + g];
                L.tabjobs.push_back({kofs, to + (long long)g * 2 * (B.p + 1), u, B.p, B.span(u)});
            }
            to += (long long)FD.Q[k] * 2 * (B.p + 1);
            // first active coarse function per fine element, support ranges in fine elements
            D.eoff[k] = io;
            std::vector<int> first(FD.E[k]);
            for (int e = 0; e < FD.E[k]; ++e) {
                first[e] = B.span(0.5 * (Bf.breaks[e] + Bf.breaks[e + 1])) - B.p;
                L.ibuf.push_back(first[e]);
            }
            io += FD.E[k];
            D.doff[k] = io;
            std::vector<int> elo(D.n[k], 1 << 30), ehi(D.n[k], -1);
            for (int e = 0; e < FD.E[k]; ++e)
                for (int s = 0; s <= B.p; ++s) {
                    elo[first[e] + s] = std::min(elo[first[e] + s], e);
                    ehi[first[e] + s] = std::max(ehi[first[e] + s], e);
                }
            for (int i = 0; i < D.n[k]; ++i) L.ibuf.push_back(elo[i]);
            for (int i = 0; i < D.n[k]; ++i) L.ibuf.push_back(ehi[i]);
            io += 2LL * D.n[k];
            D.gqoff[k] = 0;
            D.pfoff[k] = pfo;
            const long long npf = 4LL * FD.E[k] * FD.q[k] * (B.p + 1) * (B.p + 1);
            L.pfjobs.push_back({D.toff[k], pfo, npf, B.p, FD.q[k], FD.E[k], 0});
            pfo += npf;
        }
        const long long n0W = (long long)D.n[0] * D.W[0], n1W = (long long)D.n[1] * D.W[1];
        D.field_off = FD.field_off;  // the finest level's coefficient field
        D.coef_off = D.lfield_off = D.y1_off = D.y2_off = D.lv1_off = D.lv2_off = D.lvec_off = 0;
        if (d == 3) {
            D.s_off = L.s; L.s += 8LL * D.Q[2] * D.Q[1] * n0W;
            D.u_off = L.u; L.u += 4LL * D.Q[2] * n1W * n0W;
        } else {
            D.s_off = L.s; L.s += 4LL * D.Q[1] * n0W;
            D.u_off = L.u;
        }
        D.band_off = L.band; L.band += D.bandsize;
        L.dev.push_back(D);
    }
    L.ntab = to;
    L.npf = pfo;
    if (L.band >= (long long)Pattern::kMulti) throw std::invalid_argument("multigrid level too large for 31-bit band indexing");
}

static void diagSlots(const Pattern& pat, std::vector<int>& diag) {
    diag.assign(pat.n, -1);
    for (int r = 0; r < pat.n; ++r) {
        const int* b = pat.col.data() + pat.ptr[r];
        const int* e = pat.col.data() + pat.ptr[r + 1];
        const int* f = std::lower_bound(b, e, r);
        if (f == e || *f != r) throw std::runtime_error("multigrid level pattern has no diagonal entry");
        diag[r] = pat.ptr[r] + int(f - b);
    }
}

// P: rows = free dofs of the finer level, cols = free dofs of the coarser level
static void buildTransfer(const ProblemDesc& pf, const DofMap& mf, const ProblemDesc& pc, const DofMap& mc,
                          MgLevelPlan& out) {
    const int d = pf.dim;
    const int nf = mf.freeSize;
    std::vector<int> pre(nf, -1), prePatch(nf, -1);
    for (size_t pi = 0; pi < pf.patches.size(); ++pi) {
        const HostPatch& P = pf.patches[pi];
        for (int i = 0; i < P.ndofs; ++i) {
            const int I = mf.index[P.offset + i];
            if (I < nf && pre[I] < 0) { pre[I] = i; prePatch[I] = int(pi); }
        }
    }
    std::vector<std::vector<double>> T(pf.patches.size() * 3);
    for (size_t pi = 0; pi < pf.patches.size(); ++pi)
        for (int k = 0; k < d; ++k) T[pi * 3 + k] = insertionMatrix(pc.patches[pi].b[k], pf.patches[pi].b[k]);
    std::vector<std::vector<std::pair<int, double>>> rows(nf);
#pragma omp parallel for schedule(dynamic, 256)
    for (int I = 0; I < nf; ++I) {
        const int pi = prePatch[I];
        const HostPatch& F = pf.patches[pi];
        const HostPatch& Cp = pc.patches[pi];
        int c[3] = {0, 0, 0}, r = pre[I];
        for (int k = 0; k < d; ++k) { c[k] = r % F.nd[k]; r /= F.nd[k]; }
        // non-zeros of the 1-D rows
        std::vector<std::pair<int, double>> nz[3];
        for (int k = 0; k < 3; ++k) {
            if (k >= d) { nz[k].push_back({0, 1.0}); continue; }
            const int ncd = Cp.nd[k];
            const std::vector<double>& Tk = T[size_t(pi) * 3 + k];
            for (int j = 0; j < ncd; ++j) {
                const double v = Tk[size_t(c[k]) * ncd + j];
                if (v != 0.0) nz[k].push_back({j, v});
            }
        }
        auto& row = rows[I];
        for (auto& a2 : nz[2])
            for (auto& a1 : nz[1])
                for (auto& a0 : nz[0]) {
                    const int lj = a0.first + Cp.nd[0] * (a1.first + (d == 3 ? Cp.nd[1] * a2.first : 0));
                    const int J = mc.index[Cp.offset + lj];
                    if (J >= mc.freeSize) continue;
                    row.push_back({J, a0.second * a1.second * a2.second});
                }
        std::sort(row.begin(), row.end());
    }
    out.Pptr.assign(nf + 1, 0);
    for (int I = 0; I < nf; ++I) out.Pptr[I + 1] = out.Pptr[I] + int(rows[I].size());
    out.Pcol.resize(out.Pptr[nf]);
    out.Pval.resize(out.Pptr[nf]);
    for (int I = 0; I < nf; ++I)
        for (size_t k = 0; k < rows[I].size(); ++k) {
            out.Pcol[out.Pptr[I] + k] = rows[I][k].first;
            out.Pval[out.Pptr[I] + k] = rows[I][k].second;
        }
    // transpose
    const int nc = mc.freeSize;
    out.Rptr.assign(nc + 1, 0);
    for (int c2 : out.Pcol) ++out.Rptr[c2 + 1];
    for (int i = 0; i < nc; ++i) out.Rptr[i + 1] += out.Rptr[i];
    out.Rcol.resize(out.Pcol.size());
    out.Rval.resize(out.Pcol.size());
    std::vector<int> fill(out.Rptr.begin(), out.Rptr.end() - 1);
    for (int I = 0; I < nf; ++I)
        for (int k = out.Pptr[I]; k < out.Pptr[I + 1]; ++k) {
            const int J = out.Pcol[k];
            out.Rcol[fill[J]] = I;
            out.Rval[fill[J]++] = out.Pval[k];
        }
}

void buildMgPlan(const ProblemDesc& fine, const DofMap& fineMap, const Layout& fineLayout, int nlevels,
                 std::vector<MgLevelPlan>& levels) {
    levels.clear();
    if (nlevels < 2) return;
    const ProblemDesc* prevPd = &fine;
    const DofMap* prevMap = &fineMap;
    levels.resize(nlevels - 1);
    for (int l = 0; l + 1 < nlevels; ++l) {
        MgLevelPlan& M = levels[l];
        M.pd = *prevPd;
        int off = 0;
        for (HostPatch& P : M.pd.patches) {
            P.ndofs = 1;
            for (int k = 0; k < M.pd.dim; ++k) {
                if (P.b[k].nelem() < 2) throw std::invalid_argument("multigrid: a patch has too few elements to coarsen");
                P.b[k] = coarsenBasis(P.b[k]);
                P.nd[k] = P.b[k].n();
                P.ndofs *= P.nd[k];
            }
            P.offset = off;
            off += P.ndofs;
        }
        buildDofMap(M.pd, M.map);
        layoutOnGrid(M.pd, fine, fineLayout, M.L);
        buildPattern(M.pd, M.map, M.L, M.pat, 0);
        diagSlots(M.pat, M.diag);
        buildTransfer(*prevPd, *prevMap, M.pd, M.map, M);
        prevPd = &M.pd;
        prevMap = &M.map;
    }
}

}  // namespace gsgpu
