// Host set-up of the GPU assembly (see plan.h).
#include "plan.h"

#include "../../include/gsgpu.h"

#include <algorithm>
#include <cmath>
#include <numeric>
#include <stdexcept>
#include <unordered_map>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace gsgpu {

// ---------------------------------------------------------------------------------------------
// knot vectors and 1-D B-splines (G+Smo: gsKnotVector, gsBSplineBasis)

void Basis1D::init(int deg, const double* k, int nk) {
    if (deg < 0 || nk < 2 * deg + 2) throw std::invalid_argument("invalid knot vector / degree");
    p = deg;
    t.assign(k, k + nk);
    for (int i = 1; i < nk; ++i)
        if (t[i] < t[i - 1]) throw std::invalid_argument("knot vector is not non-decreasing");
    breaks.clear();
    for (double v : t)
        if (breaks.empty() || v > breaks.back()) breaks.push_back(v);
}

// last s with t[s] <= u < t[s+1], clamped to [p, n-1]; the right end maps into the last
// non-empty span (gsKnotVector::iFind, src/gsNurbs/gsKnotVector.hpp:747-790)
int Basis1D::span(double u) const {
    const int nn = n();
    if (u >= t[nn]) {
        int s = nn - 1;
        while (s > p && t[s] == t[s + 1]) --s;
        return s;
    }
    int s = int(std::upper_bound(t.begin(), t.end(), u) - t.begin()) - 1;
    return std::max(p, std::min(s, nn - 1));
}

int Basis1D::elementSpan(int e) const { return span(0.5 * (breaks[e] + breaks[e + 1])); }

std::vector<double> Basis1D::greville() const {
    std::vector<double> g(n());
    for (int i = 0; i < n(); ++i) {
        if (p == 0) { g[i] = 0.5 * (t[i] + t[i + 1]); continue; }
        double s = 0;
        for (int j = 1; j <= p; ++j) s += t[i + j];
        g[i] = s / p;
    }
    return g;
}

// Cox-de Boor triangle for the p+1 non-zero functions of span s, then first derivatives from
// the degree p-1 values: N'_{i,p} = p N_{i,p-1}/(t_{i+p}-t_i) - p N_{i+1,p-1}/(t_{i+p+1}-t_{i+1})
void Basis1D::eval(int s, double u, double* out) const {
    double N[32], Nm1[32];
    N[0] = 1.0;
    if (p == 0) { out[0] = 1.0; out[1] = 0.0; return; }
    for (int k = 1; k <= p; ++k) {
        if (k == p)
            for (int r = 0; r < p; ++r) Nm1[r] = N[r];
        double saved = 0.0;
        for (int r = 0; r < k; ++r) {
            const double tr = t[s + 1 + r], tl = t[s + 1 + r - k];
            const double tmp = N[r] / (tr - tl);
            N[r] = saved + (tr - u) * tmp;
            saved = (u - tl) * tmp;
        }
        N[k] = saved;
    }
    const int a = s - p;
    for (int r = 0; r <= p; ++r) {
        out[r] = N[r];
        double d = 0.0;
        if (r >= 1) d += p * Nm1[r - 1] / (t[a + r + p] - t[a + r]);
        if (r <= p - 1) d -= p * Nm1[r] / (t[a + r + p + 1] - t[a + r + 1]);
        out[p + 1 + r] = d;
    }
}

void gaussLegendre(int n, std::vector<double>& x, std::vector<double>& w) {
    // roots of the Legendre polynomial P_n by Newton's method from Tricomi's initial guesses
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    for (int i = 0; i < n; ++i) {
        long double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
        long double dp = 0;
        for (int it = 0; it < 100; ++it) {
            long double p0 = 1, p1 = 0;
            for (int k = 1; k <= n; ++k) {
                const long double p2 = p1;
                p1 = p0;
                p0 = ((2 * k - 1) * z * p1 - (k - 1) * p2) / k;
            }
            dp = n * (z * p0 - p1) / (z * z - 1);
            const long double dz = p0 / dp;
            z -= dz;
            if (std::fabs((double)dz) < 1e-19) break;
        }
        x[n - 1 - i] = (double)z;
        w[n - 1 - i] = (double)(2.0L / ((1 - z * z) * dp * dp));
    }
    if (n % 2 == 1) x[n / 2] = 0.0;
}

// ---------------------------------------------------------------------------------------------
// closed-form fields: kappa = exp(alpha g), g = scale sum_m amp_m cos(pi k_m.x + phase_m),
// u = prod_i sin(freq pi x_i), f = -div(kappa grad u)
// u alone (the Dirichlet data): the same operations as the u of evalFields, so the same value
static double evalU(const FieldParams& F, const double* x) {
    const double w = F.ufreq * M_PI;
    double u = 1.0;
    for (int i = 0; i < F.dim; ++i) u *= std::sin(w * x[i]);
    return u;
}

void evalFields(const FieldParams& F, const double* x, double& kappa, double& f, double& u) {
    const int d = F.dim;
    const double w = F.ufreq * M_PI;
    double sn[3], cs[3];
    for (int i = 0; i < d; ++i) { sn[i] = std::sin(w * x[i]); cs[i] = std::cos(w * x[i]); }
    u = 1.0;
    for (int i = 0; i < d; ++i) u *= sn[i];
    double gu[3];
    for (int j = 0; j < d; ++j) {
        gu[j] = w * cs[j];
        for (int i = 0; i < d; ++i) if (i != j) gu[j] *= sn[i];
    }
    double g = 0, gg[3] = {0, 0, 0};
    if (F.fourier) {
        for (int m = 0; m < F.nmodes; ++m) {
            double th = F.phase[m];
            for (int i = 0; i < d; ++i) th += M_PI * F.kk[m][i] * x[i];
            g += F.amp[m] * std::cos(th);
            const double sth = std::sin(th);
            for (int i = 0; i < d; ++i) gg[i] -= F.amp[m] * sth * M_PI * F.kk[m][i];
        }
        g *= F.scale;
        for (int i = 0; i < d; ++i) gg[i] *= F.scale;
        kappa = std::exp(F.alpha * g);
    } else {
        kappa = F.kconst;
    }
    double dot = 0;
    for (int i = 0; i < d; ++i) dot += gg[i] * gu[i];
    f = kappa * (d * w * w * u - F.alpha * dot);
}

// ---------------------------------------------------------------------------------------------
// side slices: local indices with coordinate dir fixed, increasing order
// (gsTensorBasis::boundaryOffset, src/gsTensor/gsTensorBasis.hpp:303-311)
static void sideDofs(const HostPatch& P, int side, std::vector<int>& out) {
    const int dir = (side - 1) / 2, par = (side - 1) % 2;
    const int fix = par ? P.nd[dir] - 1 : 0;
    out.clear();
    const int n0 = P.nd[0], n1 = P.dim > 1 ? P.nd[1] : 1, n2 = P.dim > 2 ? P.nd[2] : 1;
    for (int c2 = 0; c2 < n2; ++c2)
        for (int c1 = 0; c1 < n1; ++c1)
            for (int c0 = 0; c0 < n0; ++c0) {
                const int c[3] = {c0, c1, c2};
                if (c[dir] == fix) out.push_back(c0 + n0 * (c1 + n1 * c2));
            }
}

// gsDofMapper: eliminated / coupled / standard classes by union-find, final numbering
// standard (scan order), coupled classes (first appearance), eliminated classes (first appearance)
void buildDofMap(const ProblemDesc& pd, DofMap& map) {
    int nl = 0;
    for (const HostPatch& P : pd.patches) nl += P.ndofs;
    std::vector<int> par(nl);
    std::iota(par.begin(), par.end(), 0);
    std::vector<uint8_t> el(nl, 0), cp(nl, 0);
    auto find = [&](int a) {
        while (par[a] != a) { par[a] = par[par[a]]; a = par[a]; }
        return a;
    };
    std::vector<int> s1, s2;
    for (size_t i = 0; i < pd.dsides.size(); i += 2) {
        const HostPatch& P = pd.patches.at(pd.dsides[i]);
        sideDofs(P, pd.dsides[i + 1], s1);
        for (int l : s1) el[find(P.offset + l)] = 1;
    }
    for (size_t i = 0; i < pd.ifaces.size(); i += 4) {
        const HostPatch& A = pd.patches.at(pd.ifaces[i]);
        const HostPatch& B = pd.patches.at(pd.ifaces[i + 2]);
        sideDofs(A, pd.ifaces[i + 1], s1);
        sideDofs(B, pd.ifaces[i + 3], s2);
        if (s1.size() != s2.size()) throw std::invalid_argument("interface sides do not conform");
        for (size_t k = 0; k < s1.size(); ++k) {
            int ra = find(A.offset + s1[k]), rb = find(B.offset + s2[k]);
            if (ra != rb) {
                if (ra > rb) std::swap(ra, rb);
                par[rb] = ra;
                el[ra] |= el[rb];
            }
            if (!el[ra]) cp[ra] = 1;
        }
    }
    map.index.assign(nl, -1);
    map.nlocal = nl;
    int nstd = 0;
    for (int i = 0; i < nl; ++i) {
        const int r = find(i);
        if (!el[r] && !cp[r]) ++nstd;
    }
    std::vector<int> cls(nl, -1);
    int curFree = 0, curCpl = nstd;
    for (int i = 0; i < nl; ++i) {
        const int r = find(i);
        if (el[r]) continue;
        if (!cp[r]) map.index[i] = curFree++;
        else {
            if (cls[r] < 0) cls[r] = curCpl++;
            map.index[i] = cls[r];
        }
    }
    map.freeSize = curCpl;
    int curElim = curCpl;
    for (int i = 0; i < nl; ++i) {
        const int r = find(i);
        if (!el[r]) continue;
        if (cls[r] < 0) cls[r] = curElim++;
        map.index[i] = cls[r];
    }
    map.boundarySize = curElim - map.freeSize;
}

// ---------------------------------------------------------------------------------------------
void buildLayout(const ProblemDesc& pd, Layout& L) {
    L = Layout();
    const int d = pd.dim;
    long long xo = 0, ko = 0, gko = 0, io = 0, to = 0, gto = 0, pfo = 0;
    std::vector<double> gx, gw;
    for (const HostPatch& P : pd.patches) {
        DevPatch D{};
        D.dim = d;
        D.field_id = pd.pfields.empty() ? 0 : P.field;
        D.ngeo = 1;
        D.nq = 1;
        D.ndof = 1;
        D.bandsize = 1;
        for (int k = 0; k < 3; ++k) {
            if (k >= d) {
                D.p[k] = 0; D.n[k] = 1; D.E[k] = 1; D.q[k] = 1; D.Q[k] = 1; D.W[k] = 1; D.gp[k] = 0; D.gn[k] = 1;
                continue;
            }
            const Basis1D& B = P.b[k];
            const Basis1D& G = P.g[k];
            D.p[k] = B.p;
            D.n[k] = B.n();
            D.E[k] = B.nelem();
            D.q[k] = int(pd.quA * B.p + pd.quB + 0.5);
            D.Q[k] = D.E[k] * D.q[k];
            D.W[k] = 2 * B.p + 1;
            D.gp[k] = G.p;
            D.gn[k] = G.n();
            if (B.p < 1 || B.p > 4 || G.p > 15 || D.q[k] > 32)
                throw std::invalid_argument("discretisation degree must be 1..4 (geometry degree <= 15, <= 32 Gauss points)");
            D.ngeo *= D.gn[k];
            D.nq *= D.Q[k];
            D.ndof *= D.n[k];
            D.bandsize *= (long long)D.n[k] * D.W[k];
            // quadrature abscissae and weights (gsQuadRule::mapTo, gsQuadRule.hpp:23-37)
            gaussLegendre(D.q[k], gx, gw);
            D.qoff[k] = xo;
            for (int e = 0; e < D.E[k]; ++e) {
                const double lo = B.breaks[e], hi = B.breaks[e + 1];
                const double h = (hi - lo) / 2.0;
                const int sp = B.elementSpan(e);
                for (int r = 0; r < D.q[k]; ++r) {
                    const double u = h * (gx[r] + 1) + lo;
                    L.xi.push_back(u);
                    L.wq.push_back((h == 0 ? 0.5 : h) * gw[r]);
                    L.qspan.push_back(sp);
                    L.gqspan.push_back(G.span(u));
                }
            }
            xo += D.Q[k];
            // knots
            const long long kofs = ko, gkofs = gko;
            L.knots.insert(L.knots.end(), B.t.begin(), B.t.end());
            ko += (long long)B.t.size();
            L.gknots.insert(L.gknots.end(), G.t.begin(), G.t.end());
            gko += (long long)G.t.size();
            // basis tables: per abscissa [V_0..V_p, D_0..D_p]
            D.toff[k] = to;
            D.gtoff[k] = gto;
            for (int g = 0; g < D.Q[k]; ++g) {
                const long long gi = D.qoff[k] + g;
                L.tabjobs.push_back({kofs, to + (long long)g * 2 * (B.p + 1), L.xi[gi], B.p, L.qspan[gi]});
                L.gtabjobs.push_back({gkofs, gto + (long long)g * 2 * (G.p + 1), L.xi[gi], G.p, L.gqspan[gi]});
            }
            to += (long long)D.Q[k] * 2 * (B.p + 1);
            gto += (long long)D.Q[k] * 2 * (G.p + 1);
            // integer tables: first active per element, elo/ehi per dof, geometry first per abscissa
            D.eoff[k] = io;
            for (int e = 0; e < D.E[k]; ++e) L.ibuf.push_back(B.elementSpan(e) - B.p);
            io += D.E[k];
            D.doff[k] = io;
            std::vector<int> elo(D.n[k], 1 << 30), ehi(D.n[k], -1);
            for (int e = 0; e < D.E[k]; ++e) {
                const int f = B.elementSpan(e) - B.p;
                for (int s = 0; s <= B.p; ++s) {
                    elo[f + s] = std::min(elo[f + s], e);
                    ehi[f + s] = std::max(ehi[f + s], e);
                }
            }
            for (int i = 0; i < D.n[k]; ++i) {
                if (ehi[i] < 0) throw std::invalid_argument("basis function with empty support");
                L.ibuf.push_back(elo[i]);
            }
            for (int i = 0; i < D.n[k]; ++i) L.ibuf.push_back(ehi[i]);
            io += 2LL * D.n[k];
            {
                bool simple = D.q[k] == B.p + 1 && D.n[k] == D.E[k] + B.p;
                for (int e = 0; e < D.E[k] && simple; ++e) simple = B.elementSpan(e) - B.p == e;
                for (int i = 0; i < D.n[k] && simple; ++i)
                    simple = elo[i] == std::max(0, i - B.p) && ehi[i] == std::min(D.E[k] - 1, i);
                D.simple[k] = simple ? 1 : 0;
            }
            D.gqoff[k] = io;
            for (int g = 0; g < D.Q[k]; ++g) L.ibuf.push_back(L.gqspan[D.qoff[k] + g] - G.p);
            io += D.Q[k];
            D.pfoff[k] = pfo;
            const long long npf = 4LL * D.E[k] * D.q[k] * (B.p + 1) * (B.p + 1);
            L.pfjobs.push_back({D.toff[k], pfo, npf, B.p, D.q[k], D.E[k], 0});
            pfo += npf;
        }
        // big buffers
        const int ncomp = d == 3 ? 6 : 3;
        D.coef_off = L.coefs; L.coefs += (long long)d * D.ngeo;
        D.field_off = L.fields; L.fields += (long long)ncomp * D.nq;
        D.lfield_off = L.lfield; L.lfield += D.nq;
        const long long n0W = (long long)D.n[0] * D.W[0], n1W = (long long)D.n[1] * D.W[1];
        if (d == 3) {
            D.y1_off = L.y1; L.y1 += (long long)d * 2 * D.gn[2] * D.gn[1] * D.Q[0];
            D.y2_off = L.y2; L.y2 += (long long)d * 3 * D.gn[2] * D.Q[1] * D.Q[0];
            D.s_off = L.s; L.s += 8LL * D.Q[2] * D.Q[1] * n0W;
            D.u_off = L.u; L.u += 4LL * D.Q[2] * n1W * n0W;
            D.lv1_off = L.lv1; L.lv1 += (long long)D.Q[2] * D.Q[1] * D.n[0];
            D.lv2_off = L.lv2; L.lv2 += (long long)D.Q[2] * D.n[1] * D.n[0];
        } else {
            D.y1_off = L.y1; L.y1 += (long long)d * 2 * D.gn[1] * D.Q[0];
            D.y2_off = L.y2;
            D.s_off = L.s; L.s += 4LL * D.Q[1] * n0W;
            D.u_off = L.u;
            D.lv1_off = L.lv1; L.lv1 += (long long)D.Q[1] * D.n[0];
            D.lv2_off = L.lv2;
        }
        D.band_off = L.band; L.band += D.bandsize;
        D.lvec_off = L.lvec; L.lvec += D.ndof;
        L.dev.push_back(D);
    }
    L.ntab = to;
    L.ngtab = gto;
    L.npf = pfo;
    if (L.band >= (long long)Pattern::kMulti || L.lvec >= (long long)Pattern::kMulti)
        throw std::invalid_argument("problem too large for 31-bit band indexing");
}

// ---------------------------------------------------------------------------------------------
namespace {
struct RowScratch {
    std::vector<std::pair<int, uint32_t>> ent;  // (column, band entry)
    std::vector<std::pair<uint32_t, uint32_t>> lift;
};

// all (column, band entry) pairs of global free row I and its Dirichlet lift terms
void rowEntries(const ProblemDesc& pd, const DofMap& map, const Layout& L, const std::vector<int>& preptr,
                const std::vector<int>& preloc, const std::vector<int>& prepatch, int I, RowScratch& rs,
                bool& sorted) {
    rs.ent.clear();
    rs.lift.clear();
    const int d = pd.dim;
    for (int k = preptr[I]; k < preptr[I + 1]; ++k) {
        const int pi = prepatch[k];
        const HostPatch& P = pd.patches[pi];
        const DevPatch& D = L.dev[pi];
        const int li = preloc[k] - P.offset;
        int c[3] = {0, 0, 0}, r = li;
        for (int a = 0; a < d; ++a) { c[a] = r % P.nd[a]; r /= P.nd[a]; }
        int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
        const int* elo[3];
        const int* ehi[3];
        for (int a = 0; a < d; ++a) {
            lo[a] = std::max(0, c[a] - D.p[a]);
            hi[a] = std::min(P.nd[a] - 1, c[a] + D.p[a]);
            elo[a] = L.ibuf.data() + D.doff[a];
            ehi[a] = elo[a] + D.n[a];
        }
        const long long n0W = (long long)D.n[0] * D.W[0], n1W = (long long)D.n[1] * D.W[1];
        for (int z = lo[2]; z <= hi[2]; ++z)
            for (int y = lo[1]; y <= hi[1]; ++y)
                for (int x = lo[0]; x <= hi[0]; ++x) {
                    const int cc[3] = {x, y, z};
                    bool share = true;
                    for (int a = 0; a < d && share; ++a)
                        share = std::max(elo[a][c[a]], elo[a][cc[a]]) <= std::min(ehi[a][c[a]], ehi[a][cc[a]]);
                    if (!share) continue;
                    const int lj = x + P.nd[0] * (y + (d == 3 ? P.nd[1] * z : 0));
                    const int J = map.index[P.offset + lj];
                    long long b = (long long)c[0] * D.W[0] + (x - c[0] + D.p[0]);
                    b += ((long long)c[1] * D.W[1] + (y - c[1] + D.p[1])) * n0W;
                    if (d == 3) b += ((long long)c[2] * D.W[2] + (z - c[2] + D.p[2])) * n0W * n1W;
                    b += D.band_off;
                    if (J < map.freeSize) rs.ent.push_back({J, uint32_t(b)});
                    else rs.lift.push_back({uint32_t(b), uint32_t(J - map.freeSize)});
                }
    }
    sorted = true;
    for (size_t i = 1; i < rs.ent.size() && sorted; ++i) sorted = rs.ent[i - 1].first < rs.ent[i].first;
    if (!sorted)
        std::stable_sort(rs.ent.begin(), rs.ent.end(),
                         [](const std::pair<int, uint32_t>& a, const std::pair<int, uint32_t>& b) { return a.first < b.first; });
}
}  // namespace

// rows of a problem without interfaces: pre-image of each free row and support-sharing neighbour
// ranges per patch and direction (false if a free dof has two pre-images or a range is not
// contiguous)
bool rowPlanSingle(const ProblemDesc& pd, const DofMap& map, const Layout& L, RowPlan& rp) {
    if (!pd.ifaces.empty()) return false;
    const int n = map.freeSize;
    const int d = pd.dim;
    const size_t np = pd.patches.size();
    rp = RowPlan();
    rp.rowPatch.assign(n, -1);
    rp.rowLoc.assign(n, -1);
    for (size_t pi = 0; pi < np; ++pi) {
        const HostPatch& P = pd.patches[pi];
        for (int i = 0; i < P.ndofs; ++i) {
            const int J = map.index[P.offset + i];
            if (J >= n) continue;
            if (rp.rowPatch[J] >= 0) return false;
            rp.rowPatch[J] = int(pi);
            rp.rowLoc[J] = i;
        }
    }
    // support-sharing neighbour range [jlo, jhi] of every function, per patch and direction
    rp.rngOff.assign(np * 3, 0);
    for (size_t pi = 0; pi < np; ++pi) {
        const HostPatch& P = pd.patches[pi];
        const DevPatch& D = L.dev[pi];
        for (int a = 0; a < 3; ++a) {
            rp.rngOff[pi * 3 + a] = (long long)rp.rng.size();
            if (a >= d) continue;
            const int* elo = L.ibuf.data() + D.doff[a];
            const int* ehi = elo + D.n[a];
            const size_t base = rp.rng.size();
            rp.rng.resize(base + 2 * size_t(P.nd[a]));
            for (int i = 0; i < P.nd[a]; ++i) {
                int first = -1, last = -2;
                for (int j = std::max(0, i - D.p[a]); j <= std::min(P.nd[a] - 1, i + D.p[a]); ++j) {
                    const bool share = std::max(elo[i], elo[j]) <= std::min(ehi[i], ehi[j]);
                    if (!share) continue;
                    if (first < 0) first = j;
                    else if (j != last + 1) return false;  // not a contiguous range
                    last = j;
                }
                rp.rng[base + i] = first;
                rp.rng[base + P.nd[a] + i] = last;
            }
        }
    }
    return true;
}

// Problems without interfaces (single patches, batches of independent patches): every free row has
// one pre-image, and a patch's free dofs are numbered in its local lexicographic order, so a row's
// columns come out ascending from its neighbour box with no sorting and no multi-source slots. The
// neighbour set per direction is the support-sharing range the generic path tests pair by pair, and
// the loop order (and so the lift order) is the same. Returns false (generic path) if an assumption
// does not hold.
static bool buildPatternSingle(const ProblemDesc& pd, const DofMap& map, const Layout& L, Pattern& pat) {
    const int n = map.freeSize;
    const int d = pd.dim;
    RowPlan rp;
    if (!rowPlanSingle(pd, map, L, rp)) return false;
    const std::vector<int>& rowPatch = rp.rowPatch;
    const std::vector<int>& rowLoc = rp.rowLoc;
    auto box = [&](int I, int c[3], int lo[3], int hi[3]) {
        const int pi = rowPatch[I];
        const HostPatch& P = pd.patches[pi];
        int r = rowLoc[I];
        for (int a = 0; a < 3; ++a) {
            if (a < d) {
                c[a] = r % P.nd[a];
                r /= P.nd[a];
                lo[a] = rp.rng[rp.rngOff[size_t(pi) * 3 + a] + c[a]];
                hi[a] = rp.rng[rp.rngOff[size_t(pi) * 3 + a] + P.nd[a] + c[a]];
            } else {
                c[a] = lo[a] = hi[a] = 0;
            }
        }
    };
    std::vector<long long> nslot(n + 1, 0), nlift(n + 1, 0);
#pragma omp parallel for schedule(dynamic, 512)
    for (int I = 0; I < n; ++I) {
        const HostPatch& P = pd.patches[rowPatch[I]];
        int c[3], lo[3], hi[3];
        box(I, c, lo, hi);
        long long ns = 0, nl = 0;
        for (int z = lo[2]; z <= hi[2]; ++z)
            for (int y = lo[1]; y <= hi[1]; ++y)
                for (int x = lo[0]; x <= hi[0]; ++x) {
                    const int lj = x + P.nd[0] * (y + (d == 3 ? P.nd[1] * z : 0));
                    if (map.index[P.offset + lj] < n) ++ns;
                    else ++nl;
                }
        nslot[I + 1] = ns;
        nlift[I + 1] = nl;
    }
    for (int i = 0; i < n; ++i) {
        nslot[i + 1] += nslot[i];
        nlift[i + 1] += nlift[i];
    }
    if (nslot[n] >= (1LL << 31)) throw std::invalid_argument("more than 2^31 non-zeros");
    pat.ptr.resize(n + 1);
    for (int i = 0; i <= n; ++i) pat.ptr[i] = int(nslot[i]);
    pat.col.resize(nslot[n]);
    pat.src.resize(nslot[n]);
    pat.fptr.resize(n + 1);
    pat.fband.resize(nlift[n]);
    pat.fbidx.resize(nlift[n]);
    for (int i = 0; i <= n; ++i) pat.fptr[i] = uint32_t(nlift[i]);
    int ordered = 1;
#pragma omp parallel for schedule(dynamic, 512) reduction(& : ordered)
    for (int I = 0; I < n; ++I) {
        const int pi = rowPatch[I];
        const HostPatch& P = pd.patches[pi];
        const DevPatch& D = L.dev[pi];
        int c[3], lo[3], hi[3];
        box(I, c, lo, hi);
        const long long n0W = (long long)D.n[0] * D.W[0], n1W = (long long)D.n[1] * D.W[1];
        long long s = nslot[I], f = nlift[I];
        int prev = -1;
        for (int z = lo[2]; z <= hi[2]; ++z)
            for (int y = lo[1]; y <= hi[1]; ++y)
                for (int x = lo[0]; x <= hi[0]; ++x) {
                    const int lj = x + P.nd[0] * (y + (d == 3 ? P.nd[1] * z : 0));
                    const int J = map.index[P.offset + lj];
                    long long b = (long long)c[0] * D.W[0] + (x - c[0] + D.p[0]);
                    b += ((long long)c[1] * D.W[1] + (y - c[1] + D.p[1])) * n0W;
                    if (d == 3) b += ((long long)c[2] * D.W[2] + (z - c[2] + D.p[2])) * n0W * n1W;
                    b += D.band_off;
                    if (J < n) {
                        if (J <= prev) ordered = 0;
                        prev = J;
                        pat.col[s] = J;
                        pat.src[s] = uint32_t(b);
                        ++s;
                    } else {
                        pat.fband[f] = uint32_t(b);
                        pat.fbidx[f] = uint32_t(J - n);
                        ++f;
                    }
                }
    }
    if (!ordered) return false;
    pat.ovf_ptr.assign(1, 0);
    pat.lptr.resize(n + 1);
    for (int i = 0; i <= n; ++i) pat.lptr[i] = uint32_t(i);
    pat.lidx.resize(n);
    for (int I = 0; I < n; ++I) pat.lidx[I] = uint32_t(L.dev[rowPatch[I]].lvec_off + rowLoc[I]);
    return true;
}

void buildPattern(const ProblemDesc& pd, const DofMap& map, const Layout& L, Pattern& pat, int nthreads) {
    const int n = map.freeSize;
    pat = Pattern();
    pat.n = n;
    if (pd.ifaces.empty()) {
#ifdef _OPENMP
        if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
        if (buildPatternSingle(pd, map, L, pat)) return;
        pat = Pattern();
        pat.n = n;
    }
    // pre-images of every free global dof
    std::vector<int> preptr(n + 1, 0), preloc, prepatch;
    for (size_t pi = 0; pi < pd.patches.size(); ++pi) {
        const HostPatch& P = pd.patches[pi];
        for (int i = 0; i < P.ndofs; ++i) {
            const int J = map.index[P.offset + i];
            if (J < n) ++preptr[J + 1];
        }
    }
    for (int i = 0; i < n; ++i) preptr[i + 1] += preptr[i];
    preloc.resize(preptr[n]);
    prepatch.resize(preptr[n]);
    {
        std::vector<int> fill(preptr.begin(), preptr.end() - 1);
        for (size_t pi = 0; pi < pd.patches.size(); ++pi) {
            const HostPatch& P = pd.patches[pi];
            for (int i = 0; i < P.ndofs; ++i) {
                const int J = map.index[P.offset + i];
                if (J < n) { preloc[fill[J]] = P.offset + i; prepatch[fill[J]++] = int(pi); }
            }
        }
    }
    // pass 1: counts
    std::vector<long long> nslot(n + 1, 0), nsrc(n + 1, 0), nlift(n + 1, 0);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
    {
        RowScratch rs;
        bool sorted;
#pragma omp for schedule(dynamic, 256)
        for (int I = 0; I < n; ++I) {
            rowEntries(pd, map, L, preptr, preloc, prepatch, I, rs, sorted);
            long long ns = 0, extra = 0;
            for (size_t k = 0; k < rs.ent.size();) {
                size_t e = k + 1;
                while (e < rs.ent.size() && rs.ent[e].first == rs.ent[k].first) ++e;
                ++ns;
                if (e - k > 1) extra += (long long)(e - k);
                k = e;
            }
            nslot[I + 1] = ns;
            nsrc[I + 1] = extra;
            nlift[I + 1] = (long long)rs.lift.size();
        }
    }
    for (int i = 0; i < n; ++i) { nslot[i + 1] += nslot[i]; nsrc[i + 1] += nsrc[i]; nlift[i + 1] += nlift[i]; }
    if (nslot[n] >= (1LL << 31)) throw std::invalid_argument("more than 2^31 non-zeros");
    pat.ptr.resize(n + 1);
    for (int i = 0; i <= n; ++i) pat.ptr[i] = int(nslot[i]);
    pat.col.resize(nslot[n]);
    pat.src.resize(nslot[n]);
    pat.ovf_idx.resize(nsrc[n]);
    pat.fptr.resize(n + 1);
    pat.fband.resize(nlift[n]);
    pat.fbidx.resize(nlift[n]);
    for (int i = 0; i <= n; ++i) pat.fptr[i] = uint32_t(nlift[i]);
    // overflow pointer list: one entry per multi-source slot (filled in pass 2 per row, in order)
    std::vector<long long> novf(n + 1, 0);
#pragma omp parallel
    {
        RowScratch rs;
        bool sorted;
        std::vector<uint32_t> optr;
#pragma omp for schedule(dynamic, 256)
        for (int I = 0; I < n; ++I) {
            rowEntries(pd, map, L, preptr, preloc, prepatch, I, rs, sorted);
            long long s = nslot[I], o = nsrc[I];
            long long nov = 0;
            for (size_t k = 0; k < rs.ent.size();) {
                size_t e = k + 1;
                while (e < rs.ent.size() && rs.ent[e].first == rs.ent[k].first) ++e;
                pat.col[s] = rs.ent[k].first;
                if (e - k == 1) pat.src[s] = rs.ent[k].second;
                else {
                    pat.src[s] = Pattern::kMulti;  // patched below with the overflow slot index
                    for (size_t m = k; m < e; ++m) pat.ovf_idx[o++] = rs.ent[m].second;
                    ++nov;
                }
                ++s;
                k = e;
            }
            novf[I + 1] = nov;
            long long f = nlift[I];
            for (auto& lt : rs.lift) { pat.fband[f] = lt.first; pat.fbidx[f] = lt.second; ++f; }
        }
    }
    for (int i = 0; i < n; ++i) novf[i + 1] += novf[i];
    if (novf[n] >= (long long)Pattern::kMulti) throw std::invalid_argument("too many multi-source slots");
    pat.ovf_ptr.assign(novf[n] + 1, 0);
    // number the multi-source slots in slot order (row by row, columns ascending)
    {
        long long ov = 0;
        for (int I = 0; I < n; ++I)
            for (int s = pat.ptr[I]; s < pat.ptr[I + 1]; ++s)
                if (pat.src[s] == Pattern::kMulti) pat.src[s] = Pattern::kMulti | uint32_t(ov++);
    }
    // second sweep: the overflow ranges of each row's multi-source slots, same order
    if (novf[n] > 0) {
#pragma omp parallel
        {
            RowScratch rs;
            bool sorted;
#pragma omp for schedule(dynamic, 256)
            for (int I = 0; I < n; ++I) {
                if (novf[I + 1] == novf[I]) continue;
                rowEntries(pd, map, L, preptr, preloc, prepatch, I, rs, sorted);
                long long ov = novf[I], o = nsrc[I];
                for (size_t k = 0; k < rs.ent.size();) {
                    size_t e = k + 1;
                    while (e < rs.ent.size() && rs.ent[e].first == rs.ent[k].first) ++e;
                    if (e - k > 1) { pat.ovf_ptr[ov++] = uint32_t(o); o += (long long)(e - k); }
                    k = e;
                }
            }
        }
        pat.ovf_ptr[novf[n]] = uint32_t(nsrc[n]);
    }
    // load-vector sources
    pat.lptr.assign(n + 1, 0);
    for (int i = 0; i <= n; ++i) pat.lptr[i] = uint32_t(preptr[i]);
    pat.lidx.resize(preptr[n]);
    for (int I = 0; I < n; ++I)
        for (int k = preptr[I]; k < preptr[I + 1]; ++k) {
            const int pi = prepatch[k];
            pat.lidx[k] = uint32_t(L.dev[pi].lvec_off + (preloc[k] - pd.patches[pi].offset));
        }
}

// ---------------------------------------------------------------------------------------------
// values of one Dirichlet side at its boundary dofs (sideDofs order); `par`: OpenMP inside the side
static std::vector<double> sideValues(const ProblemDesc& pd, size_t si, bool par) {
    const int dim = pd.dim;
    const HostPatch& P = pd.patches[pd.dsides[si]];
    const int side = pd.dsides[si + 1];
    const int dir = (side - 1) / 2, parity = (side - 1) % 2;
    int odirs[2], no = 0;
    for (int k = 0; k < dim; ++k) if (k != dir) odirs[no++] = k;
    std::vector<double> gv[2];
    int npts = 1;
    for (int o = 0; o < no; ++o) { gv[o] = P.b[odirs[o]].greville(); npts *= int(gv[o].size()); }
    const double fixv = parity ? P.b[dir].t.back() : P.b[dir].t.front();
    const FieldParams& F = pd.fieldsOf(pd.dsides[si]);
    // the geometry map on the side's Greville grid, sum-factorised: the geometry control points
    // contracted with the basis of the fixed direction at the side's parameter, then with the
    // basis of one side direction at a time (each evaluated once per abscissa)
    const int ng[3] = {P.g[0].n(), dim > 1 ? P.g[1].n() : 1, dim > 2 ? P.g[2].n() : 1};
    const long long gstride[3] = {1, ng[0], (long long)ng[0] * ng[1]};
    auto basisAt = [](const Basis1D& B, double u, int& first, std::vector<double>& v) {
        std::vector<double> buf(2 * (B.p + 1));
        const int sp = B.span(u);
        B.eval(sp, u, buf.data());
        first = sp - B.p;
        v.assign(buf.begin(), buf.begin() + B.p + 1);
    };
    int ffirst;
    std::vector<double> fv;
    basisAt(P.g[dir], fixv, ffirst, fv);
    // F[j0 + n0 j1][m] over the control points of the side directions
    const int n0 = ng[odirs[0]], n1 = no > 1 ? ng[odirs[1]] : 1;
    std::vector<double> Fc(size_t(n0) * n1 * dim, 0.0);
    for (int j1 = 0; j1 < n1; ++j1)
        for (int j0 = 0; j0 < n0; ++j0)
            for (int c = 0; c <= P.g[dir].p; ++c) {
                long long gi = (long long)j0 * gstride[odirs[0]] + (long long)(ffirst + c) * gstride[dir];
                if (no > 1) gi += (long long)j1 * gstride[odirs[1]];
                for (int m = 0; m < dim; ++m) Fc[(size_t(j0) + size_t(n0) * j1) * dim + m] += fv[c] * P.coefs[gi * dim + m];
            }
    // direction odirs[0] at its abscissae: G[a + na j1][m]
    const int na = int(gv[0].size()), nb = no > 1 ? int(gv[1].size()) : 1;
    std::vector<double> G(size_t(na) * n1 * dim, 0.0);
    for (int a = 0; a < na; ++a) {
        int f0;
        std::vector<double> v0;
        basisAt(P.g[odirs[0]], gv[0][a], f0, v0);
        for (int j1 = 0; j1 < n1; ++j1)
            for (int i = 0; i < int(v0.size()); ++i)
                for (int m = 0; m < dim; ++m)
                    G[(size_t(a) + size_t(na) * j1) * dim + m] += v0[i] * Fc[(size_t(f0 + i) + size_t(n0) * j1) * dim + m];
    }
    // direction odirs[1] (3D) at its abscissae: the points x[a + na b][m]
    std::vector<double> X(size_t(npts) * dim, 0.0);
    if (no > 1) {
        for (int b = 0; b < nb; ++b) {
            int f1;
            std::vector<double> v1;
            basisAt(P.g[odirs[1]], gv[1][b], f1, v1);
            for (int a = 0; a < na; ++a)
                for (int j = 0; j < int(v1.size()); ++j)
                    for (int m = 0; m < dim; ++m)
                        X[(size_t(a) + size_t(na) * b) * dim + m] += v1[j] * G[(size_t(a) + size_t(na) * (f1 + j)) * dim + m];
        }
    } else {
        X = G;
    }
    std::vector<double> f(npts);
#pragma omp parallel for schedule(static) if (par && npts >= 4096)
    for (int i = 0; i < npts; ++i) f[i] = evalU(F, &X[size_t(i) * dim]);
    // tensor collocation solve, one direction at a time (LU with partial pivoting). The
    // collocation matrix is banded (p sub- and super-diagonals); with pivoting inside the band the
    // factors stay within w = 3(p+1) of the diagonal, so the loops skip only exact zeros.
    int stride = 1;
    for (int o = 0; o < no; ++o) {
        const Basis1D& B = P.b[odirs[o]];
        const int n = B.n();
        const int w = 3 * (B.p + 1);
        std::vector<double> M(size_t(n) * n, 0.0), buf(2 * (B.p + 1));
        for (int a = 0; a < n; ++a) {
            const double u = gv[o][a];
            const int s = B.span(u);
            B.eval(s, u, buf.data());
            for (int r = 0; r <= B.p; ++r) M[size_t(a) * n + (s - B.p + r)] = buf[r];
        }
        std::vector<int> piv(n);
        for (int k = 0; k < n; ++k) {
            int pm = k;
            for (int i = k + 1; i < std::min(n, k + B.p + 2); ++i)
                if (std::fabs(M[size_t(i) * n + k]) > std::fabs(M[size_t(pm) * n + k])) pm = i;
            piv[k] = pm;
            const int jlo = std::max(0, k - w), jhi = std::min(n, k + w + 1);
            if (pm != k)
                for (int j = jlo; j < jhi; ++j) std::swap(M[size_t(k) * n + j], M[size_t(pm) * n + j]);
            const double dk = M[size_t(k) * n + k];
            for (int i = k + 1; i < std::min(n, k + 2 * B.p + 2); ++i) {
                const double l = M[size_t(i) * n + k] / dk;
                if (l == 0.0) continue;
                M[size_t(i) * n + k] = l;
                for (int j = k + 1; j < jhi; ++j) M[size_t(i) * n + j] -= l * M[size_t(k) * n + j];
            }
        }
        const int outer = npts / (n * stride);
#pragma omp parallel for collapse(2) schedule(static) if (par)
        for (int ob = 0; ob < outer; ++ob)
            for (int ib = 0; ib < stride; ++ib) {
                std::vector<double> col(n);
                for (int a = 0; a < n; ++a) col[a] = f[size_t(ob) * n * stride + size_t(a) * stride + ib];
                for (int k = 0; k < n; ++k) std::swap(col[k], col[piv[k]]);
                for (int i = 0; i < n; ++i)
                    for (int j = std::max(0, i - w); j < i; ++j) col[i] -= M[size_t(i) * n + j] * col[j];
                for (int i = n - 1; i >= 0; --i) {
                    for (int j = i + 1; j < std::min(n, i + w + 1); ++j) col[i] -= M[size_t(i) * n + j] * col[j];
                    col[i] /= M[size_t(i) * n + i];
                }
                for (int a = 0; a < n; ++a) f[size_t(ob) * n * stride + size_t(a) * stride + ib] = col[a];
            }
        stride *= n;
    }
    return f;
}

// geometry map of patch P at the parameter xi: point x and Jacobian J[m][k] = d x_m / d xi_k
static void geoMapHost(const HostPatch& P, const double* xi, double* x, double J[3][3]) {
    const int d = P.dim;
    int first[3] = {0, 0, 0}, pp[3] = {0, 0, 0}, ng[3] = {1, 1, 1};
    double v[3][32], dv[3][32];
    double buf[64];
    for (int k = 0; k < 3; ++k) {
        v[k][0] = 1.0;
        dv[k][0] = 0.0;
    }
    for (int k = 0; k < d; ++k) {
        const Basis1D& B = P.g[k];
        const int sp = B.span(xi[k]);
        B.eval(sp, xi[k], buf);
        first[k] = sp - B.p;
        pp[k] = B.p;
        ng[k] = B.n();
        for (int r = 0; r <= B.p; ++r) {
            v[k][r] = buf[r];
            dv[k][r] = buf[B.p + 1 + r];
        }
    }
    for (int m = 0; m < d; ++m) {
        x[m] = 0.0;
        for (int k = 0; k < d; ++k) J[m][k] = 0.0;
    }
    for (int c = 0; c <= pp[2]; ++c)
        for (int b = 0; b <= pp[1]; ++b)
            for (int a = 0; a <= pp[0]; ++a) {
                const long long gi = first[0] + a + (long long)ng[0] * (first[1] + b + (long long)ng[1] * (first[2] + c));
                const int idx[3] = {a, b, c};
                double w = 1.0, dw[3];
                for (int k = 0; k < d; ++k) w *= v[k][idx[k]];
                for (int k = 0; k < d; ++k) {
                    dw[k] = dv[k][idx[k]];
                    for (int l = 0; l < d; ++l)
                        if (l != k) dw[k] *= v[l][idx[l]];
                }
                for (int m = 0; m < d; ++m) {
                    const double cm = P.coefs[size_t(gi) * d + m];
                    x[m] += w * cm;
                    for (int k = 0; k < d; ++k) J[m][k] += dw[k] * cm;
                }
            }
}

// Dirichlet values by L2 projection (gsAssembler::computeDirichletDofsL2Proj,
// gsAssembler.hpp:392-534): one mass system over all eliminated dofs, assembled on the elements of
// every Dirichlet side with p_k + 1 Gauss points in each side direction (the fixed direction
// weighs 1), the weight times |det J| of the full geometry Jacobian at the boundary point (the
// reference's map data carries no side, so that is its measure), the boundary data u at the
// mapped point; solved by Jacobi-preconditioned CG to round-off (the reference: Eigen's
// diagonal-preconditioned CG at its default tolerance)
static void dirichletValuesL2(const ProblemDesc& pd, const DofMap& map, std::vector<double>& ddof) {
    const int nb = map.boundarySize;
    ddof.assign(nb, 0.0);
    if (nb == 0) return;
    const int dim = pd.dim;
    const int nsides = int(pd.dsides.size() / 2);
    struct Trip {
        int i, j;
        double v;
    };
    std::vector<std::vector<Trip>> trips(nsides);
    std::vector<std::vector<std::pair<int, double>>> rhsParts(nsides);
#pragma omp parallel for schedule(dynamic, 1) if (nsides >= 2)
    for (int sd = 0; sd < nsides; ++sd) {
        const HostPatch& P = pd.patches[pd.dsides[2 * sd]];
        const int side = pd.dsides[2 * sd + 1];
        const int dir = (side - 1) / 2, parity = (side - 1) % 2;
        int od[2] = {0, 0}, no = 0;
        for (int k = 0; k < dim; ++k)
            if (k != dir) od[no++] = k;
        const double fixv = parity ? P.b[dir].t.back() : P.b[dir].t.front();
        const FieldParams& F = pd.fieldsOf(pd.dsides[2 * sd]);
        std::vector<double> gx[2], gw[2];
        for (int o = 0; o < no; ++o) gaussLegendre(P.b[od[o]].p + 1, gx[o], gw[o]);
        const int ne0 = P.b[od[0]].nelem(), ne1 = no > 1 ? P.b[od[1]].nelem() : 1;
        const int sfix = P.b[dir].span(fixv);
        std::vector<double> fixBuf(2 * (P.b[dir].p + 1));
        P.b[dir].eval(sfix, fixv, fixBuf.data());
        std::vector<Trip>& T = trips[sd];
        std::vector<std::pair<int, double>>& R = rhsParts[sd];
        for (int e1 = 0; e1 < ne1; ++e1)
            for (int e0 = 0; e0 < ne0; ++e0) {
                const int e[2] = {e0, e1};
                int spn[3];
                double lo[3], hi[3];
                spn[dir] = sfix;
                for (int o = 0; o < no; ++o) {
                    const Basis1D& B = P.b[od[o]];
                    spn[od[o]] = B.elementSpan(e[o]);
                    lo[o] = B.breaks[e[o]];
                    hi[o] = B.breaks[e[o] + 1];
                }
                // eliminated dofs active on this element (local slot, boundary index)
                int pp[3] = {0, 0, 0}, nloc[3] = {1, 1, 1};
                for (int k = 0; k < dim; ++k) {
                    pp[k] = P.b[k].p;
                    nloc[k] = P.b[k].n();
                }
                std::vector<std::pair<int, int>> act;
                for (int c = 0; c <= (dim > 2 ? pp[2] : 0); ++c)
                    for (int b = 0; b <= pp[1]; ++b)
                        for (int a = 0; a <= pp[0]; ++a) {
                            const int i0 = spn[0] - pp[0] + a, i1 = spn[1] - pp[1] + b;
                            const int i2 = dim > 2 ? spn[2] - pp[2] + c : 0;
                            const int loc = i0 + nloc[0] * (i1 + nloc[1] * i2);
                            const int gl = map.index[P.offset + loc];
                            if (gl >= map.freeSize) act.push_back({a + (pp[0] + 1) * (b + (pp[1] + 1) * c), gl - map.freeSize});
                        }
                if (act.empty()) continue;
                const int na = int(act.size());
                std::vector<double> Me(size_t(na) * na, 0.0), re(na, 0.0), vals(na);
                const int nq0 = int(gx[0].size()), nq1 = no > 1 ? int(gx[1].size()) : 1;
                for (int q1 = 0; q1 < nq1; ++q1)
                    for (int q0 = 0; q0 < nq0; ++q0) {
                        double xi[3] = {0, 0, 0};
                        xi[dir] = fixv;
                        double w = 1.0;  // the fixed direction: weight 2 on a zero-length interval, factor 1/2
                        const int q[2] = {q0, q1};
                        for (int o = 0; o < no; ++o) {
                            const double h = 0.5 * (hi[o] - lo[o]);
                            xi[od[o]] = lo[o] + h * (gx[o][q[o]] + 1.0);
                            w *= (h == 0.0 ? 0.5 : h) * gw[o][q[o]];
                        }
                        double x[3], J[3][3];
                        geoMapHost(P, xi, x, J);
                        double det;
                        if (dim == 3)
                            det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) -
                                  J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                                  J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
                        else
                            det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
                        const double wk = w * std::fabs(det);
                        const double g = evalU(F, x);
                        double bv[3][32];
                        double buf[64];
                        for (int k = 0; k < dim; ++k) {
                            if (k == dir) {
                                for (int r = 0; r <= pp[k]; ++r) bv[k][r] = fixBuf[r];
                            } else {
                                P.b[k].eval(spn[k], xi[k], buf);
                                for (int r = 0; r <= pp[k]; ++r) bv[k][r] = buf[r];
                            }
                        }
                        for (int i = 0; i < na; ++i) {
                            int sl = act[i].first;
                            const int a = sl % (pp[0] + 1);
                            sl /= pp[0] + 1;
                            const int b = sl % (pp[1] + 1);
                            const int c = sl / (pp[1] + 1);
                            double v = bv[0][a] * bv[1][b];
                            if (dim > 2) v *= bv[2][c];
                            vals[i] = v;
                        }
                        for (int i = 0; i < na; ++i) {
                            for (int j = 0; j < na; ++j) Me[size_t(i) * na + j] += wk * vals[i] * vals[j];
                            re[i] += wk * vals[i] * g;
                        }
                    }
                for (int i = 0; i < na; ++i) {
                    for (int j = 0; j < na; ++j) T.push_back({act[i].second, act[j].second, Me[size_t(i) * na + j]});
                    R.push_back({act[i].second, re[i]});
                }
            }
    }
    // CSR of the projection matrix (entries summed in side order, then element order)
    std::vector<Trip> all;
    std::vector<double> rhs(nb, 0.0);
    for (int sd = 0; sd < nsides; ++sd) {
        all.insert(all.end(), trips[sd].begin(), trips[sd].end());
        for (auto& pr : rhsParts[sd]) rhs[pr.first] += pr.second;
    }
    std::stable_sort(all.begin(), all.end(), [](const Trip& a, const Trip& b) { return a.i != b.i ? a.i < b.i : a.j < b.j; });
    std::vector<int> ptr(nb + 1, 0), col;
    std::vector<double> val;
    for (size_t k = 0; k < all.size();) {
        size_t e = k;
        double v = 0.0;
        while (e < all.size() && all[e].i == all[k].i && all[e].j == all[k].j) v += all[e++].v;
        col.push_back(all[k].j);
        val.push_back(v);
        ++ptr[all[k].i + 1];
        k = e;
    }
    for (int i = 0; i < nb; ++i) ptr[i + 1] += ptr[i];
    // Jacobi-PCG to round-off
    std::vector<double> dinv(nb, 0.0), r = rhs, z(nb), p(nb), t(nb);
    for (int i = 0; i < nb; ++i)
        for (int k = ptr[i]; k < ptr[i + 1]; ++k)
            if (col[k] == i && val[k] != 0.0) dinv[i] = 1.0 / val[k];
    double bb = 0.0;
    for (double v : rhs) bb += v * v;
    if (bb == 0.0) return;
    for (int i = 0; i < nb; ++i) z[i] = dinv[i] * r[i];
    p = z;
    double rz = 0.0;
    for (int i = 0; i < nb; ++i) rz += r[i] * z[i];
    for (int it = 0; it < 10 * nb + 100; ++it) {
        double pt = 0.0;
        for (int i = 0; i < nb; ++i) {
            double acc = 0.0;
            for (int k = ptr[i]; k < ptr[i + 1]; ++k) acc += val[k] * p[col[k]];
            t[i] = acc;
            pt += p[i] * acc;
        }
        const double a = rz / pt;
        double rr = 0.0;
        for (int i = 0; i < nb; ++i) {
            ddof[i] += a * p[i];
            r[i] -= a * t[i];
            rr += r[i] * r[i];
        }
        if (rr <= 1e-30 * bb) break;
        double rzn = 0.0;
        for (int i = 0; i < nb; ++i) {
            z[i] = dinv[i] * r[i];
            rzn += r[i] * z[i];
        }
        const double beta = rzn / rz;
        rz = rzn;
        for (int i = 0; i < nb; ++i) p[i] = z[i] + beta * p[i];
    }
}

void dirichletValues(const ProblemDesc& pd, const DofMap& map, std::vector<double>& ddof) {
    if (pd.dirL2) {
        dirichletValuesL2(pd, map, ddof);
        return;
    }
    ddof.assign(map.boundarySize, 0.0);
    const int nsides = int(pd.dsides.size() / 2);
    // one side per thread; threads inside the side only for a single side (the work of one side is
    // a few milliseconds at most, below what OpenMP regions inside it would save)
    const bool across = nsides >= 2;
    std::vector<std::vector<double>> vals(nsides);
#pragma omp parallel for schedule(dynamic, 1) if (across)
    for (int k = 0; k < nsides; ++k) vals[k] = sideValues(pd, size_t(2 * k), !across);
    // scatter in side order (a dof on two sides takes the later side's value)
    std::vector<int> bd;
    for (int k = 0; k < nsides; ++k) {
        const HostPatch& P = pd.patches[pd.dsides[2 * k]];
        sideDofs(P, pd.dsides[2 * k + 1], bd);
        for (size_t l = 0; l < bd.size(); ++l) {
            const int gi = map.index[P.offset + bd[l]];
            ddof[gi - map.freeSize] = vals[k][l];
        }
    }
}

void problemFromC(const void* ptr, ProblemDesc& pd) {
    const gsgpu_problem* pr = static_cast<const gsgpu_problem*>(ptr);
    if (!pr || (pr->dim != 2 && pr->dim != 3) || pr->npatches < 1)
        throw std::invalid_argument("problem: dim must be 2 or 3 and npatches >= 1");
    pd = ProblemDesc();
    pd.dim = pr->dim;
    const double* kp = pr->knots;
    const double* gkp = pr->gknots;
    const double* cp = pr->coefs;
    int off = 0;
    for (int i = 0; i < pr->npatches; ++i) {
        HostPatch P;
        P.dim = pr->dim;
        long long ngeo = 1;
        P.ndofs = 1;
        for (int k = 0; k < pr->dim; ++k) {
            P.b[k].init(pr->degree[3 * i + k], kp, pr->nknots[3 * i + k]);
            kp += pr->nknots[3 * i + k];
            P.g[k].init(pr->gdegree[3 * i + k], gkp, pr->gnknots[3 * i + k]);
            gkp += pr->gnknots[3 * i + k];
            if (P.g[k].t.front() != P.b[k].t.front() || P.g[k].t.back() != P.b[k].t.back())
                throw std::invalid_argument("geometry and discretisation bases must share the parameter domain");
            P.nd[k] = P.b[k].n();
            P.ndofs *= P.nd[k];
            ngeo *= P.g[k].n();
        }
        P.coefs.assign(cp, cp + ngeo * pr->dim);
        cp += ngeo * pr->dim;
        P.offset = off;
        off += P.ndofs;
        pd.patches.push_back(std::move(P));
    }
    for (int i = 0; i < pr->ninterfaces; ++i) {
        const int* f = pr->interfaces + 4 * i;
        if (f[0] < 0 || f[0] >= pr->npatches || f[2] < 0 || f[2] >= pr->npatches || f[1] < 1 || f[1] > 2 * pr->dim ||
            f[3] < 1 || f[3] > 2 * pr->dim)
            throw std::invalid_argument("interface: bad patch or side index");
        pd.ifaces.insert(pd.ifaces.end(), f, f + 4);
    }
    for (int i = 0; i < pr->ndirichlet; ++i) {
        const int* f = pr->dirichlet + 2 * i;
        if (f[0] < 0 || f[0] >= pr->npatches || f[1] < 1 || f[1] > 2 * pr->dim)
            throw std::invalid_argument("dirichlet: bad patch or side index");
        pd.dsides.insert(pd.dsides.end(), f, f + 2);
    }
    // Neumann sides: one condition per side, on a boundary side (gsBoundaryConditions holds one
    // condition per side; interface sides are not boundaries)
    for (int i = 0; i < pr->nneumann; ++i) {
        const int* f = pr->neumann + 2 * i;
        if (f[0] < 0 || f[0] >= pr->npatches || f[1] < 1 || f[1] > 2 * pr->dim)
            throw std::invalid_argument("neumann: bad patch or side index");
        auto onList = [&](const std::vector<int>& v, int stride) {
            for (size_t k = 0; k < v.size(); k += size_t(stride))
                if (v[k] == f[0] && v[k + 1] == f[1]) return true;
            return false;
        };
        if (onList(pd.dsides, 2) || onList(pd.nsides, 2))
            throw std::invalid_argument("neumann: side already carries a boundary condition");
        for (size_t k = 0; k < pd.ifaces.size(); k += 4)
            if ((pd.ifaces[k] == f[0] && pd.ifaces[k + 1] == f[1]) || (pd.ifaces[k + 2] == f[0] && pd.ifaces[k + 3] == f[1]))
                throw std::invalid_argument("neumann: side is an interface");
        pd.nsides.insert(pd.nsides.end(), f, f + 2);
    }
    FieldParams& F = pd.fields;
    F = FieldParams{};
    F.dim = pr->dim;
    F.fourier = pr->kappa_fourier ? 1 : 0;
    F.kconst = pr->kappa_const;
    F.alpha = F.fourier ? pr->kappa_alpha : 0.0;
    F.scale = pr->kappa_scale;
    F.nmodes = F.fourier ? pr->kappa_nmodes : 0;
    if (F.nmodes < 0 || F.nmodes > kMaxModes) throw std::invalid_argument("kappa: too many Fourier modes");
    for (int m = 0; m < F.nmodes; ++m) {
        F.amp[m] = pr->kappa_amp[m];
        F.phase[m] = pr->kappa_phase[m];
        F.cph[m] = std::cos(F.phase[m]);
        F.sph[m] = std::sin(F.phase[m]);
        for (int k = 0; k < 3; ++k) {
            F.kk[m][k] = k < pr->dim ? pr->kappa_k[3 * m + k] : 0;
            if (F.kk[m][k] < 0 || F.kk[m][k] > 8) throw std::invalid_argument("kappa: wave numbers must be in [0, 8]");
        }
    }
    F.kmax = 0;
    for (int m = 0; m < F.nmodes; ++m)
        for (int k = 0; k < 3; ++k) F.kmax = std::max(F.kmax, F.kk[m][k]);
    F.ufreq = pr->ufreq;
    pd.quA = pr->quA;
    pd.quB = pr->quB;
    if (pr->dirichlet_strategy != 0 && pr->dirichlet_strategy != 1)
        throw std::invalid_argument("dirichlet_strategy must be interpolation (0) or L2 projection (1)");
    pd.dirL2 = pr->dirichlet_strategy;
}

void batchFromDescs(std::vector<ProblemDesc>& items, ProblemDesc& pd) {
    if (items.empty()) throw std::invalid_argument("batch: count must be >= 1");
    pd = ProblemDesc();
    int off = 0;
    for (size_t j = 0; j < items.size(); ++j) {
        ProblemDesc& one = items[j];
        if (one.patches.size() != 1 || !one.ifaces.empty())
            throw std::invalid_argument("batch: every problem must be a single patch without interfaces");
        if (j == 0) {
            pd.dim = one.dim;
            pd.quA = one.quA;
            pd.quB = one.quB;
            pd.fields = one.fields;
            pd.dirL2 = one.dirL2;
        } else if (one.dim != pd.dim || one.quA != pd.quA || one.quB != pd.quB || one.dirL2 != pd.dirL2) {
            throw std::invalid_argument(
                "batch: dimension, quadrature rule and Dirichlet strategy must agree across problems");
        }
        HostPatch P = std::move(one.patches[0]);
        P.field = int(j);
        P.offset = off;
        off += P.ndofs;
        pd.patches.push_back(std::move(P));
        for (size_t i = 0; i < one.dsides.size(); i += 2) {
            pd.dsides.push_back(int(j));
            pd.dsides.push_back(one.dsides[i + 1]);
        }
        for (size_t i = 0; i < one.nsides.size(); i += 2) {
            pd.nsides.push_back(int(j));
            pd.nsides.push_back(one.nsides[i + 1]);
        }
        pd.pfields.push_back(one.fields);
    }
}

void batchFromC(int count, const void* ptr, ProblemDesc& pd) {
    const gsgpu_problem* pr = static_cast<const gsgpu_problem*>(ptr);
    if (!pr || count < 1) throw std::invalid_argument("batch: count must be >= 1");
    std::vector<ProblemDesc> items(static_cast<size_t>(count));
    for (int j = 0; j < count; ++j) problemFromC(&pr[j], items[size_t(j)]);
    batchFromDescs(items, pd);
}

void buildNeumann(const ProblemDesc& pd, const Layout& L, int block, NeumannPlan& np) {
    np = NeumannPlan();
    const int dim = pd.dim;
    const int nside = int(pd.nsides.size() / 2);
    std::unordered_map<long long, size_t> slot;  // load-vector slot -> entry of np.dofs
    for (int k = 0; k < nside; ++k) {
        const int pi = pd.nsides[2 * k], side = pd.nsides[2 * k + 1];
        const HostPatch& P = pd.patches[size_t(pi)];
        const DevPatch& D = L.dev[size_t(pi)];
        NeuSide S{};
        S.patch = pi;
        S.dir = (side - 1) / 2;
        S.upper = (side - 1) % 2;
        int no = 0;
        S.t[1] = -1;
        for (int a = 0; a < dim; ++a)
            if (a != S.dir) S.t[no++] = a;
        // the bases of the fixed direction at the boundary parameter
        const Basis1D& G = P.g[S.dir];
        const Basis1D& B = P.b[S.dir];
        if (G.p > kMaxNeuDeg || B.p > kMaxNeuDeg) throw std::invalid_argument("neumann: degree too high");
        const double fixv = S.upper ? B.t.back() : B.t.front();
        std::vector<double> buf(2 * (kMaxNeuDeg + 1));
        int sp = G.span(fixv);
        G.eval(sp, fixv, buf.data());
        S.gfirst = sp - G.p;
        S.gp = G.p;
        for (int c = 0; c <= G.p; ++c) S.gval[c] = buf[size_t(c)];
        sp = B.span(fixv);
        B.eval(sp, fixv, buf.data());
        S.bfirst = sp - B.p;
        S.bp = B.p;
        for (int c = 0; c <= B.p; ++c) S.bval[c] = buf[size_t(c)];
        S.qbase = np.nvals;
        S.nq = (long long)D.Q[S.t[0]] * (dim == 3 ? D.Q[S.t[1]] : 1);
        np.nvals += S.nq;
        for (long long b = 0; b < S.nq; b += block) np.blocks.push_back({k, 0, b});
        // the functions on the side: the layers of the fixed direction with a non-zero value
        const int n0 = D.n[S.t[0]], n1 = dim == 3 ? D.n[S.t[1]] : 1;
        for (int c = 0; c <= B.p; ++c) {
            if (S.bval[c] == 0.0) continue;
            for (int j1 = 0; j1 < n1; ++j1)
                for (int j0 = 0; j0 < n0; ++j0) {
                    int ii[3] = {0, 0, 0};
                    ii[S.dir] = S.bfirst + c;
                    ii[S.t[0]] = j0;
                    if (dim == 3) ii[S.t[1]] = j1;
                    const long long loc = ii[0] + (long long)D.n[0] * (ii[1] + (long long)D.n[1] * ii[2]);
                    const long long lv = D.lvec_off + loc;
                    auto it = slot.find(lv);
                    if (it == slot.end()) {
                        NeuDof J{};
                        J.patch = pi;
                        for (int a = 0; a < 3; ++a) J.i[a] = ii[a];
                        J.lvec = lv;
                        it = slot.emplace(lv, np.dofs.size()).first;
                        np.dofs.push_back(J);
                    }
                    NeuDof& J = np.dofs[it->second];
                    if (J.nside >= 6) throw std::invalid_argument("neumann: function on more than six sides");
                    J.side[J.nside++] = k;
                }
        }
        np.sides.push_back(S);
    }
    // load-vector order: neighbouring threads write neighbouring slots
    std::sort(np.dofs.begin(), np.dofs.end(), [](const NeuDof& a, const NeuDof& b) { return a.lvec < b.lvec; });
}

void blockTable(const std::vector<long long>& work, int block, std::vector<BlkEnt>& tab) {
    tab.clear();
    for (size_t p = 0; p < work.size(); ++p)
        for (long long b = 0; b < work[p]; b += block) tab.push_back({int(p), 0, b});
}

}  // namespace gsgpu
