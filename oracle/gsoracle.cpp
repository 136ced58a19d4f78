// CPU oracle: a plain FP64 restatement of G+Smo's isogeometric Poisson / diffusion path.
//
// TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
// leg as the checker; never by the GPU product. Each function cites the reference code it
// restates (paths relative to the G+Smo source tree).
#include "gsoracle.h"

#include <algorithm>
#include <map>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------------------------
// Gauss-Legendre reference rule on [-1,1], nodes ascending
// (src/gsAssembler/gsGaussRule.hpp:74-117 tabulates these; the values are the roots of P_n).
void gaussRule(int n, std::vector<double>& x, std::vector<double>& w) {
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    for (int i = 0; i < n; ++i) {
        long double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
        long double dp = 0;
        for (int it = 0; it < 100; ++it) {
            long double p0 = 1, p1 = 0;
            for (int k = 1; k <= n; ++k) {
                long double p2 = p1;
                p1 = p0;
                p0 = ((2 * k - 1) * z * p1 - (k - 1) * p2) / k;
            }
            dp = n * (z * p0 - p1) / (z * z - 1);
            long double dz = p0 / dp;
            z -= dz;
            if (std::fabs((double)dz) < 1e-19) break;
        }
        x[n - 1 - i] = (double)z;
        w[n - 1 - i] = (double)(2.0L / ((1 - z * z) * dp * dp));
    }
    if (n % 2 == 1) x[n / 2] = 0.0;
}

// ---------------------------------------------------------------------------------------------
// 1-D B-spline basis (src/gsNurbs/gsBSplineBasis.hpp, gsKnotVector.hpp)
struct Basis1D {
    int p = 0;
    std::vector<double> t;
    std::vector<double> breaks;  // distinct knot values (element boundaries)
    int n() const { return int(t.size()) - p - 1; }
    int nelem() const { return int(breaks.size()) - 1; }
    void init(int deg, const double* k, int nk) {
        p = deg;
        t.assign(k, k + nk);
        breaks.clear();
        for (double v : t)
            if (breaks.empty() || v > breaks.back()) breaks.push_back(v);
    }
    // knot span containing u: last s with t[s] <= u < t[s+1], clamped to the last non-empty span
    // at the right end (gsKnotVector::uFind/iFind, gsKnotVector.hpp:747-790)
    int span(double u) const {
        const int nn = n();
        if (u >= t[nn]) {
            int s = nn - 1;
            while (s > p && t[s] == t[s + 1]) --s;
            return s;
        }
        int s = int(std::upper_bound(t.begin(), t.end(), u) - t.begin()) - 1;
        return std::max(p, std::min(s, nn - 1));
    }
    // Greville abscissae (gsKnotVector::greville_into, gsKnotVector.hpp:991-1026)
    std::vector<double> greville() const {
        std::vector<double> g(n());
        for (int i = 0; i < n(); ++i) {
            if (p == 0) { g[i] = 0.5 * (t[i] + t[i + 1]); continue; }
            double s = 0;
            for (int j = 1; j <= p; ++j) s += t[i + j];
            g[i] = s / p;
        }
        return g;
    }
    // values and derivatives 0..nd of the p+1 non-zero functions at u in span s
    // (gsTensorBSplineBasis<1>::evalAllDers_into, gsBSplineBasis.hpp:862-1041; the "ndu" triangle
    // of knot differences followed by the derivative recurrences and the factorial scaling).
    // out[k*(p+1)+r] = d^k/du^k N_{s-p+r}(u)
    void ders(int s, double u, int nd, double* out) const {
        const int P = p;
        std::vector<double> left(P + 1), right(P + 1);
        std::vector<double> ndu((P + 1) * (P + 1));
        auto NDU = [&](int a, int b) -> double& { return ndu[a * (P + 1) + b]; };
        NDU(0, 0) = 1.0;
        for (int j = 1; j <= P; ++j) {
            left[j] = u - t[s + 1 - j];
            right[j] = t[s + j] - u;
            double saved = 0.0;
            for (int r = 0; r < j; ++r) {
                NDU(j, r) = right[r + 1] + left[j - r];
                const double tmp = NDU(r, j - 1) / NDU(j, r);
                NDU(r, j) = saved + right[r + 1] * tmp;
                saved = left[j - r] * tmp;
            }
            NDU(j, j) = saved;
        }
        for (int j = 0; j <= P; ++j) out[j] = NDU(j, P);
        std::vector<double> a(2 * (P + 1));
        for (int r = 0; r <= P; ++r) {
            int s1 = 0, s2 = 1;
            a[0] = 1.0;
            for (int k = 1; k <= nd; ++k) {
                double dv = 0.0;
                const int rk = r - k, pk = P - k;
                if (k > P) { out[k * (P + 1) + r] = 0.0; continue; }
                if (r >= k) {
                    a[s2 * (P + 1) + 0] = a[s1 * (P + 1) + 0] / NDU(pk + 1, rk);
                    dv = a[s2 * (P + 1)] * NDU(rk, pk);
                }
                const int j1 = (rk >= -1) ? 1 : -rk;
                const int j2 = (r - 1 <= pk) ? k - 1 : P - r;
                for (int j = j1; j <= j2; ++j) {
                    a[s2 * (P + 1) + j] = (a[s1 * (P + 1) + j] - a[s1 * (P + 1) + j - 1]) / NDU(pk + 1, rk + j);
                    dv += a[s2 * (P + 1) + j] * NDU(rk + j, pk);
                }
                if (r <= pk) {
                    a[s2 * (P + 1) + k] = -a[s1 * (P + 1) + k - 1] / NDU(pk + 1, r);
                    dv += a[s2 * (P + 1) + k] * NDU(r, pk);
                }
                out[k * (P + 1) + r] = dv;
                std::swap(s1, s2);
            }
        }
        double fac = P;
        for (int k = 1; k <= nd; ++k) {
            for (int j = 0; j <= P; ++j) out[k * (P + 1) + j] *= fac;
            fac *= (P - k);
        }
    }
};

// ---------------------------------------------------------------------------------------------
struct PatchData {
    int dim = 2;
    Basis1D b[3], g[3];
    std::vector<double> coefs;  // ngeo x dim
    int nd[3] = {1, 1, 1};      // discretisation dofs per direction
    int ndofs = 0;
    int offset = 0;             // patch offset in the concatenated local numbering
    long long nelem = 0;
    int ne[3] = {1, 1, 1};
};

// boundary(side): local indices with coordinate dir fixed at 0 or n-1, increasing local index
// (gsTensorBasis::boundaryOffset -> coefSlice, src/gsTensor/gsTensorBasis.hpp:303-311)
std::vector<int> boundaryDofs(const PatchData& P, int side) {
    const int dir = (side - 1) / 2, par = (side - 1) % 2;
    const int fix = par ? P.nd[dir] - 1 : 0;
    std::vector<int> out;
    for (int i = 0; i < P.ndofs; ++i) {
        int c[3], r = i;
        for (int k = 0; k < P.dim; ++k) { c[k] = r % P.nd[k]; r /= P.nd[k]; }
        if (c[dir] == fix) out.push_back(i);
    }
    return out;
}

// ---------------------------------------------------------------------------------------------
// gsDofMapper restated with union-find. The reference tags each patch-local dof as free (0),
// eliminated (<0) or coupled (>0) and merges tags with global replaces
// (src/gsCore/gsDofMapper.cpp:99-167 matchDof, :217-238 eliminateDof). Its final numbering
// (finalizeComp, :271-344) depends only on the resulting equivalence classes and their type:
// standard free dofs in scan order, then one index per coupled class in order of first
// appearance, then one index per eliminated class in order of first appearance.
struct DofMapper {
    std::vector<int> parent;
    std::vector<char> elim, coupled;
    std::vector<int> index;  // final global index per local dof
    int freeSize = 0, boundarySize = 0;

    void init(int n) {
        parent.resize(n);
        std::iota(parent.begin(), parent.end(), 0);
        elim.assign(n, 0);
        coupled.assign(n, 0);
    }
    int find(int a) {
        while (parent[a] != a) { parent[a] = parent[parent[a]]; a = parent[a]; }
        return a;
    }
    void unite(int a, int b) {
        a = find(a); b = find(b);
        if (a == b) return;
        if (a > b) std::swap(a, b);
        parent[b] = a;
        elim[a] = elim[a] || elim[b];
        coupled[a] = coupled[a] || coupled[b];
    }
    void eliminate(int a) { elim[find(a)] = 1; }
    void match(int a, int b) {
        const int ra = find(a), rb = find(b);
        if (ra == rb) {
            if (!elim[ra]) coupled[ra] = 1;  // markCoupled on itself
            return;
        }
        unite(ra, rb);
        const int r = find(ra);
        if (!elim[r]) coupled[r] = 1;
    }
    void finalize() {
        const int n = int(parent.size());
        index.assign(n, -1);
        int nstd = 0;
        for (int i = 0; i < n; ++i) {
            const int r = find(i);
            if (!elim[r] && !coupled[r]) ++nstd;
        }
        std::vector<int> cls(n, -1);
        int curFree = 0, curCpl = nstd;
        for (int i = 0; i < n; ++i) {
            const int r = find(i);
            if (elim[r]) continue;
            if (!coupled[r]) index[i] = curFree++;
            else {
                if (cls[r] < 0) cls[r] = curCpl++;
                index[i] = cls[r];
            }
        }
        freeSize = curCpl;
        int curElim = freeSize;
        for (int i = 0; i < n; ++i) {
            const int r = find(i);
            if (!elim[r]) continue;
            if (cls[r] < 0) cls[r] = curElim++;
            index[i] = cls[r];
        }
        boundarySize = curElim - freeSize;
    }
};

// closed-form coefficient, source and exact solution (the functions the tests feed to the
// reference through gsFunction subclasses)
struct Fields {
    int dim, fourier, nmodes, ufreq;
    double kconst, alpha, scale;
    std::vector<double> amp, phase;
    std::vector<int> kk;
    void eval(const double* x, double& kappa, double& f, double& u) const {
        const double w = ufreq * M_PI;
        double sn[3], cs[3];
        for (int i = 0; i < dim; ++i) { sn[i] = std::sin(w * x[i]); cs[i] = std::cos(w * x[i]); }
        u = 1.0;
        for (int i = 0; i < dim; ++i) u *= sn[i];
        double gu[3];
        for (int j = 0; j < dim; ++j) {
            gu[j] = w * cs[j];
            for (int i = 0; i < dim; ++i) if (i != j) gu[j] *= sn[i];
        }
        double g = 0, gg[3] = {0, 0, 0};
        if (fourier) {
            for (int m = 0; m < nmodes; ++m) {
                double th = phase[m];
                for (int i = 0; i < dim; ++i) th += M_PI * kk[3 * m + i] * x[i];
                g += amp[m] * std::cos(th);
                const double sth = std::sin(th);
                for (int i = 0; i < dim; ++i) gg[i] -= amp[m] * sth * M_PI * kk[3 * m + i];
            }
            g *= scale;
            for (int i = 0; i < dim; ++i) gg[i] *= scale;
            kappa = std::exp(alpha * g);
        } else {
            kappa = kconst;
        }
        double dot = 0;
        for (int i = 0; i < dim; ++i) dot += gg[i] * gu[i];
        f = kappa * (dim * w * w * u - alpha * dot);
    }
};

struct Csr {
    int n = 0;
    std::vector<int> ptr, idx;
    std::vector<double> val;
    double& at(int r, int c) {
        const int* b = idx.data() + ptr[r];
        const int* e = idx.data() + ptr[r + 1];
        const int* p = std::lower_bound(b, e, c);
        return val[size_t(p - idx.data())];
    }
    void spmv(const double* x, double* y) const {
        for (int r = 0; r < n; ++r) {
            double s = 0;
            for (int k = ptr[r]; k < ptr[r + 1]; ++k) s += val[k] * x[idx[k]];
            y[r] = s;
        }
    }
};

struct Oracle {
    int dim = 2;
    std::vector<PatchData> patches;
    std::vector<int> ifaces, dsides, nsides;
    Fields F;
    double quA = 1.0;
    int quB = 1;
    DofMapper map;
    int nlocal = 0;
    Csr A;
    std::vector<double> rhs, ddof;
    bool dirL2 = false;  // Dirichlet values by L2 projection instead of interpolation
    bool assembled = false;

    int nq(int p) const { return int(quA * p + quB + 0.5); }

    // geometry map value and Jacobian at parametric point xi (gsGeometry::compute,
    // src/gsCore/gsGeometry.hpp:538-570): x = sum c_i N_i, J(m,n) = sum c_i,m dN_i/dxi_n
    void geoEval(const PatchData& P, const double* xi, double* x, double* J) const {
        const int d = P.dim;
        int s[3], first[3];
        double v[3][16], dv[3][16];
        double buf[64];
        for (int k = 0; k < d; ++k) {
            const Basis1D& B = P.g[k];
            s[k] = B.span(xi[k]);
            first[k] = s[k] - B.p;
            B.ders(s[k], xi[k], 1, buf);
            for (int r = 0; r <= B.p; ++r) { v[k][r] = buf[r]; dv[k][r] = buf[B.p + 1 + r]; }
        }
        int ng[3] = {1, 1, 1};
        for (int k = 0; k < d; ++k) ng[k] = P.g[k].n();
        for (int m = 0; m < d; ++m) { x[m] = 0; for (int n = 0; n < d; ++n) J[m * d + n] = 0; }
        const int p0 = P.g[0].p, p1 = P.g[1].p, p2 = d == 3 ? P.g[2].p : 0;
        for (int c = 0; c <= p2; ++c)
            for (int b = 0; b <= p1; ++b)
                for (int a = 0; a <= p0; ++a) {
                    int gi = first[0] + a + ng[0] * (first[1] + b + (d == 3 ? ng[1] * (first[2] + c) : 0));
                    double val = v[0][a] * v[1][b];
                    double dd[3] = {dv[0][a] * v[1][b], v[0][a] * dv[1][b], 0};
                    if (d == 3) {
                        dd[0] *= v[2][c]; dd[1] *= v[2][c];
                        dd[2] = v[0][a] * v[1][b] * dv[2][c];
                        val *= v[2][c];
                    }
                    for (int m = 0; m < d; ++m) {
                        const double cm = P.coefs[size_t(gi) * d + m];
                        x[m] += cm * val;
                        for (int n = 0; n < d; ++n) J[m * d + n] += cm * dd[n];
                    }
                }
    }

    static double det(int d, const double* J) {
        if (d == 2) return J[0] * J[3] - J[1] * J[2];
        return J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
               J[2] * (J[3] * J[7] - J[4] * J[6]);
    }
    // inverse transpose of J (gsFunction::computeAuxiliaryData, gsFunction.hpp:733-748)
    static void invT(int d, const double* J, double* G) {
        const double D = det(d, J);
        if (d == 2) {
            G[0] = J[3] / D; G[1] = -J[2] / D;
            G[2] = -J[1] / D; G[3] = J[0] / D;
            return;
        }
        // inv(J)(i,j) = cof(J)(j,i)/D ; inv(J)^T(i,j) = cof(J)(i,j)/D
        G[0] = (J[4] * J[8] - J[5] * J[7]) / D;
        G[1] = -(J[3] * J[8] - J[5] * J[6]) / D;
        G[2] = (J[3] * J[7] - J[4] * J[6]) / D;
        G[3] = -(J[1] * J[8] - J[2] * J[7]) / D;
        G[4] = (J[0] * J[8] - J[2] * J[6]) / D;
        G[5] = -(J[0] * J[7] - J[1] * J[6]) / D;
        G[6] = (J[1] * J[5] - J[2] * J[4]) / D;
        G[7] = -(J[0] * J[5] - J[2] * J[3]) / D;
        G[8] = (J[0] * J[4] - J[1] * J[3]) / D;
    }

    void setup(const orc_problem* pr) {
        dim = pr->dim;
        const double* kp = pr->knots;
        const double* gkp = pr->gknots;
        const double* cp = pr->coefs;
        int off = 0;
        for (int i = 0; i < pr->npatches; ++i) {
            PatchData P;
            P.dim = dim;
            int ngeo = 1;
            P.ndofs = 1;
            P.nelem = 1;
            for (int k = 0; k < dim; ++k) {
                P.b[k].init(pr->degree[3 * i + k], kp, pr->nknots[3 * i + k]);
                kp += pr->nknots[3 * i + k];
                P.g[k].init(pr->gdegree[3 * i + k], gkp, pr->gnknots[3 * i + k]);
                gkp += pr->gnknots[3 * i + k];
                P.nd[k] = P.b[k].n();
                P.ndofs *= P.nd[k];
                P.ne[k] = P.b[k].nelem();
                P.nelem *= P.ne[k];
                ngeo *= P.g[k].n();
            }
            P.coefs.assign(cp, cp + size_t(ngeo) * dim);
            cp += size_t(ngeo) * dim;
            P.offset = off;
            off += P.ndofs;
            patches.push_back(std::move(P));
        }
        nlocal = off;
        ifaces.assign(pr->interfaces, pr->interfaces + 4 * pr->ninterfaces);
        dsides.assign(pr->dirichlet, pr->dirichlet + 2 * pr->ndirichlet);
        if (pr->nneumann > 0) nsides.assign(pr->neumann, pr->neumann + 2 * pr->nneumann);
        F.dim = dim;
        F.fourier = pr->kappa_fourier;
        F.kconst = pr->kappa_const;
        F.alpha = pr->kappa_fourier ? pr->kappa_alpha : 0.0;
        F.scale = pr->kappa_scale;
        F.nmodes = pr->kappa_fourier ? pr->kappa_nmodes : 0;
        F.amp.assign(pr->kappa_amp, pr->kappa_amp + F.nmodes);
        F.phase.assign(pr->kappa_phase, pr->kappa_phase + F.nmodes);
        F.kk.assign(pr->kappa_k, pr->kappa_k + 3 * F.nmodes);
        F.ufreq = pr->ufreq;
        quA = pr->quA;
        quB = pr->quB;
        dirL2 = pr->dirichlet_l2 != 0;

        // gsDofMapper(mb, bc, 0): markBoundary for every Dirichlet side
        // (gsDofMapper.hpp:100-111), then matchInterface for every interface
        // (gsMultiBasis.hpp:392-425); interfaces here are conforming with identity orientation,
        // so gsTensorBasis::matchWith pairs the two side slices in order.
        map.init(nlocal);
        for (size_t i = 0; i < dsides.size(); i += 2) {
            const PatchData& P = patches[dsides[i]];
            for (int l : boundaryDofs(P, dsides[i + 1])) map.eliminate(P.offset + l);
        }
        for (size_t i = 0; i < ifaces.size(); i += 4) {
            const PatchData& P1 = patches[ifaces[i]];
            const PatchData& P2 = patches[ifaces[i + 2]];
            std::vector<int> b1 = boundaryDofs(P1, ifaces[i + 1]);
            std::vector<int> b2 = boundaryDofs(P2, ifaces[i + 3]);
            if (b1.size() != b2.size()) throw std::runtime_error("non-conforming interface");
            for (size_t k = 0; k < b1.size(); ++k) map.match(P1.offset + b1[k], P2.offset + b2[k]);
        }
        map.finalize();
    }

    // element iteration helpers
    struct Elem {
        int patch;
        int e[3];
    };
    Elem elemAt(long long gidx) const {
        Elem E{0, {0, 0, 0}};
        for (size_t p = 0; p < patches.size(); ++p) {
            if (gidx < patches[p].nelem) {
                E.patch = int(p);
                long long r = gidx;
                for (int k = 0; k < dim; ++k) { E.e[k] = int(r % patches[p].ne[k]); r /= patches[p].ne[k]; }
                return E;
            }
            gidx -= patches[p].nelem;
        }
        return E;
    }
    long long totalElems() const {
        long long s = 0;
        for (auto& P : patches) s += P.nelem;
        return s;
    }

    // quadrature nodes / weights on an element, tensor order with direction 0 fastest
    // (gsQuadRule::mapTo, src/gsAssembler/gsQuadRule.hpp:23-37 and gsQuadRule.h:132)
    // evaluatorRule: p + 1 points per direction, the default rule of gsExprEvaluator
    // (gsExprEvaluator.h:79-80, quA = 1, quB = 1), which gsField::distanceL2/H1 integrate with
    void elementRule(const PatchData& P, const Elem& E, std::vector<double>& pts, std::vector<double>& wts,
                     int q[3], bool evaluatorRule = false) const {
        std::vector<double> xr[3], wr[3];
        int nqt = 1;
        for (int k = 0; k < dim; ++k) {
            q[k] = evaluatorRule ? P.b[k].p + 1 : nq(P.b[k].p);
            gaussRule(q[k], xr[k], wr[k]);
            const double lo = P.b[k].breaks[E.e[k]], hi = P.b[k].breaks[E.e[k] + 1];
            const double h = (hi - lo) / 2.0;
            for (int r = 0; r < q[k]; ++r) { xr[k][r] = h * (xr[k][r] + 1) + lo; wr[k][r] *= (h == 0 ? 0.5 : h); }
            nqt *= q[k];
        }
        pts.resize(size_t(nqt) * dim);
        wts.resize(nqt);
        for (int i = 0; i < nqt; ++i) {
            int r = i;
            double w = 1.0;
            for (int k = 0; k < dim; ++k) {
                const int c = r % q[k];
                r /= q[k];
                pts[size_t(i) * dim + k] = xr[k][c];
                w *= wr[k][c];
            }
            wts[i] = w;
        }
    }

    // active functions and their values/gradients at the element's quadrature points
    // (gsTensorBasis::active_into / evalAllDers_into, gsTensorBasis.hpp:203-236, 633-728)
    void elementBasis(const PatchData& P, const Elem& E, const std::vector<double>& pts, int nqt,
                      std::vector<int>& act, std::vector<double>& N, std::vector<double>& dN) const {
        const int d = dim;
        int first[3], pp[3] = {0, 0, 0}, na = 1;
        for (int k = 0; k < d; ++k) {
            const Basis1D& B = P.b[k];
            const double mid = 0.5 * (B.breaks[E.e[k]] + B.breaks[E.e[k] + 1]);
            first[k] = B.span(mid) - B.p;
            pp[k] = B.p;
            na *= B.p + 1;
        }
        act.resize(na);
        for (int a = 0; a < na; ++a) {
            int r = a, idx = 0, str = 1;
            for (int k = 0; k < d; ++k) {
                const int c = r % (pp[k] + 1);
                r /= (pp[k] + 1);
                idx += (first[k] + c) * str;
                str *= P.nd[k];
            }
            act[a] = idx;
        }
        N.assign(size_t(na) * nqt, 0.0);
        dN.assign(size_t(na) * nqt * d, 0.0);
        double buf[3][32];
        for (int qi = 0; qi < nqt; ++qi) {
            for (int k = 0; k < d; ++k) {
                const Basis1D& B = P.b[k];
                B.ders(first[k] + B.p, pts[size_t(qi) * d + k], 1, buf[k]);
            }
            for (int a = 0; a < na; ++a) {
                int r = a, c[3];
                for (int k = 0; k < d; ++k) { c[k] = r % (pp[k] + 1); r /= (pp[k] + 1); }
                double v = 1.0;
                for (int k = 0; k < d; ++k) v *= buf[k][c[k]];
                N[size_t(a) * nqt + qi] = v;
                for (int n = 0; n < d; ++n) {
                    double g = 1.0;
                    for (int k = 0; k < d; ++k) g *= (k == n) ? buf[k][pp[k] + 1 + c[k]] : buf[k][c[k]];
                    dN[(size_t(a) * d + n) * nqt + qi] = g;
                }
            }
        }
    }

    // Dirichlet values by L2 projection (gsAssembler::computeDirichletDofsL2Proj,
    // src/gsAssembler/gsAssembler.hpp:392-534): on every element of every Dirichlet side,
    // p_k + 1 Gauss points per side direction (the fixed direction: one node of weight 2 on a
    // zero-length interval, i.e. 1), weight times |det J| of the full map (the map data carries no
    // side), the mass matrix and the moments of u over the eliminated dofs active there; the
    // global system is solved by Jacobi-preconditioned CG (gsSparseSolver::CGDiagonal)
    void dirichletValuesL2() {
        const int nb = map.boundarySize;
        ddof.assign(nb, 0.0);
        std::vector<std::map<int, double>> M(nb);
        std::vector<double> g(nb, 0.0);
        for (size_t si = 0; si < dsides.size(); si += 2) {
            const PatchData& P = patches[dsides[si]];
            const int side = dsides[si + 1];
            const int dir = (side - 1) / 2, par = (side - 1) % 2;
            std::vector<int> odirs;
            for (int k = 0; k < dim; ++k) if (k != dir) odirs.push_back(k);
            const double fixv = par ? P.b[dir].t.back() : P.b[dir].t.front();
            const int no = int(odirs.size());
            std::vector<std::vector<double>> qx(no), qw(no);
            for (int o = 0; o < no; ++o) gaussRule(P.b[odirs[o]].p + 1, qx[o], qw[o]);
            const int ne0 = P.b[odirs[0]].nelem(), ne1 = no > 1 ? P.b[odirs[1]].nelem() : 1;
            for (int e1 = 0; e1 < ne1; ++e1)
                for (int e0 = 0; e0 < ne0; ++e0) {
                    const int el[2] = {e0, e1};
                    const int nq0 = int(qx[0].size()), nq1 = no > 1 ? int(qx[1].size()) : 1;
                    for (int q1 = 0; q1 < nq1; ++q1)
                        for (int q0 = 0; q0 < nq0; ++q0) {
                            const int qq[2] = {q0, q1};
                            double xi[3] = {0, 0, 0};
                            xi[dir] = fixv;
                            double w = 1.0;
                            for (int o = 0; o < no; ++o) {
                                const Basis1D& B = P.b[odirs[o]];
                                const double a = B.breaks[el[o]], b = B.breaks[el[o] + 1];
                                const double h = 0.5 * (b - a);
                                xi[odirs[o]] = a + h * (qx[o][qq[o]] + 1.0);
                                w *= h * qw[o][qq[o]];
                            }
                            double x[3], J[9];
                            geoEval(P, xi, x, J);
                            double det = dim == 2 ? J[0] * J[3] - J[1] * J[2]
                                                  : J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                                                        J[2] * (J[3] * J[7] - J[4] * J[6]);
                            const double wk = w * std::fabs(det);
                            double kap, ff, u;
                            F.eval(x, kap, ff, u);
                            // discretisation basis values at xi; the eliminated dofs among them
                            int sp[3], first[3];
                            double v[3][16], buf[64];
                            for (int k = 0; k < dim; ++k) {
                                const Basis1D& B = P.b[k];
                                sp[k] = B.span(xi[k]);
                                first[k] = sp[k] - B.p;
                                B.ders(sp[k], xi[k], 0, buf);
                                for (int r = 0; r <= B.p; ++r) v[k][r] = buf[r];
                            }
                            std::vector<std::pair<int, double>> act;
                            const int p2 = dim == 3 ? P.b[2].p : 0;
                            for (int c = 0; c <= p2; ++c)
                                for (int b = 0; b <= P.b[1].p; ++b)
                                    for (int a = 0; a <= P.b[0].p; ++a) {
                                        const int loc = first[0] + a +
                                                        P.b[0].n() * (first[1] + b + (dim == 3 ? P.b[1].n() * (first[2] + c) : 0));
                                        const int gi = map.index[P.offset + loc];
                                        if (gi < map.freeSize) continue;
                                        double val = v[0][a] * v[1][b];
                                        if (dim == 3) val *= v[2][c];
                                        act.push_back({gi - map.freeSize, val});
                                    }
                            for (auto& ai : act) {
                                for (auto& aj : act) M[ai.first][aj.first] += wk * ai.second * aj.second;
                                g[ai.first] += wk * ai.second * u;
                            }
                        }
                }
        }
        // Jacobi-preconditioned CG to round-off
        std::vector<double> dinv(nb, 0.0), r = g, z(nb), pv(nb), t(nb);
        for (int i = 0; i < nb; ++i) {
            auto it = M[i].find(i);
            if (it != M[i].end() && it->second != 0.0) dinv[i] = 1.0 / it->second;
        }
        double bb = 0.0;
        for (double a : g) bb += a * a;
        if (bb == 0.0) return;
        for (int i = 0; i < nb; ++i) z[i] = dinv[i] * r[i];
        pv = z;
        double rz = 0.0;
        for (int i = 0; i < nb; ++i) rz += r[i] * z[i];
        for (int it = 0; it < 10 * nb + 100; ++it) {
            double pt = 0.0;
            for (int i = 0; i < nb; ++i) {
                double acc = 0.0;
                for (auto& e : M[i]) acc += e.second * pv[e.first];
                t[i] = acc;
                pt += pv[i] * acc;
            }
            const double al = rz / pt;
            double rr = 0.0;
            for (int i = 0; i < nb; ++i) {
                ddof[i] += al * pv[i];
                r[i] -= al * t[i];
                rr += r[i] * r[i];
            }
            if (rr <= 1e-30 * bb) break;
            double rzn = 0.0;
            for (int i = 0; i < nb; ++i) { z[i] = dinv[i] * r[i]; rzn += r[i] * z[i]; }
            const double be = rzn / rz;
            rz = rzn;
            for (int i = 0; i < nb; ++i) pv[i] = z[i] + be * pv[i];
        }
    }

    // Neumann boundary integrals (gsVisitorNeumann, src/gsAssembler/gsVisitorNeumann.h:60-135, pushed
    // after the volume terms by gsPoissonAssembler.hpp:59 / gsCDRAssembler.hpp:58; the boundary
    // element loop of gsAssembler::apply, gsAssembler.h:668-722): on every element of the side,
    // quA p + quB Gauss points in each side direction and one node of weight 1 in the fixed one
    // (gsQuadrature::get with fixDir, gsQuadrature.h:153-170; gsQuadRule::mapTo, gsQuadRule.h:177-200);
    // weight |n| with n the outer normal of outerNormal (gsAssembler.h:79-130), whose components
    // are the signed minors of J without the fixed direction's column; data
    // h = sgn kappa du/dx_dir; the element's local vector is added to the free rows
    // (gsSparseSystem::pushToRhs)
    void neumannRhs() {
        for (size_t si = 0; si < nsides.size(); si += 2) {
            const PatchData& P = patches[nsides[si]];
            const int side = nsides[si + 1];
            const int dir = (side - 1) / 2, par = (side - 1) % 2;
            const double sgn = par ? 1.0 : -1.0;
            std::vector<int> odirs;
            for (int k = 0; k < dim; ++k) if (k != dir) odirs.push_back(k);
            const double fixv = par ? P.b[dir].t.back() : P.b[dir].t.front();
            const int no = int(odirs.size());
            std::vector<std::vector<double>> qx(no), qw(no);
            for (int o = 0; o < no; ++o) gaussRule(nq(P.b[odirs[o]].p), qx[o], qw[o]);
            const int ne0 = P.b[odirs[0]].nelem(), ne1 = no > 1 ? P.b[odirs[1]].nelem() : 1;
            const int na = (P.b[0].p + 1) * (P.b[1].p + 1) * (dim == 3 ? P.b[2].p + 1 : 1);
            for (int e1 = 0; e1 < ne1; ++e1)
                for (int e0 = 0; e0 < ne0; ++e0) {
                    const int el[2] = {e0, e1};
                    std::vector<double> loc(na, 0.0);
                    std::vector<int> act(na);
                    const int nq0 = int(qx[0].size()), nq1 = no > 1 ? int(qx[1].size()) : 1;
                    for (int q1 = 0; q1 < nq1; ++q1)
                        for (int q0 = 0; q0 < nq0; ++q0) {
                            const int qq[2] = {q0, q1};
                            double xi[3] = {0, 0, 0};
                            xi[dir] = fixv;
                            double w = 1.0;
                            for (int o = 0; o < no; ++o) {
                                const Basis1D& B = P.b[odirs[o]];
                                const double a = B.breaks[el[o]], b = B.breaks[el[o] + 1];
                                const double h = 0.5 * (b - a);
                                xi[odirs[o]] = a + h * (qx[o][qq[o]] + 1.0);
                                w *= h * qw[o][qq[o]];
                            }
                            double x[3], J[9];
                            geoEval(P, xi, x, J);
                            // |n|: minors of J with row i and column dir removed
                            double nn = 0.0;
                            for (int i = 0; i < dim; ++i) {
                                double mnr;
                                if (dim == 2) {
                                    mnr = J[(1 - i) * 2 + (1 - dir)];
                                } else {
                                    int r[2], c[2], nr = 0, nc = 0;
                                    for (int k = 0; k < 3; ++k) {
                                        if (k != i) r[nr++] = k;
                                        if (k != dir) c[nc++] = k;
                                    }
                                    mnr = J[r[0] * 3 + c[0]] * J[r[1] * 3 + c[1]] - J[r[1] * 3 + c[0]] * J[r[0] * 3 + c[1]];
                                }
                                nn += mnr * mnr;
                            }
                            const double wk = w * std::sqrt(nn);
                            double kap, ff, u;
                            F.eval(x, kap, ff, u);
                            const double wf = F.ufreq * M_PI;
                            double du = wf;
                            for (int i = 0; i < dim; ++i) du *= i == dir ? std::cos(wf * x[i]) : std::sin(wf * x[i]);
                            const double hN = sgn * kap * du;
                            int sp[3], first[3];
                            double v[3][16], buf[64];
                            for (int k = 0; k < dim; ++k) {
                                const Basis1D& B = P.b[k];
                                sp[k] = B.span(xi[k]);
                                first[k] = sp[k] - B.p;
                                B.ders(sp[k], xi[k], 0, buf);
                                for (int r = 0; r <= B.p; ++r) v[k][r] = buf[r];
                            }
                            int a = 0;
                            const int p2 = dim == 3 ? P.b[2].p : 0;
                            for (int c = 0; c <= p2; ++c)
                                for (int b = 0; b <= P.b[1].p; ++b)
                                    for (int aa = 0; aa <= P.b[0].p; ++aa, ++a) {
                                        act[a] = first[0] + aa +
                                                 P.b[0].n() * (first[1] + b + (dim == 3 ? P.b[1].n() * (first[2] + c) : 0));
                                        double val = v[0][aa] * v[1][b];
                                        if (dim == 3) val *= v[2][c];
                                        loc[a] += wk * val * hN;
                                    }
                        }
                    for (int a = 0; a < na; ++a) {
                        const int gi = map.index[P.offset + act[a]];
                        if (gi < map.freeSize) rhs[gi] += loc[a];
                    }
                }
        }
    }

    // Dirichlet values by interpolation at the boundary basis anchors
    // (gsAssembler::computeDirichletDofsIntpl, src/gsAssembler/gsAssembler.hpp:314-390, with
    //  gsTensorBasis::interpolateAtAnchors, gsTensorBasis.hpp:906-960)
    void dirichletValues() {
        if (dirL2) {
            dirichletValuesL2();
            return;
        }
        ddof.assign(map.boundarySize, 0.0);
        for (size_t si = 0; si < dsides.size(); si += 2) {
            const PatchData& P = patches[dsides[si]];
            const int side = dsides[si + 1];
            const int dir = (side - 1) / 2, par = (side - 1) % 2;
            std::vector<int> odirs;
            for (int k = 0; k < dim; ++k) if (k != dir) odirs.push_back(k);
            std::vector<std::vector<double>> gv;
            int npts = 1;
            for (int k : odirs) { gv.push_back(P.b[k].greville()); npts *= int(gv.back().size()); }
            const double fixv = par ? P.b[dir].t.back() : P.b[dir].t.front();
            // values g(x(xi)) on the anchor grid (first remaining direction fastest)
            std::vector<double> f(npts);
            for (int i = 0; i < npts; ++i) {
                double xi[3], x[3], J[9];
                int r = i;
                for (size_t o = 0; o < odirs.size(); ++o) {
                    const int c = r % int(gv[o].size());
                    r /= int(gv[o].size());
                    xi[odirs[o]] = gv[o][c];
                }
                xi[dir] = fixv;
                geoEval(P, xi, x, J);
                double kap, ff, u;
                F.eval(x, kap, ff, u);
                f[i] = u;
            }
            // solve the tensor collocation system one direction at a time
            int stride = 1;
            for (size_t o = 0; o < odirs.size(); ++o) {
                const Basis1D& B = P.b[odirs[o]];
                const int n = B.n();
                std::vector<double> M(size_t(n) * n, 0.0);
                std::vector<double> buf(2 * (B.p + 1));
                for (int a = 0; a < n; ++a) {
                    const double u = gv[o][a];
                    const int s = B.span(u);
                    B.ders(s, u, 0, buf.data());
                    for (int r = 0; r <= B.p; ++r) M[size_t(a) * n + (s - B.p + r)] = buf[r];
                }
                // LU with partial pivoting
                std::vector<int> piv(n);
                for (int k = 0; k < n; ++k) {
                    int pmax = k;
                    for (int i = k + 1; i < n; ++i)
                        if (std::fabs(M[size_t(i) * n + k]) > std::fabs(M[size_t(pmax) * n + k])) pmax = i;
                    piv[k] = pmax;
                    if (pmax != k)
                        for (int j = 0; j < n; ++j) std::swap(M[size_t(k) * n + j], M[size_t(pmax) * n + j]);
                    for (int i = k + 1; i < n; ++i) {
                        const double l = M[size_t(i) * n + k] / M[size_t(k) * n + k];
                        M[size_t(i) * n + k] = l;
                        for (int j = k + 1; j < n; ++j) M[size_t(i) * n + j] -= l * M[size_t(k) * n + j];
                    }
                }
                const int outer = npts / (n * stride);
                std::vector<double> col(n);
                for (int ob = 0; ob < outer; ++ob)
                    for (int ib = 0; ib < stride; ++ib) {
                        for (int a = 0; a < n; ++a) col[a] = f[size_t(ob) * n * stride + size_t(a) * stride + ib];
                        for (int k = 0; k < n; ++k) std::swap(col[k], col[piv[k]]);
                        for (int i = 0; i < n; ++i)
                            for (int j = 0; j < i; ++j) col[i] -= M[size_t(i) * n + j] * col[j];
                        for (int i = n - 1; i >= 0; --i) {
                            for (int j = i + 1; j < n; ++j) col[i] -= M[size_t(i) * n + j] * col[j];
                            col[i] /= M[size_t(i) * n + i];
                        }
                        for (int a = 0; a < n; ++a) f[size_t(ob) * n * stride + size_t(a) * stride + ib] = col[a];
                    }
                stride *= n;
            }
            const std::vector<int> bd = boundaryDofs(P, side);
            for (size_t l = 0; l < bd.size(); ++l) {
                const int gi = map.index[P.offset + bd[l]];
                ddof[gi - map.freeSize] = f[l];
            }
        }
    }

    // symbolic pattern: all free x free pairs sharing an element (what gsSparseSystem::push's
    // coeffRef insertions create, gsSparseSystem.h:972-1010)
    void buildPattern() {
        const int n = map.freeSize;
        std::vector<std::vector<int>> rows(n);
        for (const PatchData& P : patches) {
            // neighbours of local dof i within the band |i_k - j_k| <= p_k restricted to pairs that
            // share an element
            for (int i = 0; i < P.ndofs; ++i) {
                const int gi = map.index[P.offset + i];
                if (gi >= map.freeSize) continue;
                int c[3] = {0, 0, 0}, r = i;
                for (int k = 0; k < dim; ++k) { c[k] = r % P.nd[k]; r /= P.nd[k]; }
                int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
                for (int k = 0; k < dim; ++k) {
                    // elements supporting function c: spans c..c+p in knot-index terms; the
                    // functions sharing an element with c are those whose support overlaps.
                    lo[k] = std::max(0, c[k] - P.b[k].p);
                    hi[k] = std::min(P.nd[k] - 1, c[k] + P.b[k].p);
                }
                for (int z = lo[2]; z <= hi[2]; ++z)
                    for (int y = lo[1]; y <= hi[1]; ++y)
                        for (int x = lo[0]; x <= hi[0]; ++x) {
                            int cc[3] = {x, y, z};
                            bool share = true;
                            for (int k = 0; k < dim; ++k) share = share && supportsOverlap(P.b[k], c[k], cc[k]);
                            if (!share) continue;
                            const int j = x + P.nd[0] * (y + (dim == 3 ? P.nd[1] * z : 0));
                            const int gj = map.index[P.offset + j];
                            if (gj < map.freeSize) rows[gi].push_back(gj);
                        }
            }
        }
        A.n = n;
        A.ptr.assign(n + 1, 0);
        for (int r = 0; r < n; ++r) {
            std::sort(rows[r].begin(), rows[r].end());
            rows[r].erase(std::unique(rows[r].begin(), rows[r].end()), rows[r].end());
            A.ptr[r + 1] = A.ptr[r] + int(rows[r].size());
        }
        A.idx.resize(A.ptr[n]);
        for (int r = 0; r < n; ++r) std::copy(rows[r].begin(), rows[r].end(), A.idx.begin() + A.ptr[r]);
        A.val.assign(A.idx.size(), 0.0);
    }
    // two B-splines share a non-empty element iff their supports intersect in a non-empty span
    static bool supportsOverlap(const Basis1D& B, int a, int b) {
        const double lo = std::max(B.t[a], B.t[b]);
        const double hi = std::min(B.t[a + B.p + 1], B.t[b + B.p + 1]);
        return hi > lo;
    }

    // the element loop (gsAssembler::apply with gsVisitorPoisson / gsVisitorCDR,
    // gsAssembler.h:666-722, gsVisitorPoisson.h:62-118, gsVisitorCDR.h:107-200) and the scatter
    // with Dirichlet elimination (gsSparseSystem::push, gsSparseSystem.h:972-1010)
    double assemble(int nthreads, long long maxElems) {
        auto t0 = std::chrono::steady_clock::now();
        dirichletValues();
        if (A.ptr.empty()) buildPattern();  // symbolic set-up once per problem
        std::fill(A.val.begin(), A.val.end(), 0.0);
        rhs.assign(map.freeSize, 0.0);
        long long ne = totalElems();
        if (maxElems >= 0) ne = std::min(ne, maxElems);
#ifdef _OPENMP
        if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
        {
            int tid = 0, nt = 1;
#ifdef _OPENMP
            tid = omp_get_thread_num();
            nt = omp_get_num_threads();
#endif
            std::vector<double> pts, wts, N, dN, K, fe, phys;
            std::vector<int> act;
            for (long long ge = tid; ge < ne; ge += nt) {  // round-robin like domIt->next(nt)
                const Elem E = elemAt(ge);
                const PatchData& P = patches[E.patch];
                int q[3];
                elementRule(P, E, pts, wts, q);
                const int nqt = int(wts.size());
                elementBasis(P, E, pts, nqt, act, N, dN);
                const int na = int(act.size());
                K.assign(size_t(na) * na, 0.0);
                fe.assign(na, 0.0);
                phys.resize(size_t(na) * dim);
                for (int qi = 0; qi < nqt; ++qi) {
                    double x[3], J[9], G[9];
                    geoEval(P, &pts[size_t(qi) * dim], x, J);
                    const double meas = std::fabs(det(dim, J));
                    invT(dim, J, G);
                    double kap, ff, u;
                    F.eval(x, kap, ff, u);
                    const double w = wts[qi] * meas;
                    for (int a = 0; a < na; ++a)
                        for (int m = 0; m < dim; ++m) {
                            double s = 0;
                            for (int n = 0; n < dim; ++n) s += G[m * dim + n] * dN[(size_t(a) * dim + n) * nqt + qi];
                            phys[size_t(a) * dim + m] = s;
                        }
                    for (int a = 0; a < na; ++a) {
                        fe[a] += w * N[size_t(a) * nqt + qi] * ff;
                        for (int b = 0; b < na; ++b) {
                            double s = 0;
                            for (int m = 0; m < dim; ++m) s += phys[size_t(a) * dim + m] * phys[size_t(b) * dim + m];
                            K[size_t(a) * na + b] += w * kap * s;
                        }
                    }
                }
#pragma omp critical(localToGlobal)
                {
                    for (int a = 0; a < na; ++a) {
                        const int ii = map.index[P.offset + act[a]];
                        if (ii >= map.freeSize) continue;
                        rhs[ii] += fe[a];
                        for (int b = 0; b < na; ++b) {
                            const int jj = map.index[P.offset + act[b]];
                            if (jj < map.freeSize) A.at(ii, jj) += K[size_t(a) * na + b];
                            else rhs[ii] -= K[size_t(a) * na + b] * ddof[jj - map.freeSize];
                        }
                    }
                }
            }
        }
        if (maxElems < 0) neumannRhs();
        assembled = true;
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }

    // gsGenericAssembler::assembleMass (src/gsAssembler/gsGenericAssembler.h:103, its mass visitor
    // integrating phi_i phi_j |det J| with the assembler's Gauss rule) on the free dofs, in the CSR
    // pattern of the stiffness matrix; element loop in element order (serial)
    void mass(double* val) {
        if (A.ptr.empty()) buildPattern();
        Csr M = A;
        std::fill(M.val.begin(), M.val.end(), 0.0);
        std::vector<double> pts, wts, N, dN;
        std::vector<int> act;
        const long long ne = totalElems();
        for (long long ge = 0; ge < ne; ++ge) {
            const Elem E = elemAt(ge);
            const PatchData& P = patches[E.patch];
            int q[3];
            elementRule(P, E, pts, wts, q);
            const int nqt = int(wts.size());
            elementBasis(P, E, pts, nqt, act, N, dN);
            const int na = int(act.size());
            for (int qi = 0; qi < nqt; ++qi) {
                double x[3], J[9];
                geoEval(P, &pts[size_t(qi) * dim], x, J);
                const double w = wts[qi] * std::fabs(det(dim, J));
                for (int a = 0; a < na; ++a) {
                    const int ii = map.index[P.offset + act[a]];
                    if (ii >= map.freeSize) continue;
                    for (int b = 0; b < na; ++b) {
                        const int jj = map.index[P.offset + act[b]];
                        if (jj < map.freeSize)
                            M.at(ii, jj) += w * N[size_t(a) * nqt + qi] * N[size_t(b) * nqt + qi];
                    }
                }
            }
        }
        std::copy(M.val.begin(), M.val.end(), val);
    }

    // gsConjugateGradient with gsJacobiOp (gsConjugateGradient.hpp:19-84,
    // gsIterativeSolver.h:114-202, gsSimplePreconditioners.h:145-244)
    template <class Precond>
    void pcg(const Csr& M, Precond&& prec, const double* b, double* x, double tol, int maxit, int& iters,
             double& relres) const {
        const int n = M.n;
        std::vector<double> r(n), z(n), p(n), t(n);
        double bn = 0;
        for (int i = 0; i < n; ++i) bn += b[i] * b[i];
        bn = std::sqrt(bn);
        iters = 0;
        if (bn == 0) { std::fill(x, x + n, 0.0); relres = 0; return; }
        std::fill(x, x + n, 0.0);
        M.spmv(x, t.data());
        for (int i = 0; i < n; ++i) r[i] = b[i] - t[i];
        auto nrm = [&](const std::vector<double>& v) { double s = 0; for (double e : v) s += e * e; return std::sqrt(s); };
        relres = nrm(r) / bn;
        if (relres < tol) return;
        prec(r.data(), p.data());
        double absNew = 0;
        for (int i = 0; i < n; ++i) absNew += r[i] * p[i];
        while (iters < maxit) {
            ++iters;
            M.spmv(p.data(), t.data());
            double pt = 0;
            for (int i = 0; i < n; ++i) pt += p[i] * t[i];
            const double alpha = absNew / pt;
            for (int i = 0; i < n; ++i) { x[i] += alpha * p[i]; r[i] -= alpha * t[i]; }
            relres = nrm(r) / bn;
            if (relres < tol) break;
            prec(r.data(), t.data());
            const double absOld = absNew;
            absNew = 0;
            for (int i = 0; i < n; ++i) absNew += r[i] * t[i];
            const double beta = absNew / absOld;
            for (int i = 0; i < n; ++i) p[i] = t[i] + beta * p[i];
        }
    }

    double solveCG(double tol, int maxit, double* x, int& iters, double& relres) const {
        auto t0 = std::chrono::steady_clock::now();
        const int n = A.n;
        std::vector<double> dinv(n);
        for (int r = 0; r < n; ++r)
            for (int k = A.ptr[r]; k < A.ptr[r + 1]; ++k)
                if (A.idx[k] == r) dinv[r] = 1.0 / A.val[k];
        pcg(A, [&](const double* in, double* out) { for (int i = 0; i < n; ++i) out[i] = in[i] * dinv[i]; },
            rhs.data(), x, tol, maxit, iters, relres);
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }

    // L2 error of the discrete solution against the exact one (gsField::distanceL2,
    // src/gsCore/gsField.hpp:23-41, gsAssembler::constructSolution gsAssembler.hpp:536-581)
    // gsField::distanceH1 (src/gsCore/gsField.hpp:44-60) for the parametric solution field against
    // the physical exact function: sqrt(sum w |det J| |J^-T grad_xi u_h - grad u|^2)
    double h1error(const double* x, bool evaluatorRule = false) const {
        double acc = 0;
        const long long ne = totalElems();
#pragma omp parallel for reduction(+ : acc) schedule(static)
        for (long long ge = 0; ge < ne; ++ge) {
            std::vector<double> pts, wts, N, dN;
            std::vector<int> act;
            const Elem E = elemAt(ge);
            const PatchData& P = patches[E.patch];
            int q[3];
            elementRule(P, E, pts, wts, q, evaluatorRule);
            const int nqt = int(wts.size());
            elementBasis(P, E, pts, nqt, act, N, dN);
            for (int qi = 0; qi < nqt; ++qi) {
                double xx[3], J[9], G[9];
                geoEval(P, &pts[size_t(qi) * dim], xx, J);
                invT(dim, J, G);
                double gxi[3] = {0, 0, 0};
                for (size_t a = 0; a < act.size(); ++a) {
                    const int gi = map.index[P.offset + act[a]];
                    const double c = gi < map.freeSize ? x[gi] : ddof[gi - map.freeSize];
                    for (int n = 0; n < dim; ++n) gxi[n] += c * dN[(a * dim + n) * nqt + qi];
                }
                const double w = F.ufreq * M_PI;
                double e2 = 0;
                for (int m = 0; m < dim; ++m) {
                    double gh = 0;
                    for (int n = 0; n < dim; ++n) gh += G[m * dim + n] * gxi[n];
                    double gu = w;
                    for (int i = 0; i < dim; ++i) gu *= i == m ? std::cos(w * xx[i]) : std::sin(w * xx[i]);
                    e2 += (gh - gu) * (gh - gu);
                }
                acc += e2 * wts[qi] * std::fabs(det(dim, J));
            }
        }
        return std::sqrt(acc);
    }

    double l2error(const double* x, bool evaluatorRule = false) const {
        double acc = 0;
        const long long ne = totalElems();
#pragma omp parallel for reduction(+ : acc) schedule(static)
        for (long long ge = 0; ge < ne; ++ge) {
            std::vector<double> pts, wts, N, dN;
            std::vector<int> act;
            const Elem E = elemAt(ge);
            const PatchData& P = patches[E.patch];
            int q[3];
            elementRule(P, E, pts, wts, q, evaluatorRule);
            const int nqt = int(wts.size());
            elementBasis(P, E, pts, nqt, act, N, dN);
            for (int qi = 0; qi < nqt; ++qi) {
                double xx[3], J[9];
                geoEval(P, &pts[size_t(qi) * dim], xx, J);
                double uh = 0;
                for (size_t a = 0; a < act.size(); ++a) {
                    const int gi = map.index[P.offset + act[a]];
                    const double c = gi < map.freeSize ? x[gi] : ddof[gi - map.freeSize];
                    uh += c * N[a * nqt + qi];
                }
                double kap, ff, u;
                F.eval(xx, kap, ff, u);
                acc += (uh - u) * (uh - u) * wts[qi] * std::fabs(det(dim, J));
            }
        }
        return std::sqrt(acc);
    }

    double solveMG(double tol, int maxit, int levels, int npre, int npost, double damping, int cycles, double cgc,
                   double* x, int& iters, double& relres);
};

}  // namespace

// ---------------------------------------------------------------------------------------------
// Geometric h-multigrid (gsGridHierarchy::buildByCoarsening, gsMultiGrid.hpp) restated for
// tensor B-spline patches: coarse spaces remove every other interior knot, transfers are the
// knot-insertion matrices restricted to free dofs of each level's dof mapper, coarse operators
// are Galerkin products P^T A P, the smoother is damped Jacobi, the coarsest level is solved
// directly.
namespace {

struct SparseRows {  // row-major sparse matrix (fine x coarse transfer)
    int rows = 0, cols = 0;
    std::vector<int> ptr, idx;
    std::vector<double> val;
};

// knot-insertion matrix from the coarse 1-D basis Bc to the fine basis Bf (same degree, knots of
// Bc a subset of Bf): fine function values of coarse functions, T(f, c). Computed from
// the Oslo algorithm / Boehm insertion one knot at a time (gsBoehm.hpp).
std::vector<double> transfer1D(const Basis1D& Bc, const Basis1D& Bf) {
    const int p = Bc.p;
    std::vector<double> t = Bc.t;
    int n = Bc.n();
    std::vector<double> T(size_t(n) * n, 0.0);  // current (n x nc)
    const int nc = n;
    for (int i = 0; i < n; ++i) T[size_t(i) * nc + i] = 1.0;
    // insert missing knots
    std::vector<double> add;
    {
        size_t i = 0, j = 0;
        while (j < Bf.t.size()) {
            if (i < t.size() && t[i] == Bf.t[j]) { ++i; ++j; }
            else { add.push_back(Bf.t[j]); ++j; }
        }
    }
    for (double u : add) {
        int s = int(std::upper_bound(t.begin(), t.end(), u) - t.begin()) - 1;
        std::vector<double> Tn(size_t(n + 1) * nc, 0.0);
        for (int i = 0; i <= n; ++i) {
            double a;
            if (i <= s - p) a = 1.0;
            else if (i > s) a = 0.0;
            else a = (u - t[i]) / (t[i + p] - t[i]);
            for (int c = 0; c < nc; ++c) {
                double v = 0;
                if (i < n) v += a * T[size_t(i) * nc + c];
                if (i >= 1) v += (1.0 - a) * T[size_t(i - 1) * nc + c];
                Tn[size_t(i) * nc + c] = v;
            }
        }
        t.insert(t.begin() + s + 1, u);
        ++n;
        T.swap(Tn);
    }
    return T;  // (nf x nc)
}

Basis1D coarsen(const Basis1D& B) {
    // uniformCoarsen: remove every second interior break (gsKnotVector::coarsen)
    std::vector<double> brk = B.breaks;
    std::vector<double> keep;
    for (size_t i = 0; i < brk.size(); ++i)
        if (i == 0 || i + 1 == brk.size() || i % 2 == 0) keep.push_back(brk[i]);
    std::vector<double> t;
    for (int i = 0; i <= B.p; ++i) t.push_back(keep.front());
    for (size_t i = 1; i + 1 < keep.size(); ++i) t.push_back(keep[i]);
    for (int i = 0; i <= B.p; ++i) t.push_back(keep.back());
    Basis1D C;
    C.init(B.p, t.data(), int(t.size()));
    return C;
}

struct Level {
    Oracle* geom = nullptr;      // structure holder (patches + mapper) for this level
    Csr A;
    std::vector<double> dinv;
    SparseRows P;                // this level (fine) <- next coarser
};

}  // namespace

double Oracle::solveMG(double tol, int maxit, int levels, int npre, int npost, double damping, int cycles,
                       double cgc, double* x, int& iters, double& relres) {
    auto t0 = std::chrono::steady_clock::now();
    // build the level structures (finest = this)
    std::vector<Oracle*> lv;
    lv.push_back(this);
    std::vector<std::unique_ptr<Oracle>> owned;
    for (int l = 1; l < levels; ++l) {
        std::unique_ptr<Oracle> c(new Oracle(*lv.back()));
        for (PatchData& P : c->patches) {
            P.ndofs = 1;
            for (int k = 0; k < dim; ++k) {
                P.b[k] = coarsen(P.b[k]);
                P.nd[k] = P.b[k].n();
                P.ndofs *= P.nd[k];
            }
        }
        int off = 0;
        for (PatchData& P : c->patches) { P.offset = off; off += P.ndofs; }
        c->nlocal = off;
        c->map = DofMapper();
        c->map.init(off);
        for (size_t i = 0; i < dsides.size(); i += 2) {
            const PatchData& P = c->patches[dsides[i]];
            for (int b : boundaryDofs(P, dsides[i + 1])) c->map.eliminate(P.offset + b);
        }
        for (size_t i = 0; i < ifaces.size(); i += 4) {
            const PatchData& P1 = c->patches[ifaces[i]];
            const PatchData& P2 = c->patches[ifaces[i + 2]];
            std::vector<int> b1 = boundaryDofs(P1, ifaces[i + 1]), b2 = boundaryDofs(P2, ifaces[i + 3]);
            for (size_t k = 0; k < b1.size(); ++k) c->map.match(P1.offset + b1[k], P2.offset + b2[k]);
        }
        c->map.finalize();
        lv.push_back(c.get());
        owned.push_back(std::move(c));
    }
    const int L = int(lv.size());
    // transfers P_l: free dofs of level l (finer) <- free dofs of level l+1 (coarser).
    // Combined over patches through the dof mappers; a fine free dof takes its row from any one
    // patch pre-image (all pre-images of a coupled dof give the same row for conforming meshes).
    std::vector<SparseRows> Ps(L - 1);
    for (int l = 0; l + 1 < L; ++l) {
        Oracle& Fm = *lv[l];
        Oracle& Cm = *lv[l + 1];
        SparseRows& R = Ps[l];
        R.rows = Fm.map.freeSize;
        R.cols = Cm.map.freeSize;
        std::vector<std::vector<std::pair<int, double>>> rows(R.rows);
        std::vector<char> done(R.rows, 0);
        for (size_t pi = 0; pi < Fm.patches.size(); ++pi) {
            const PatchData& PF = Fm.patches[pi];
            const PatchData& PC = Cm.patches[pi];
            std::vector<double> T[3];
            for (int k = 0; k < dim; ++k) T[k] = transfer1D(PC.b[k], PF.b[k]);
            for (int i = 0; i < PF.ndofs; ++i) {
                const int gi = Fm.map.index[PF.offset + i];
                if (gi >= Fm.map.freeSize || done[gi]) continue;
                done[gi] = 1;
                int c[3] = {0, 0, 0}, r = i;
                for (int k = 0; k < dim; ++k) { c[k] = r % PF.nd[k]; r /= PF.nd[k]; }
                for (int j = 0; j < PC.ndofs; ++j) {
                    int cc[3] = {0, 0, 0}, rr = j;
                    for (int k = 0; k < dim; ++k) { cc[k] = rr % PC.nd[k]; rr /= PC.nd[k]; }
                    double v = 1.0;
                    for (int k = 0; k < dim && v != 0.0; ++k) v *= T[k][size_t(c[k]) * PC.nd[k] + cc[k]];
                    if (v == 0.0) continue;
                    const int gj = Cm.map.index[PC.offset + j];
                    if (gj >= Cm.map.freeSize) continue;
                    rows[gi].push_back({gj, v});
                }
            }
        }
        R.ptr.assign(R.rows + 1, 0);
        for (int i = 0; i < R.rows; ++i) {
            auto& rw = rows[i];
            std::sort(rw.begin(), rw.end());
            std::vector<std::pair<int, double>> m;
            for (auto& e : rw) {
                if (!m.empty() && m.back().first == e.first) continue;  // coupled duplicates
                m.push_back(e);
            }
            rw.swap(m);
            R.ptr[i + 1] = R.ptr[i] + int(rw.size());
        }
        for (int i = 0; i < R.rows; ++i)
            for (auto& e : rows[i]) { R.idx.push_back(e.first); R.val.push_back(e.second); }
    }
    // Galerkin coarse operators A_{l+1} = P^T A_l P (gsMultiGridOp::init, gsMultiGrid.hpp:69-95)
    std::vector<Csr> As(L);
    As[0] = A;
    for (int l = 0; l + 1 < L; ++l) {
        const Csr& Af = As[l];
        const SparseRows& R = Ps[l];
        const int nc = R.cols;
        std::vector<std::vector<std::pair<int, double>>> acc(nc);
        // C = P^T (A P): row of A P for fine row i, then scatter into coarse rows P(i,:)
        std::vector<double> work(nc, 0.0);
        std::vector<char> mark(nc, 0);
        std::vector<int> list;
        std::vector<std::vector<double>> dense;  // not used
        std::vector<std::vector<int>> cidx(nc);
        std::vector<std::vector<double>> cval(nc);
        for (int i = 0; i < Af.n; ++i) {
            list.clear();
            for (int k = Af.ptr[i]; k < Af.ptr[i + 1]; ++k) {
                const int j = Af.idx[k];
                const double a = Af.val[k];
                for (int m = R.ptr[j]; m < R.ptr[j + 1]; ++m) {
                    const int c = R.idx[m];
                    if (!mark[c]) { mark[c] = 1; list.push_back(c); work[c] = 0; }
                    work[c] += a * R.val[m];
                }
            }
            for (int m = R.ptr[i]; m < R.ptr[i + 1]; ++m) {
                const int rc = R.idx[m];
                const double pv = R.val[m];
                for (int c : list) { cidx[rc].push_back(c); cval[rc].push_back(pv * work[c]); }
            }
            for (int c : list) mark[c] = 0;
        }
        Csr& Ac = As[l + 1];
        Ac.n = nc;
        Ac.ptr.assign(nc + 1, 0);
        for (int r = 0; r < nc; ++r) {
            std::vector<std::pair<int, double>> e(cidx[r].size());
            for (size_t k = 0; k < e.size(); ++k) e[k] = {cidx[r][k], cval[r][k]};
            std::sort(e.begin(), e.end(), [](auto& a, auto& b) { return a.first < b.first; });
            std::vector<int> ii;
            std::vector<double> vv;
            for (auto& q : e) {
                if (!ii.empty() && ii.back() == q.first) vv.back() += q.second;
                else { ii.push_back(q.first); vv.push_back(q.second); }
            }
            Ac.ptr[r + 1] = Ac.ptr[r] + int(ii.size());
            Ac.idx.insert(Ac.idx.end(), ii.begin(), ii.end());
            Ac.val.insert(Ac.val.end(), vv.begin(), vv.end());
        }
    }
    // coarse solver: dense Cholesky of A_{L-1}
    const Csr& Ac = As[L - 1];
    const int nc = Ac.n;
    std::vector<double> Lc(size_t(nc) * nc, 0.0);
    for (int r = 0; r < nc; ++r)
        for (int k = Ac.ptr[r]; k < Ac.ptr[r + 1]; ++k) Lc[size_t(r) * nc + Ac.idx[k]] = Ac.val[k];
    for (int j = 0; j < nc; ++j) {
        double s = Lc[size_t(j) * nc + j];
        for (int k = 0; k < j; ++k) s -= Lc[size_t(j) * nc + k] * Lc[size_t(j) * nc + k];
        const double dj = std::sqrt(s);
        Lc[size_t(j) * nc + j] = dj;
        for (int i = j + 1; i < nc; ++i) {
            double t = Lc[size_t(i) * nc + j];
            for (int k = 0; k < j; ++k) t -= Lc[size_t(i) * nc + k] * Lc[size_t(j) * nc + k];
            Lc[size_t(i) * nc + j] = t / dj;
        }
    }
    std::vector<std::vector<double>> Dinv(L);
    for (int l = 0; l < L; ++l) {
        Dinv[l].assign(As[l].n, 0.0);
        for (int r = 0; r < As[l].n; ++r)
            for (int k = As[l].ptr[r]; k < As[l].ptr[r + 1]; ++k)
                if (As[l].idx[k] == r) Dinv[l][r] = 1.0 / As[l].val[k];
    }
    // one cycle (gsMultiGridOp::multiGridStep, gsMultiGrid.hpp:147-201) from the x passed in: the
    // coarse correction starts at zero and is cycled `cycles` times on every level but the
    // coarsest (NumCycles, 1 = V-cycle, 2 = W-cycle; gsMultiGrid.h:328-333), then enters x scaled
    // by the coarse-grid correction damping
    std::function<void(int, const double*, double*)> vcycle = [&](int l, const double* b, double* xl) {
        const Csr& M = As[l];
        const int n = M.n;
        if (l == L - 1) {
            std::vector<double> y(b, b + n);
            for (int i = 0; i < n; ++i) {
                for (int k = 0; k < i; ++k) y[i] -= Lc[size_t(i) * n + k] * y[k];
                y[i] /= Lc[size_t(i) * n + i];
            }
            for (int i = n - 1; i >= 0; --i) {
                for (int k = i + 1; k < n; ++k) y[i] -= Lc[size_t(k) * n + i] * y[k];
                y[i] /= Lc[size_t(i) * n + i];
            }
            std::copy(y.begin(), y.end(), xl);
            return;
        }
        std::vector<double> t(n), r(n);
        auto smooth = [&]() {
            M.spmv(xl, t.data());
            for (int i = 0; i < n; ++i) xl[i] += damping * Dinv[l][i] * (b[i] - t[i]);
        };
        for (int s = 0; s < npre; ++s) smooth();
        M.spmv(xl, t.data());
        for (int i = 0; i < n; ++i) r[i] = t[i] - b[i];
        const SparseRows& R = Ps[l];
        std::vector<double> rc(R.cols, 0.0), ec(R.cols, 0.0);
        for (int i = 0; i < R.rows; ++i)
            for (int m = R.ptr[i]; m < R.ptr[i + 1]; ++m) rc[R.idx[m]] += R.val[m] * r[i];
        const int nc = l + 2 == L ? 1 : cycles;
        for (int c = 0; c < nc; ++c) vcycle(l + 1, rc.data(), ec.data());
        for (int i = 0; i < R.rows; ++i) {
            double s = 0;
            for (int m = R.ptr[i]; m < R.ptr[i + 1]; ++m) s += R.val[m] * ec[R.idx[m]];
            xl[i] -= cgc * s;
        }
        for (int s = 0; s < npost; ++s) smooth();
    };
    const int n = A.n;
    pcg(A,
        [&](const double* in, double* out) {
            std::fill(out, out + n, 0.0);
            vcycle(0, in, out);
        },
        rhs.data(), x, tol, maxit, iters, relres);
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// ---------------------------------------------------------------------------------------------
extern "C" {

void* orc_create(const orc_problem* prob) {
    Oracle* o = new Oracle();
    try {
        o->setup(prob);
    } catch (...) {
        delete o;
        return nullptr;
    }
    return o;
}
void orc_destroy(void* h) { delete static_cast<Oracle*>(h); }
double orc_assemble(void* h, int nthreads, long long max_elements) {
    return static_cast<Oracle*>(h)->assemble(nthreads, max_elements);
}
void orc_sizes(void* h, int* nfree, long long* nnz, int* nbound, int* nlocal) {
    Oracle* o = static_cast<Oracle*>(h);
    *nfree = o->map.freeSize;
    *nnz = (long long)o->A.idx.size();
    *nbound = o->map.boundarySize;
    *nlocal = o->nlocal;
}
void orc_dofmap(void* h, int* out) {
    Oracle* o = static_cast<Oracle*>(h);
    std::copy(o->map.index.begin(), o->map.index.end(), out);
}
void orc_csr(void* h, int* ptr, int* idx, double* val) {
    Oracle* o = static_cast<Oracle*>(h);
    std::copy(o->A.ptr.begin(), o->A.ptr.end(), ptr);
    std::copy(o->A.idx.begin(), o->A.idx.end(), idx);
    std::copy(o->A.val.begin(), o->A.val.end(), val);
}
void orc_rhs(void* h, double* out) {
    Oracle* o = static_cast<Oracle*>(h);
    std::copy(o->rhs.begin(), o->rhs.end(), out);
}
void orc_ddof(void* h, double* out) {
    Oracle* o = static_cast<Oracle*>(h);
    std::copy(o->ddof.begin(), o->ddof.end(), out);
}
double orc_solve_cg(void* h, double tol, int maxit, double* x, int* iters, double* relres) {
    return static_cast<Oracle*>(h)->solveCG(tol, maxit, x, *iters, *relres);
}
double orc_solve_mg(void* h, double tol, int maxit, int levels, int npre, int npost, double damping, int cycles,
                    double cgc, double* x, int* iters, double* relres) {
    return static_cast<Oracle*>(h)->solveMG(tol, maxit, levels, npre, npost, damping, cycles, cgc, x, *iters,
                                            *relres);
}
void orc_mass(void* h, double* val) { static_cast<Oracle*>(h)->mass(val); }
double orc_l2_error(void* h, const double* x) { return static_cast<Oracle*>(h)->l2error(x); }
double orc_h1_error(void* h, const double* x) { return static_cast<Oracle*>(h)->h1error(x); }
double orc_error_evaluator_rule(void* h, const double* x, int h1) {
    const Oracle* o = static_cast<Oracle*>(h);
    return h1 ? o->h1error(x, true) : o->l2error(x, true);
}
void orc_gauss(int n, double* nodes, double* weights) {
    std::vector<double> x, w;
    gaussRule(n, x, w);
    std::copy(x.begin(), x.end(), nodes);
    std::copy(w.begin(), w.end(), weights);
}

}  // extern "C"
