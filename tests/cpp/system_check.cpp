// The C++ layer of the drop-ins (include/gsgpu.hpp, gsgpu::System) driven on the GPU without
// G+Smo: the 2D unit square as an identity tensor B-spline map of degree p with n x n elements,
// Dirichlet u on all sides, kappa = 1, u = sin(pi x) sin(pi y), assembled and solved by CG +
// Jacobi to 1e-10, the matrix read straight into compressed-storage arrays (csrInto). Writes the
// CSR arrays, the rhs and the solution as raw binary files into the output directory and prints
// "free nnz iterations relres l2 h1" for the test to compare with the reference's fixture.
//   system_check <n> <p> <outdir>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "gsgpu.hpp"

template <class V>
static void dump(const std::string& path, const V& v) {
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f) throw std::runtime_error("cannot write " + path);
    std::fwrite(v.data(), sizeof(v[0]), v.size(), f);
    std::fclose(f);
}

int main(int argc, char** argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: system_check <n> <p> <outdir>\n");
        return 2;
    }
    const int ne = std::atoi(argv[1]), p = std::atoi(argv[2]);
    const std::string out = argv[3];
    // open uniform knots, the identity map's control points at the Greville abscissae
    std::vector<double> kv;
    for (int i = 0; i < p; ++i) kv.push_back(0.0);
    for (int i = 0; i <= ne; ++i) kv.push_back(double(i) / ne);
    for (int i = 0; i < p; ++i) kv.push_back(1.0);
    const int n = int(kv.size()) - p - 1;
    std::vector<double> gr(n);
    for (int i = 0; i < n; ++i) {
        double s = 0.0;
        for (int k = 1; k <= p; ++k) s += kv[size_t(i + k)];
        gr[size_t(i)] = s / p;
    }
    std::vector<double> knots(kv), coefs;
    knots.insert(knots.end(), kv.begin(), kv.end());
    for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i) {
            coefs.push_back(gr[size_t(i)]);
            coefs.push_back(gr[size_t(j)]);
        }
    std::vector<int> degree = {p, p, 0}, nknots = {int(kv.size()), int(kv.size()), 0};
    std::vector<int> dirichlet = {0, 1, 0, 2, 0, 3, 0, 4};
    gsgpu_problem pr{};
    pr.dim = 2;
    pr.npatches = 1;
    pr.degree = degree.data(); pr.nknots = nknots.data(); pr.knots = knots.data();
    pr.gdegree = degree.data(); pr.gnknots = nknots.data(); pr.gknots = knots.data();
    pr.coefs = coefs.data();
    pr.ndirichlet = 4; pr.dirichlet = dirichlet.data();
    pr.kappa_const = 1.0;
    pr.ufreq = 1;
    pr.quA = 1.0;
    pr.quB = 1;
    try {
        gsgpu::System S(0);
        S.setProblem(pr);
        S.refresh();
        S.assemble(GSGPU_PREC_FP64);
        const gsgpu::Sizes sz = S.sizes();
        std::vector<int> outer(size_t(sz.nfree) + 1), inner(size_t(sz.nnz));
        std::vector<double> values(size_t(sz.nnz)), b(size_t(sz.nfree)), x(size_t(sz.nfree));
        S.csrInto(outer.data(), inner.data(), values.data());
        S.rhs(b.data());
        gsgpu_solver_opts o = {GSGPU_SOLVER_CG_JACOBI, GSGPU_PREC_FP64, 1e-10, 1000, 4, 2, 2, 0.6, 1e-4, 1, 1.0};
        gsgpu_solve_info info{};
        const int rc = S.solve(o, x.data(), &info);
        const double l2 = S.l2Error(), h1 = S.h1Error();
        // the same system in mixed precision reaches the FP64 solution
        S.assemble(GSGPU_PREC_MIXED);
        o.precision = GSGPU_PREC_MIXED;
        o.tol = 1e-11;
        std::vector<double> xm(size_t(sz.nfree));
        gsgpu_solve_info im{};
        S.solve(o, xm.data(), &im);
        double num = 0.0, den = 0.0;
        for (size_t i = 0; i < x.size(); ++i) num += (xm[i] - x[i]) * (xm[i] - x[i]), den += x[i] * x[i];
        dump(out + "/ptr.i32", outer);
        dump(out + "/col.i32", inner);
        dump(out + "/val.f64", values);
        dump(out + "/rhs.f64", b);
        dump(out + "/x.f64", x);
        // errors surface as exceptions: an out-of-order call must throw gsgpu::Error
        bool threw = false;
        try {
            gsgpu::System T(0);
            T.assemble();
        } catch (const gsgpu::Error& e) {
            threw = e.code == GSGPU_ERR_STATE;
        }
        std::printf("%d %lld %d %.17g %.17g %.17g %d %.3g %d\n", sz.nfree, sz.nnz, info.iterations, info.relres, l2, h1,
                    rc == GSGPU_OK ? 1 : 0, std::sqrt(num / den), threw ? 1 : 0);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
