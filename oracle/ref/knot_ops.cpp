// Applies the reference's knot-vector operations to a knot vector given on the command line and
// prints the result (test infrastructure only; never shipped):
//   gsknot <degree> <elevate> <refine> t_0 t_1 ... t_m
// degreeElevate(elevate) then uniformRefine() `refine` times (gsKnotVector::degreeElevate,
// uniformRefine, src/gsNurbs/gsKnotVector.hpp:820-834, 937-941); prints "<degree> t_0 .. t_k".
#include <cstdio>
#include <cstdlib>
#include <vector>

#include <gsNurbs/gsKnotVector.h>

using namespace gismo;

int main(int argc, char** argv) {
    if (argc < 5) { std::fprintf(stderr, "usage: gsknot degree elevate refine knots...\n"); return 2; }
    const int p = std::atoi(argv[1]), e = std::atoi(argv[2]), r = std::atoi(argv[3]);
    std::vector<real_t> t;
    for (int i = 4; i < argc; ++i) t.push_back(std::strtod(argv[i], nullptr));
    gsKnotVector<> kv(t, p);
    if (e > 0) kv.degreeElevate(short_t(e));
    for (int i = 0; i < r; ++i) kv.uniformRefine();
    std::printf("%d", int(kv.degree()));
    for (auto it = kv.begin(); it != kv.end(); ++it) std::printf(" %.17g", *it);
    std::printf("\n");
    return 0;
}
