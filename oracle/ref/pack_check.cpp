// Host-side check of the C++ drop-in's problem packing (include/gsGpuPoissonAssembler.h
// gsGpuProblemPack) against the reference's own objects, without a GPU: glued multipatch grids
// built by gsNurbsCreator (interfaces found by the reference's topology code, with its orientation
// flags), Dirichlet and Neumann sides from gsBoundaryConditions, packed and handed to a host-only
// context of libgsgpu; its dof map must equal the reference's gsDofMapper
// (gsMultiBasis::getMapper with dirichlet::elimination, iFace::glue) and its sizes the mapper's.
// Test infrastructure only; prints "ok" and exits 0 on success.
#include <cstdio>
#include <iostream>
#include <vector>

#include <gsNurbs/gsNurbsCreator.h>

#include "gsGpuPoissonAssembler.h"

using namespace gismo;

static int check(const gsMultiPatch<>& mp0, int refine, const char* name) {
    gsMultiPatch<> mp = mp0;
    gsMultiBasis<> mb(mp);
    mb.degreeElevate(1);
    for (int r = 0; r < refine; ++r) mb.uniformRefine();
    gsBoundaryConditions<> bc;
    gsConstantFunction<> zero(0.0, mp.parDim());
    std::vector<int> dsides, nsides;
    for (auto it = mp.bBegin(); it != mp.bEnd(); ++it) {
        // lower sides Dirichlet, upper sides Neumann
        const bool upper = it->side().parameter();
        bc.addCondition(it->patch, it->side(), upper ? condition_type::neumann : condition_type::dirichlet, &zero);
        (upper ? nsides : dsides).push_back(it->patch);
        (upper ? nsides : dsides).push_back(it->side().index());
    }
    gsDofMapper map;
    mb.getMapper(dirichlet::elimination, iFace::glue, bc, map, 0);
    gsGpuProblemPack<> pk;
    gsGpuFields F;
    pk.pack(mp, mb, dsides, F, 1.0, 1, GSGPU_DIRICHLET_INTERPOLATION, nsides);
    gsgpu_context* ctx = nullptr;
    if (gsgpu_create(&ctx, -1) != GSGPU_OK) { std::cerr << "create failed\n"; return 1; }
    int rc = gsgpu_set_problem(ctx, &pk.prob);
    if (rc == GSGPU_OK) rc = gsgpu_refresh(ctx);
    if (rc != GSGPU_OK) { std::cerr << name << ": " << gsgpu_last_error(ctx) << "\n"; gsgpu_destroy(ctx); return 1; }
    int n = 0, nb = 0, nl = 0;
    long long nnz = 0;
    gsgpu_sizes(ctx, &n, &nnz, &nb, &nl);
    std::vector<int> dm(static_cast<size_t>(nl));
    gsgpu_dof_map(ctx, dm.data());
    gsgpu_destroy(ctx);
    const gsVector<index_t> ref = map.asVector();
    if (n != map.freeSize() || nb != map.boundarySize() || index_t(dm.size()) != ref.size()) {
        std::cerr << name << ": sizes differ\n";
        return 1;
    }
    for (size_t i = 0; i < dm.size(); ++i)
        if (dm[i] != ref[index_t(i)]) { std::cerr << name << ": dof map differs at " << i << "\n"; return 1; }
    std::printf("%s: %d free, %d eliminated, %zu interfaces\n", name, n, nb, mp.interfaces().size());
    return 0;
}

int main() {
    int bad = 0;
    bad += check(gsNurbsCreator<>::BSplineSquareGrid(3, 2, 1.0), 3, "square grid 3x2");
    bad += check(gsNurbsCreator<>::BSplineCubeGrid(2, 2, 2, 1.0), 1, "cube grid 2x2x2");
    if (bad) return 1;
    std::printf("ok\n");
    return 0;
}
