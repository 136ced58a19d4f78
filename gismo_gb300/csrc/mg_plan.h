// Host set-up of the geometric h-multigrid hierarchy (gsGridHierarchy::buildByCoarsening,
// src/gsMultiGrid/gsGridHierarchy.hpp:57-101; gsMultiGridOp::init, src/gsMultiGrid/gsMultiGrid.hpp:69-95).
//
// Level 0 is the finest. Each coarser level removes every second interior knot of every
// discretisation basis (gsMultiBasis::uniformCoarsen_withTransfer), keeps the Dirichlet sides and
// the interfaces, and numbers its dofs with the same gsDofMapper rules. Its Galerkin operator
// P^T A P is computed on the device by the same sum-factorised contractions as the fine matrix,
// with the coarse basis tabulated at the finest Gauss points: coarse B-splines lie in the fine
// spline space, so this is P^T A P in exact arithmetic (rows/columns of free dofs). The transfer
// P (fine free dofs <- coarse free dofs) is the tensor product of 1-D knot-insertion matrices,
// assembled through the two levels' dof maps.
#pragma once

#include <vector>

#include "plan.h"

namespace gsgpu {

struct MgLevelPlan {
    ProblemDesc pd;   // patches carry this level's discretisation bases
    DofMap map;
    Layout L;         // on the finest quadrature grid; DevPatch::field_off points at level 0's fields
    Pattern pat;
    std::vector<int> diag;
    // transfer from this level to the next finer one: rows = finer free dofs, cols = this level's
    std::vector<int> Pptr, Pcol;
    std::vector<double> Pval;
    std::vector<int> Rptr, Rcol;  // P^T
    std::vector<double> Rval;
};

// coarse spline space: every second interior break removed
Basis1D coarsenBasis(const Basis1D& B);
// levels 1 .. nlevels-1 of the hierarchy below the finest problem (fine, fineMap, fineLayout)
void buildMgPlan(const ProblemDesc& fine, const DofMap& fineMap, const Layout& fineLayout, int nlevels,
                 std::vector<MgLevelPlan>& levels);

}  // namespace gsgpu
