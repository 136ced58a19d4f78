"""The reference's gsPoissonSolver_test (unittests/gsPoissonSolver_test.cpp, Galerkin_test) restated
on the oracle: four glued degree-1 patches of the unit square with Dirichlet and Neumann sides,
manufactured solution, three uniform refinements after two initial ones; the L2 error must
converge at a rate above 1.85 (the test's tolerance; the expected rate is 2), measured from the last
two meshes and by a least-squares fit of log(error) against log(h)."""
import numpy as np

from gismo_gb300 import problems as P

CONVRATE_TOL = 1.85


def rates(errors, hs):
    e, h = np.log(np.asarray(errors)), np.log(np.asarray(hs))
    last = (e[-2] - e[-1]) / (h[-2] - h[-1])
    fit = np.polyfit(h, e, 1)[0]
    return last, fit


def test_galerkin_mms_rate_oracle():
    from oracle import oracle as O
    errs, hs = [], []
    for n in (8, 16, 32):
        prob = P.square_grid_mms(n, 1)
        o = O.OracleProblem(prob)
        o.assemble()
        x, it, _, _ = o.solve_cg(1e-12, 20000)
        errs.append(o.l2_error(x))
        hs.append(0.5 / n)
    last, fit = rates(errs, hs)
    assert last > CONVRATE_TOL and fit > CONVRATE_TOL, (errs, last, fit)
