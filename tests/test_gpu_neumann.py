"""Neumann boundary integrals (gsVisitorNeumann) on the GPU, beyond the reference fixtures (which
the fixture parity test covers with the plain FP64 path): the mixed-precision assembly, batches,
multigrid, and the convergence of the discrete solution under refinement.

Bars: the rhs within 1e-12 relative of the oracle's for every path (the Neumann sums are FP64 in
both precisions); solutions within 1e-8 (relative 2-norm) of the oracle's CG solution; on the
identity square with the exact flux as Neumann data, the L2 error of degree p falls at rate
p + 1 (>= p + 0.8 between successive halvings)."""
import numpy as np
import pytest

from gismo_gb300 import problems as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g
    g.build()


def _oracle(prob):
    from oracle import oracle as O
    o = O.OracleProblem(prob)
    o.assemble()
    return o


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_neumann_rhs_and_solution(precision):
    from gismo_gb300.assembler import GpuPoissonAssembler
    for prob in (P.mixed_boundary(P.displaced_single_patch(3, (9, 7, 8), (3, 2, 3), 12, 0.04, ufreq=2)),
                 P.mixed_boundary(P.displaced_single_patch(2, (40, 33), (4, 2), 13, 0.05, ufreq=2))):
        o = _oracle(prob)
        A = GpuPoissonAssembler(prob, device=0)
        A.assemble(precision)
        orhs = o.rhs()
        assert np.abs(A.rhs() - orhs).max() <= 1e-12 * np.abs(orhs).max()
        x, info = A.solve(tol=1e-11, max_iters=5000, precision=precision)
        assert info["converged"]
        xo, _, _, _ = o.solve_cg(1e-11, 5000)
        assert np.linalg.norm(x - xo) <= 1e-8 * np.linalg.norm(xo)
        A.close()


def test_neumann_batch_matches_oracle():
    from gismo_gb300.assembler import GpuPoissonBatch
    probs = [P.mixed_boundary(p) for p in P.patch_batch(count=12, seed=31, nmin=5, nmax=24)]
    B = GpuPoissonBatch(probs, device=0)
    B.assemble("fp64")
    rhs = B.rhs()
    off = B.offsets()
    xs, info = B.solve(tol=1e-10, max_iters=5000)
    assert info["converged"]
    h1 = B.h1_errors()
    for j, pr in enumerate(probs):
        o = _oracle(pr)
        orhs = o.rhs()
        a, b = off[j], off[j + 1]
        assert np.abs(rhs[a:b] - orhs).max() <= 1e-12 * np.abs(orhs).max(), j
        xo, _, _, _ = o.solve_cg(1e-10, 5000)
        assert np.linalg.norm(xs[j] - xo) <= 1e-7 * np.linalg.norm(xo), j
        oh1 = o.h1_error(xs[j])
        assert abs(h1[j] - oh1) <= 1e-9 * oh1, (j, h1[j], oh1)
    B.close()


def test_neumann_multigrid_matches_cg():
    from gismo_gb300.assembler import GpuPoissonAssembler
    prob = P.mixed_boundary(P.cube_grid(n=2, n_elem=8, p=2, seed=9, kappa_modes=8))
    o = _oracle(prob)
    xo, _, _, _ = o.solve_cg(1e-11, 5000)
    A = GpuPoissonAssembler(prob, device=0)
    A.assemble("fp64")
    x, info = A.solve(tol=1e-11, max_iters=200, method="mg", mg_levels=3)
    assert info["converged"]
    assert np.linalg.norm(x - xo) <= 1e-8 * np.linalg.norm(xo)
    A.close()


def test_neumann_exact_flux_converges():
    """u = sin(pi x) sin(pi y) on the unit square, Dirichlet west/south, its flux on east/north:
    L2 error at rate p + 1, H1 seminorm error at rate p."""
    from gismo_gb300.assembler import GpuPoissonAssembler
    p = 2
    errs, h1s = [], []
    for n in (8, 16, 32):
        A = GpuPoissonAssembler(P.mixed_boundary(P.square_poisson(n, p)), device=0)
        A.assemble("fp64")
        _, info = A.solve(tol=1e-13, max_iters=5000)
        assert info["converged"]
        errs.append(A.l2_error())
        h1s.append(A.h1_error())
        A.close()
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert np.all(rates >= p + 0.8), (errs, rates)
    rates = np.log2(np.array(h1s[:-1]) / np.array(h1s[1:]))
    assert np.all(rates >= p - 0.2), (h1s, rates)


def test_reference_mms_test_on_device():
    """gsPoissonSolver_test (Galerkin_test) on the device: four glued degree-1 patches, Dirichlet
    and Neumann sides, L2 rate above the test's 1.85 from the last two meshes and by least squares;
    the device L2 errors within 1e-9 of the oracle's quadrature of the same solutions."""
    from gismo_gb300.assembler import GpuPoissonAssembler
    from tests.test_poisson_solver_mms import CONVRATE_TOL, rates
    errs, hs = [], []
    for n in (8, 16, 32):
        prob = P.square_grid_mms(n, 1)
        A = GpuPoissonAssembler(prob, device=0)
        A.assemble("fp64")
        x, info = A.solve(tol=1e-12, max_iters=20000)
        assert info["converged"]
        e = A.l2_error()
        o = _oracle(prob)
        oe = o.l2_error(x)
        assert abs(e - oe) <= 1e-9 * oe
        errs.append(e)
        hs.append(0.5 / n)
        A.close()
    last, fit = rates(errs, hs)
    assert last > CONVRATE_TOL and fit > CONVRATE_TOL, (errs, last, fit)
