"""CG preconditioned by the h-multigrid V-cycle on the GPU, against the reference fixture and the
CPU oracle (gsMultiGridOp + gsConjugateGradient restated).

Bars: outer iteration counts within one of the reference's (the coarsest level is solved to a
tight tolerance by Jacobi-PCG instead of a Cholesky factor, and the outer CG uses the
Polak-Ribiere beta, so a difference of one iteration is allowed); the true FP64 residual of the
returned solution at the requested tolerance; the discrete L2 error to >= 3 significant digits of
the reference's. The mixed form (FP32 V-cycle, FP64 outer CG on the double-float operator) must
reach the FP64 solution within 1e-8 relative."""
import numpy as np
import pytest

from gismo_gb300 import problems as P
from tests.golden_cases import golden_problem, load_golden
from tests.test_oracle_golden import _csr_from_csc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g
    g.build()


def _assembler(prob):
    from gismo_gb300.assembler import GpuPoissonAssembler
    return GpuPoissonAssembler(prob, device=0)


def _mg(A, prob, tol, precision="fp64", levels=None):
    return A.solve(tol=tol, max_iters=500, method="mg", precision=precision,
                   mg_levels=levels or prob.mg_levels, mg_npre=prob.mg_npre, mg_npost=prob.mg_npost,
                   mg_damping=prob.mg_damping, mg_cycles=prob.mg_cycles, mg_cgc_damping=prob.mg_cgc_damping)


@pytest.mark.parametrize("name", ["cubegrid2_p2_n4_mg", "disp2d_p2_32x24_mgw"])
def test_mg_matches_reference_fixture(name):
    """V-cycle (3D, 3 levels) and W-cycle with coarse-correction damping 0.8 (2D, 4 levels)."""
    from oracle import oracle as O
    g = load_golden(name)
    prob = golden_problem(name)
    A = _assembler(prob)
    A.assemble()
    x, info = _mg(A, prob, prob.tol)
    assert info["converged"], info
    assert abs(info["iterations"] - int(g["iters"])) <= 1, (info, int(g["iters"]))
    K = _csr_from_csc(g)
    b = g["rhs"]
    assert np.linalg.norm(b - K @ x) <= 1.01 * prob.tol * np.linalg.norm(b)
    o = O.OracleProblem(prob)
    o.assemble()
    l2 = o.l2_error(x)
    assert abs(l2 - float(g["l2"])) <= 5e-4 * float(g["l2"])
    assert abs(A.l2_error() - l2) <= 1e-9 * l2
    A.close()


CASES = {
    # (problem, levels)
    "cubegrid3_p2_n4": (lambda: P.cube_grid(n=3, n_elem=4, p=2, seed=5, kappa_modes=32), 3),
    "disp3d_p3_16": (lambda: P.volume_poisson(16, 3, seed=2), 3),
    "disp2d_p3_48x40": (lambda: P.displaced_single_patch(2, (48, 40), (3, 3), 7, 0.05, ufreq=2), 4),
    "disp3d_p232_8x8x12": (lambda: P.displaced_single_patch(3, (8, 8, 12), (2, 3, 2), 11, 0.04), 3),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_mg_matches_oracle(case):
    from oracle import oracle as O
    make, levels = CASES[case]
    prob = make()
    o = O.OracleProblem(prob)
    o.assemble()
    xo, it, _, _ = o.solve_mg(1e-8, 500, levels, 2, 2, 0.6)
    A = _assembler(prob)
    A.assemble()
    x, info = A.solve(tol=1e-8, max_iters=500, method="mg", mg_levels=levels)
    assert info["converged"], info
    assert abs(info["iterations"] - it) <= 1, (info, it)
    K = A.matrix()
    b = A.rhs()
    assert np.linalg.norm(b - K @ x) <= 1.01e-8 * np.linalg.norm(b)
    assert abs(o.l2_error(x) - o.l2_error(xo)) <= 5e-4 * o.l2_error(xo)
    A.close()


@pytest.mark.parametrize("case", ["cubegrid3_p2_n4", "disp2d_p3_48x40"])
@pytest.mark.parametrize("cycles,cgc", [(2, 1.0), (1, 0.7), (2, 0.85)])
def test_mg_cycles_match_oracle(case, cycles, cgc):
    """NumCycles (W-cycle) and CoarseGridCorrectionDamping against the oracle's multiGridStep."""
    from oracle import oracle as O
    make, levels = CASES[case]
    prob = make()
    o = O.OracleProblem(prob)
    o.assemble()
    xo, it, _, _ = o.solve_mg(1e-8, 500, levels, 2, 2, 0.6, cycles, cgc)
    A = _assembler(prob)
    A.assemble()
    x, info = A.solve(tol=1e-8, max_iters=500, method="mg", mg_levels=levels, mg_cycles=cycles,
                      mg_cgc_damping=cgc)
    assert info["converged"], info
    assert abs(info["iterations"] - it) <= 1, (info, it)
    b = A.rhs()
    assert np.linalg.norm(b - A.matrix() @ x) <= 1.01e-8 * np.linalg.norm(b)
    assert np.linalg.norm(x - xo) <= 1e-6 * np.linalg.norm(xo)
    # the mixed form of the same cycle
    A.assemble("mixed")
    xm, im = A.solve(tol=1e-8, max_iters=500, method="mg", precision="mixed", mg_levels=levels,
                     mg_cycles=cycles, mg_cgc_damping=cgc)
    assert im["converged"] and im["iterations"] <= info["iterations"] + 2, (im, info)
    assert np.linalg.norm(xm - xo) <= 1e-6 * np.linalg.norm(xo)
    A.close()


def test_mg_cycle_limit_is_an_error():
    """A cycle count whose coarse visits explode is refused, not captured."""
    from gismo_gb300._lib import GsGpuError
    prob = P.displaced_single_patch(2, (48, 40), (3, 3), 7, 0.05, ufreq=2)
    A = _assembler(prob)
    A.assemble()
    with pytest.raises(GsGpuError):
        A.solve(tol=1e-8, method="mg", mg_levels=4, mg_cycles=100)
    x, info = A.solve(tol=1e-8, method="mg", mg_levels=4)
    assert info["converged"]
    A.close()


@pytest.mark.parametrize("case", ["cubegrid3_p2_n4", "disp3d_p3_16", "disp2d_p3_48x40"])
def test_mg_mixed_matches_fp64(case):
    make, levels = CASES[case]
    prob = make()
    A = _assembler(prob)
    A.assemble("fp64")
    x64, i64 = A.solve(tol=1e-13, max_iters=500, method="mg", mg_levels=levels)
    assert i64["converged"], i64
    A.assemble("mixed")
    xm, im = A.solve(tol=1e-11, max_iters=500, method="mg", precision="mixed", mg_levels=levels)
    assert im["converged"], im
    # an FP32 V-cycle preconditions about as well as the FP64 one
    assert im["iterations"] <= i64["iterations"] + 2
    err = np.linalg.norm(xm - x64) / np.linalg.norm(x64)
    assert err <= 1e-8, (err, im, i64)
    A.close()


def test_mg_repeat_and_reassemble():
    """Repeated solves are bitwise identical; new control points rebuild the coarse operators."""
    p1 = P.displaced_single_patch(2, (16, 12), (2, 3), 3, 0.05)
    p2 = P.displaced_single_patch(2, (16, 12), (2, 3), 4, 0.05)
    p2.kappa_amp, p2.kappa_k, p2.kappa_phase = p1.kappa_amp, p1.kappa_k, p1.kappa_phase
    A = _assembler(p1)
    A.assemble()
    xa, ia = A.solve(tol=1e-10, method="mg", mg_levels=3)
    xb, ib = A.solve(tol=1e-10, method="mg", mg_levels=3)
    assert np.array_equal(xa, xb) and ia["iterations"] == ib["iterations"]
    A.set_coefs(p2.patches[0].coefs)
    A.assemble()
    x1, i1 = A.solve(tol=1e-10, method="mg", mg_levels=3)
    B = _assembler(p2)
    B.assemble()
    x2, i2 = B.solve(tol=1e-10, method="mg", mg_levels=3)
    assert np.array_equal(x1, x2) and i1["iterations"] == i2["iterations"]
    A.close()
    B.close()


def test_mg_beats_jacobi_iterations():
    prob = P.volume_poisson(16, 3, seed=2)
    A = _assembler(prob)
    A.assemble()
    _, ij = A.solve(tol=1e-8)
    _, im = A.solve(tol=1e-8, method="mg", mg_levels=3)
    assert im["converged"] and im["iterations"] * 2 < ij["iterations"], (im, ij)
    A.close()
