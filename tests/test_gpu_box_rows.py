"""Box rows of the FP32 SpMVs: rows whose columns are the row plus one common offset table take
their column offsets from shared memory instead of the CSR arrays.

Bars: the same slots in the same order, so FP64 and mixed-precision CG give bitwise the same
solution and iteration count with and without box rows; the SpMV reads fewer bytes with them;
rows that only look like box rows (same length, other columns) are not taken for them."""
import os

import numpy as np
import pytest

from gismo_gb300 import problems as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g
    g.build()


def _solve(prob, box, precision):
    """Box rows belong to the CSR products: the half-diagonal inner operator of single patches is
    switched off (GSGPU_NO_SDIA=1) so that the mixed path runs them."""
    from gismo_gb300.assembler import GpuPoissonAssembler
    if box:
        os.environ.pop("GSGPU_NO_BOX_ROWS", None)
    else:
        os.environ["GSGPU_NO_BOX_ROWS"] = "1"
    os.environ["GSGPU_NO_SDIA"] = "1"
    try:
        A = GpuPoissonAssembler(prob, device=0)
        A.assemble(precision)
        A.set_profiling(True)
        x, info = A.solve(tol=1e-10, max_iters=5000, precision=precision)
        stats = A.spmv_stats()
        A.close()
    finally:
        os.environ.pop("GSGPU_NO_BOX_ROWS", None)
        os.environ.pop("GSGPU_NO_SDIA", None)
    return x, info, stats


CASES = {
    "volume_p3_28": lambda: P.volume_poisson(28, 3, seed=4),
    "disp3d_p232_30x26x28": lambda: P.displaced_single_patch(3, (30, 26, 28), (2, 3, 2), 6, 0.04),
    "disp2d_p4_160x150": lambda: P.displaced_single_patch(2, (160, 150), (4, 4), 8, 0.05, ufreq=2),
}


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_box_rows_are_bitwise_neutral(case, precision):
    prob = CASES[case]()
    xb, ib, sb = _solve(prob, True, precision)
    xn, inn, sn = _solve(prob, False, precision)
    assert ib["converged"] and inn["converged"]
    assert ib["iterations"] == inn["iterations"]
    assert np.array_equal(xb, xn)
    # bytes per SpMV launch: the FP32 box rows skip their column offsets (the FP64 SpMV keeps the
    # plain CSR rows)
    if precision == "mixed":
        assert sb[2] < 0.97 * sn[2], (sb, sn)
    else:
        assert sb[2] == sn[2], (sb, sn)


def test_multipatch_rows_are_checked():
    """Interface-coupled numbering: rows of the longest length need not share the offsets; the
    solution stays bitwise equal either way."""
    prob = P.cube_grid(n=3, n_elem=8, p=2, seed=5, kappa_modes=8)
    xb, ib, _ = _solve(prob, True, "fp64")
    xn, inn, _ = _solve(prob, False, "fp64")
    assert ib["iterations"] == inn["iterations"]
    assert np.array_equal(xb, xn)
