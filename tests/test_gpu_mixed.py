"""Mixed precision on the GPU: the double-float (two-FP32) assembly reproduces the FP64 operator,
and the FP32 inner CG with FP64-accurate residual replacement reaches the FP64 solution.

Bars: the df32 operator and rhs within 1e-11 relative of the FP64 oracle (absolute floor 1e-13 x
the row's largest entry); the mixed solution within 1e-8 relative (2-norm) of a tightly converged
FP64 GPU solution, its reported residual being the true residual."""
import numpy as np
import pytest

from gismo_gb300 import problems as P

pytestmark = pytest.mark.gpu

CASES = {
    "square_p2_64": lambda: P.square_poisson(64, 2),
    "disp2d_p4_40x33": lambda: P.displaced_single_patch(2, (40, 33), (4, 4), 9, 0.05, ufreq=3),
    "disp3d_p3_16": lambda: P.volume_poisson(16, 3, seed=2),
    "cubegrid2_p2_n4": lambda: P.cube_grid(n=2, n_elem=4, p=2, seed=3, kappa_modes=8),
}


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g
    g.build()


@pytest.mark.parametrize("case", sorted(CASES))
def test_df32_operator_matches_fp64_oracle(case):
    from gismo_gb300.assembler import GpuPoissonAssembler
    from oracle import oracle as O
    prob = CASES[case]()
    o = O.OracleProblem(prob)
    o.assemble()
    optr, ocol, oval = o.csr()
    A = GpuPoissonAssembler(prob)
    A.assemble("mixed")
    ptr, col, val = A.csr()
    assert np.array_equal(ptr, optr) and np.array_equal(col, ocol)
    rowmax = np.maximum.reduceat(np.abs(oval), optr[:-1])
    floor = np.repeat(rowmax, np.diff(optr)) * 1e-13
    assert np.all(np.abs(val - oval) <= 1e-11 * np.abs(oval) + floor)
    assert np.abs(A.rhs() - o.rhs()).max() <= 1e-11 * np.abs(o.rhs()).max()
    A.close()


@pytest.mark.parametrize("case", sorted(CASES))
def test_mixed_solution_matches_fp64(case):
    from gismo_gb300.assembler import GpuPoissonAssembler
    prob = CASES[case]()
    A = GpuPoissonAssembler(prob)
    A.assemble("fp64")
    x64, i64 = A.solve(tol=1e-13, max_iters=20000)
    A.assemble("mixed")
    xm, im = A.solve(tol=1e-11, precision="mixed", max_iters=20000)
    assert im["converged"], im
    assert im["relres"] < 1e-11 and im["refinements"] >= 1
    err = np.linalg.norm(xm - x64) / np.linalg.norm(x64)
    assert err <= 1e-8, (err, im, i64)
    # the reported residual is the true one: check it on the host in FP64
    K, b = A.matrix(), A.rhs()
    assert np.linalg.norm(b - K @ xm) <= 2e-11 * np.linalg.norm(b)
    A.close()


def _high_waves():
    """A displaced 3D degree-2 patch whose kappa modes reach wave number 8 (the point kernel's
    larger powers table; the other cases stay at 4)."""
    import numpy as np
    prob = P.displaced_single_patch(3, (6, 7, 5), (2, 2, 2), 11, 0.04)
    P.set_kappa_fourier(prob, np.random.default_rng(5), 12, kmax=8)
    assert int(np.max(prob.kappa_k)) > 4
    return prob


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_high_wave_numbers_match_the_oracle(precision):
    """Fourier modes with wave numbers above 4 take the point kernel with the 9-entry powers
    table: operator and rhs against the FP64 oracle (FP64 1e-12, df32 1e-11)."""
    from gismo_gb300.assembler import GpuPoissonAssembler
    from oracle import oracle as O
    prob = _high_waves()
    o = O.OracleProblem(prob)
    o.assemble()
    optr, ocol, oval = o.csr()
    A = GpuPoissonAssembler(prob)
    A.assemble(precision)
    ptr, col, val = A.csr()
    tol = 1e-12 if precision == "fp64" else 1e-11
    assert np.array_equal(ptr, optr) and np.array_equal(col, ocol)
    rowmax = np.maximum.reduceat(np.abs(oval), optr[:-1])
    floor = np.repeat(rowmax, np.diff(optr)) * (1e-14 if precision == "fp64" else 1e-13)
    assert np.all(np.abs(val - oval) <= tol * np.abs(oval) + floor)
    assert np.abs(A.rhs() - o.rhs()).max() <= tol * np.abs(o.rhs()).max()
    A.close()


def test_mixed_needs_mixed_assembly():
    from gismo_gb300.assembler import GpuPoissonAssembler
    from gismo_gb300._lib import GsGpuError, ERR_STATE
    A = GpuPoissonAssembler(P.square_poisson(8, 2))
    A.assemble("fp64")
    with pytest.raises(GsGpuError) as e:
        A.solve(precision="mixed")
    assert e.value.code == ERR_STATE
    A.close()


TILE_CASES = {
    "volume_p3_16": lambda: P.volume_poisson(16, 3, seed=2),
    "volume_p3_40": lambda: P.volume_poisson(40, 3, seed=6),  # two row segments per line
    "disp3d_p2_40x10x12": lambda: P.displaced_single_patch(3, (40, 10, 12), (2, 2, 2), 4, 0.04),
    "disp3d_p3x2x4_36x8x9": lambda: P.displaced_single_patch(3, (36, 8, 9), (3, 2, 4), 5, 0.04),
    "cubegrid2_p2_n4": lambda: P.cube_grid(n=2, n_elem=4, p=2, seed=3, kappa_modes=8),
}


@pytest.mark.parametrize("case", sorted(TILE_CASES))
def test_stage31_tiles_are_bitwise_neutral(case):
    """Stage 1 of the df32 stiffness contraction in shared-memory tiles gives the operator of the
    row kernel bit for bit (same products, same compensated summation order)."""
    import os
    from gismo_gb300.assembler import GpuPoissonAssembler
    prob = TILE_CASES[case]()
    vals = []
    for off in (False, True):
        if off:
            os.environ["GSGPU_NO_TILE31"] = "1"
        try:
            A = GpuPoissonAssembler(prob)
            A.assemble("mixed")
            vals.append(A.csr()[2])
            A.close()
        finally:
            os.environ.pop("GSGPU_NO_TILE31", None)
    assert np.array_equal(vals[0], vals[1])


SDIA_CASES = {
    "volume_p3_16": lambda: P.volume_poisson(16, 3, seed=2),
    "disp2d_p4_40x33": lambda: P.displaced_single_patch(2, (40, 33), (4, 4), 9, 0.05, ufreq=3),
    "disp3d_p232_5x6x7": lambda: P.displaced_single_patch(3, (5, 6, 7), (2, 3, 2), 8, 0.04),
    "square_p2_64_neu": lambda: P.mixed_boundary(P.square_poisson(64, 2)),
    "disp3d_p3_12_neu": lambda: P.mixed_boundary(P.volume_poisson(12, 3, seed=3)),
    "disp3d_p1_14x9x11": lambda: P.displaced_single_patch(3, (14, 9, 11), (1, 1, 1), 6, 0.04),
}


@pytest.mark.parametrize("case", sorted(SDIA_CASES))
def test_half_diagonal_inner_operator(case, monkeypatch):
    """Single patches whose free dofs form one box run the inner FP32 products on the half-diagonal
    form (sdia.cu). Against the CSR form of the same FP32 values (GSGPU_NO_SDIA=1): both mixed
    solutions within 1e-8 of the tight FP64 solution, iteration counts within a few of each other,
    and the half-diagonal path is the one that ran (its per-product bytes)."""
    from gismo_gb300.assembler import GpuPoissonAssembler
    prob = SDIA_CASES[case]()
    A = GpuPoissonAssembler(prob)
    A.assemble("fp64")
    x64, _ = A.solve(tol=1e-13, max_iters=20000)
    A.close()
    out = {}
    for sdia in (True, False):
        if sdia:
            monkeypatch.delenv("GSGPU_NO_SDIA", raising=False)
        else:
            monkeypatch.setenv("GSGPU_NO_SDIA", "1")
        A = GpuPoissonAssembler(prob)
        A.assemble("mixed")
        xm, im = A.solve(tol=1e-11, precision="mixed", max_iters=20000)
        assert im["converged"], im
        err = np.linalg.norm(xm - x64) / np.linalg.norm(x64)
        assert err <= 1e-8, (case, sdia, err, im)
        A.set_profiling(True)
        A.solve(tol=1e-11, precision="mixed", max_iters=20000, download=False)
        _, _, nbytes = A.spmv_stats()
        A.set_profiling(False)
        n = len(xm)
        p = list(prob.patches[0].degree) + [0] * (3 - prob.dim)
        nh = 1 + (np.prod([2 * q + 1 for q in p]) - 1) // 2
        assert (nbytes == nh * n * 4 + 8 * n) == sdia, (case, sdia, nbytes, nh * n * 4 + 8 * n)
        out[sdia] = im["iterations"]
        A.close()
    assert abs(out[True] - out[False]) <= max(3, out[False] // 20), out


@pytest.mark.parametrize("variant", ["tma", "rows4"])
@pytest.mark.parametrize("case", sorted(SDIA_CASES))
def test_half_diagonal_variants_are_bitwise_neutral(case, variant, monkeypatch):
    """The variants of the half-diagonal product form the same products in the same order as the
    default one-row load-based product: the TMA-fed one (GSGPU_SDIA_TMA=1, tiled bulk copies into a
    shared-memory ring) and the four-rows-per-thread one (GSGPU_SDIA_INNER=2, 16-byte loads, the
    window shifts instantiated per line residue); the mixed solves give the same bits. The cases
    cover odd and even box widths (every residue of the line offsets modulo 4), degrees 2 to 4 per
    direction, and row counts that are not a multiple of 4."""
    from gismo_gb300.assembler import GpuPoissonAssembler
    prob = SDIA_CASES[case]()
    xs = []
    for on in (True, False):
        for k in ("GSGPU_SDIA_TMA", "GSGPU_REQUIRE_TMA", "GSGPU_SDIA_INNER"):
            monkeypatch.delenv(k, raising=False)
        if on and variant == "tma":
            monkeypatch.setenv("GSGPU_SDIA_TMA", "1")
            monkeypatch.setenv("GSGPU_REQUIRE_TMA", "1")  # fail loudly if the tensor maps are refused
        elif on:
            monkeypatch.setenv("GSGPU_SDIA_INNER", "2")
        else:
            monkeypatch.setenv("GSGPU_SDIA_INNER", "0")
        A = GpuPoissonAssembler(prob)
        A.assemble("mixed")
        assert A.tuned_variants()[2] == ({"tma": 1, "rows4": 2}[variant] if on else 0)
        x, info = A.solve(tol=1e-11, precision="mixed", max_iters=20000)
        assert info["converged"], info
        xs.append((x, info["iterations"]))
        A.close()
    assert xs[0][1] == xs[1][1]
    assert np.array_equal(xs[0][0], xs[1][0])
