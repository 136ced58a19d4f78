"""GPU parity: the CUDA path (through the C ABI) against the reference fixtures and the CPU oracle.

Bars: dof map and sparsity pattern bit-exact; FP64 matrix and rhs entries within
1e-12 relative (absolute floor 1e-14 x the row's largest entry for entries that cancel to ~0);
CG iteration counts within one of the reference's; the discrete L2 error to >= 3 significant
digits."""
import os

import numpy as np
import pytest

from gismo_gb300 import problems as P
from tests.golden_cases import golden_problem, load_golden
from tests.test_oracle_golden import GOLDEN, _csr_from_csc

pytestmark = pytest.mark.gpu

REL = 1e-12
FLOOR = 1e-14


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g
    g.build()


def _assembler(prob):
    from gismo_gb300.assembler import GpuPoissonAssembler
    return GpuPoissonAssembler(prob, device=0)


def _check_values(val, ref_val, ref_ptr):
    rowmax = np.maximum.reduceat(np.abs(ref_val), ref_ptr[:-1])
    floor = np.repeat(rowmax, np.diff(ref_ptr)) * FLOOR
    err = np.abs(val - ref_val) - (REL * np.abs(ref_val) + floor)
    assert np.all(err <= 0), f"max excess {err.max():.3e}"


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_fp64_matches_reference_fixture(path):
    from oracle import oracle as O
    name = os.path.basename(path)[:-4]
    g = load_golden(name)
    prob = golden_problem(name)
    A = _assembler(prob)
    A.assemble()
    assert np.array_equal(A.dofMapper(), g["dofmap"])
    ptr, col, val = A.csr()
    K = _csr_from_csc(g)
    assert np.array_equal(ptr, K.indptr) and np.array_equal(col, K.indices)
    _check_values(val, K.data, K.indptr)
    rhs = A.rhs()
    assert np.abs(rhs - g["rhs"]).max() <= REL * np.abs(g["rhs"]).max()
    if len(g["ddof"]):
        assert np.abs(A.fixedDofs() - g["ddof"]).max() <= REL * max(1.0, np.abs(g["ddof"]).max())
    if prob.solver == "cg":
        x, info = A.solve(tol=prob.tol, max_iters=prob.maxit)
        assert info["converged"]
        assert abs(info["iterations"] - int(g["iters"])) <= 1
        assert np.linalg.norm(x - g["x"]) <= 1e-8 * np.linalg.norm(g["x"])
        o = O.OracleProblem(prob)
        o.assemble()
        l2 = o.l2_error(x)
        assert abs(l2 - float(g["l2"])) <= 5e-4 * float(g["l2"])
        # the device quadrature of gsField::distanceL2 / distanceH1 on the same solution
        assert abs(A.l2_error() - l2) <= 1e-9 * l2
        h1 = o.h1_error(x)
        assert abs(h1 - float(g["h1"])) <= 5e-4 * float(g["h1"])
        assert abs(A.h1_error() - h1) <= 1e-9 * h1
    A.close()


@pytest.mark.parametrize("case", ["disp3d_p3_16", "disp2d_p4_40x33", "cubegrid3_p2_n3"])
def test_fp64_matches_oracle(case):
    """Sizes beyond the fixtures, against the CPU oracle on the same seeded inputs."""
    from oracle import oracle as O
    if case == "disp3d_p3_16":
        prob = P.volume_poisson(16, 3, seed=2)
    elif case == "disp2d_p4_40x33":
        prob = P.displaced_single_patch(2, (40, 33), (4, 4), 9, 0.05, ufreq=3)
    else:
        prob = P.cube_grid(n=3, n_elem=3, p=2, seed=5, kappa_modes=32)
        prob.solver = "cg"
    o = O.OracleProblem(prob)
    o.assemble()
    A = _assembler(prob)
    A.assemble()
    assert np.array_equal(A.dofMapper(), o.dofmap())
    ptr, col, val = A.csr()
    optr, ocol, oval = o.csr()
    assert np.array_equal(ptr, optr) and np.array_equal(col, ocol)
    _check_values(val, oval, optr)
    assert np.abs(A.rhs() - o.rhs()).max() <= REL * np.abs(o.rhs()).max()
    x, info = A.solve(tol=1e-10)
    xo, it, _, _ = o.solve_cg(1e-10, 1000)
    assert info["converged"] and abs(info["iterations"] - it) <= 1
    assert np.linalg.norm(x - xo) <= 1e-8 * np.linalg.norm(xo)
    A.close()


def test_full_size_volume_properties():
    """The 3D degree-3 64^3 configuration at full size: properties that do not need the oracle."""
    prob = P.volume_poisson(64, 3, seed=1)
    A = _assembler(prob)
    A.assemble()
    nf, nnz, nb, nl = A.sizes()
    assert (nf, nnz) == (274625, 86938307)
    K = A.matrix()
    d = K.diagonal()
    assert np.all(d > 0)
    # symmetry of the assembled operator (entries computed independently per (i,j))
    D = (K - K.T).tocoo()
    assert np.abs(D.data).max() <= 1e-13 * np.abs(K.data).max()
    assert A.min_jacobian() > 0.2 * 0  # positive Jacobian everywhere
    x, info = A.solve(tol=1e-10)
    assert info["converged"] and info["iterations"] < 400
    # A x = b to the stopping tolerance, checked in FP64 on the host
    b = A.rhs()
    assert np.linalg.norm(b - K @ x) <= 2e-10 * np.linalg.norm(b)
    A.close()


def test_set_coefs_reassembles_new_geometry():
    """Changing control points without refresh() gives the same system as a fresh assembler."""
    p1 = P.displaced_single_patch(2, (9, 8), (3, 3), 3, 0.05)
    p2 = P.displaced_single_patch(2, (9, 8), (3, 3), 4, 0.05)
    p2.kappa_amp, p2.kappa_k, p2.kappa_phase = p1.kappa_amp, p1.kappa_k, p1.kappa_phase
    A = _assembler(p1)
    A.assemble()
    A.set_coefs(p2.patches[0].coefs)
    A.assemble()
    B = _assembler(p2)
    B.assemble()
    assert np.array_equal(A.csr()[2], B.csr()[2])
    assert np.array_equal(A.rhs(), B.rhs())
    A.close()
    B.close()


def test_inverted_geometry_is_reported():
    """A folded map (det J <= 0) is a status code, not a fault (G+Smo: GISMO_ENSURE)."""
    from gismo_gb300._lib import GsGpuError, ERR_JACOBIAN
    prob = P.square_poisson(6, 2)
    c = prob.patches[0].coefs.copy()
    c[:, 0] = 1.0 - c[:, 0]  # mirror x: det J < 0 everywhere
    prob.patches[0].coefs = c
    A = _assembler(prob)
    with pytest.raises(GsGpuError) as e:
        A.assemble()
    assert e.value.code == ERR_JACOBIAN
    A.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_l2_error_on_device(precision):
    """gsField::distanceL2 and distanceH1 on the device against the oracle's quadrature of the same
    solution, for a 3D and a multipatch case, after either assembly precision."""
    from oracle import oracle as O
    for prob in (P.volume_poisson(12, 3, seed=4), P.cube_grid(n=2, n_elem=5, p=2, seed=6, kappa_modes=8)):
        A = _assembler(prob)
        A.assemble(precision)
        x, info = A.solve(tol=1e-12, max_iters=5000, precision=precision)
        assert info["converged"]
        o = O.OracleProblem(prob)
        o.assemble()
        l2 = o.l2_error(x)
        assert abs(A.l2_error() - l2) <= 1e-9 * l2, (A.l2_error(), l2)
        h1 = o.h1_error(x)
        assert abs(A.h1_error() - h1) <= 1e-9 * h1, (A.h1_error(), h1)
        A.close()


def test_device_pattern_equals_host_pattern(monkeypatch):
    """Problems without interfaces build their pattern on the device: the CSR arrays, rhs and CG
    solution are bitwise those of the host builder (GSGPU_HOST_PATTERN forces the host path)."""
    from gismo_gb300.assembler import GpuPoissonAssembler, GpuPoissonBatch
    cases = [lambda: GpuPoissonAssembler(P.displaced_single_patch(3, (5, 6, 7), (2, 3, 2), 8, 0.04), device=0),
             lambda: GpuPoissonBatch(P.patch_batch(count=9, seed=4, nmin=4, nmax=20), device=0)]
    for make in cases:
        out = []
        for host in (False, True):
            if host:
                monkeypatch.setenv("GSGPU_HOST_PATTERN", "1")
            else:
                monkeypatch.delenv("GSGPU_HOST_PATTERN", raising=False)
            A = make()
            A.assemble("fp64")
            x, _ = A.solve(tol=1e-10)
            x = np.concatenate(x) if isinstance(x, list) else x
            out.append((A.csr(), A.rhs(), x))
            A.close()
        (pa, ca, va), ra, xa = out[0]
        (pb, cb, vb), rb, xb = out[1]
        assert np.array_equal(pa, pb) and np.array_equal(ca, cb) and np.array_equal(va, vb)
        assert np.array_equal(ra, rb) and np.array_equal(xa, xb)


def test_problem_from_xml_on_device(tmp_path):
    """A problem read from a G+Smo XML file (two glued squares, refined and degree-elevated, with
    Neumann data on the upper sides) through the C ABI against the oracle on the same input."""
    from oracle import oracle as O
    from gismo_gb300 import xmlio
    sq = [P.identity_patch(2, (1, 1), (1, 1)), P.identity_patch(2, (1, 1), (1, 1))]
    sq[1].coefs = sq[1].coefs - np.array([1.0, 0.0])
    f = str(tmp_path / "two.xml")
    xmlio.write_xml(P.Problem(2, sq, interfaces=[(1, 2, 0, 1)]), f)
    prob = xmlio.problem_from_xml(f, refine=4, elevate=1, neumann=[(0, 2), (0, 4), (1, 4)])
    o = O.OracleProblem(prob)
    o.assemble()
    A = _assembler(prob)
    A.assemble()
    assert np.array_equal(A.dofMapper(), o.dofmap())
    ptr, col, val = A.csr()
    optr, ocol, oval = o.csr()
    assert np.array_equal(ptr, optr) and np.array_equal(col, ocol)
    _check_values(val, oval, optr)
    assert np.abs(A.rhs() - o.rhs()).max() <= REL * np.abs(o.rhs()).max()
    x, info = A.solve(tol=1e-11)
    xo, _, _, _ = o.solve_cg(1e-11, 1000)
    assert info["converged"] and np.linalg.norm(x - xo) <= 1e-8 * np.linalg.norm(xo)
    A.close()


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_mass_matrix_matches_reference_fixture(path):
    """gsGenericAssembler::assembleMass on the device (gsgpu_mass_csr) against the reference's own
    mass matrix: the stiffness pattern, values within 1e-12 relative; a following assemble() and
    solve are unaffected."""
    name = os.path.basename(path)[:-4]
    g = load_golden(name)
    prob = golden_problem(name)
    n = int(g["free"])
    import scipy.sparse as sp
    M = sp.csc_matrix((g["mass_val"], g["mass_idx"], g["mass_ptr"]), shape=(n, n)).tocsr()
    M.sort_indices()
    A = _assembler(prob)
    A.assemble()
    _, _, v0 = A.csr()
    m = A.mass_csr()
    assert np.abs(m - M.data).max() <= REL * np.abs(M.data).max()
    A.assemble()
    _, _, v1 = A.csr()
    assert np.array_equal(v0, v1)
    A.close()


def test_mass_matrix_matches_oracle_at_size():
    """The device mass matrix of a displaced 3D degree-3 patch (16^3) and a glued 3x3x3 cube grid
    against the oracle's element loop."""
    from oracle import oracle as O
    for prob in (P.volume_poisson(16, 3, seed=2), P.cube_grid(n=3, n_elem=3, p=2, seed=5, kappa_modes=8)):
        o = O.OracleProblem(prob)
        o.assemble()
        A = _assembler(prob)
        m = A.mass_csr()
        mo = o.mass()
        assert np.abs(m - mo).max() <= REL * np.abs(mo).max()
        A.close()


@pytest.mark.parametrize("case", ["square_p2_64", "disp2d_p4_40x33", "volume_p3_12", "disp3d_p232_5x6x7"])
def test_warp_basis_tables_are_bitwise_neutral(case, monkeypatch):
    """The warp-cooperative basis kernel (a lane group per abscissa, shuffles between the lanes of
    the Cox-de Boor triangle) gives the FP64 operator and rhs of the one-lane-per-abscissa kernel
    (GSGPU_BASIS_LANE=1) bit for bit: degrees 2 to 4, 2D and 3D, mixed degrees per direction."""
    make = {"square_p2_64": lambda: P.square_poisson(64, 2),
            "disp2d_p4_40x33": lambda: P.displaced_single_patch(2, (40, 33), (4, 4), 9, 0.05, ufreq=3),
            "volume_p3_12": lambda: P.volume_poisson(12, 3, seed=4),
            "disp3d_p232_5x6x7": lambda: P.displaced_single_patch(3, (5, 6, 7), (2, 3, 2), 8, 0.04)}[case]
    prob = make()
    out = []
    for lane in (False, True):
        if lane:
            monkeypatch.setenv("GSGPU_BASIS_LANE", "1")
        else:
            monkeypatch.delenv("GSGPU_BASIS_LANE", raising=False)
        A = _assembler(prob)
        A.assemble("fp64")
        out.append((A.csr()[2], A.rhs()))
        A.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("case", ["disp2d_quad_1.5_2", "disp3d_quad_2_0", "cubegrid_quad_1_2"])
def test_error_norms_use_the_reference_rule(case):
    """gsField::distanceL2 / distanceH1 integrate with p + 1 Gauss points per direction whatever the
    assembler's quA, quB: with a non-default assembly rule the device norms take their own grid and
    match the oracle's restatement of the reference's rule (reference_norms, pinned against the
    reference itself) to 1e-9, not the assembly-rule norms."""
    from oracle import oracle as O
    if case == "disp2d_quad_1.5_2":
        prob = P.displaced_single_patch(2, (9, 7), (3, 4), 31, 0.05, ufreq=2)
        prob.quA, prob.quB = 1.5, 2
    elif case == "disp3d_quad_2_0":
        prob = P.displaced_single_patch(3, (5, 4, 6), (2, 2, 3), 33, 0.04)
        prob.quA, prob.quB = 2.0, 0
    else:
        prob = P.cube_grid(n=2, n_elem=4, p=2, seed=35, kappa_modes=8)
        prob.quA, prob.quB = 1.0, 2
    A = _assembler(prob)
    A.assemble("fp64")
    x, info = A.solve(tol=1e-12, max_iters=5000)
    assert info["converged"]
    o = O.OracleProblem(prob)
    o.assemble()
    l2r, h1r = o.reference_norms(x)
    assert abs(A.l2_error() - l2r) <= 1e-9 * l2r, (A.l2_error(), l2r, o.l2_error(x))
    assert abs(A.h1_error() - h1r) <= 1e-9 * h1r, (A.h1_error(), h1r, o.h1_error(x))
    # the assembly-rule norms differ (so the test checks the rule, not a coincidence)
    assert abs(o.l2_error(x) - l2r) > 1e-9 * l2r
    A.close()
