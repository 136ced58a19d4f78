"""The benchmark's configurations at their full sizes, against the reference and the oracle.

* The headline shape (3D, degree 3, 64^3 elements, 274,625 free dofs) with kappa = 1 on the unit
  cube, and the headline configuration itself (displaced map, 16-mode kappa field), against the
  reference's own gsPoissonAssembler / gsCDRAssembler + gsConjugateGradient(gsJacobiOp) run on the
  same inputs (fixtures `large_*.npz` from tests/golden/make_golden.py: the reference's sizes, CG
  iteration count, L2 and H1 errors, and every 97th entry of its solution, rhs and diagonal). Bars:
  iterations within one, L2 and H1 errors to 3 significant digits (5e-4 relative), rhs and diagonal
  samples within 1e-12 relative, solution samples within 1e-8 relative; the mixed-precision form to
  the same L2 digits and solution bar.
* The same configuration at 32^3 entry-wise against the oracle (bit-exact pattern, values within
  1e-12), with the reference's scalars at that size.
* A batch spanning the batch configuration's whole range (degrees 2-4, 8 to 128 elements per
  direction) problem by problem against the oracle.
* The multigrid configuration's full 8 x 8 x 8 patch layout (512 glued patches, 4^3 elements each,
  3 levels) against the oracle: dof map, pattern, values, and the MG-CG iteration count."""
import numpy as np
import pytest

from gismo_gb300 import problems as P
from tests.golden_cases import load_golden

pytestmark = pytest.mark.gpu

REL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g
    g.build()


def _assembler(prob):
    from gismo_gb300.assembler import GpuPoissonAssembler
    return GpuPoissonAssembler(prob, device=0)


def _spec_problem(name, g):
    """The fixture's problem, rebuilt by the generator and checked against the digest of the spec
    text the reference ran on."""
    import hashlib
    import os
    import tempfile
    from tests.golden_cases import golden_module
    prob = golden_module().large_cases()[name]
    with tempfile.TemporaryDirectory() as td:
        f = os.path.join(td, "spec.txt")
        P.write_spec(prob, f)
        with open(f) as fh:
            digest = hashlib.sha256(fh.read().encode()).hexdigest()
    assert digest == str(g["spec_sha256"]), name
    return prob


def _check_against_reference(A, g, precision):
    k = int(g["sample"])
    nf, nnz, _, _ = A.sizes()
    assert (nf, nnz) == (int(g["free"]), int(g["nnz"]))
    rhs = A.rhs()
    rs = g["rhs_sample"]
    assert np.abs(rhs[::k] - rs).max() <= REL * np.abs(rs).max()
    assert abs(np.linalg.norm(rhs) - float(g["rhs_norm"])) <= REL * float(g["rhs_norm"])
    x, info = A.solve(tol=1e-10, max_iters=2000, precision=precision)
    assert info["converged"], info
    if precision == "fp64":
        assert abs(info["iterations"] - int(g["iters"])) <= 1, (info, int(g["iters"]))
    xs = g["x_sample"]
    assert np.linalg.norm(x[::k] - xs) <= 1e-8 * np.linalg.norm(xs)
    for got, ref in ((A.l2_error(), float(g["l2"])), (A.h1_error(), float(g["h1"]))):
        assert abs(got - ref) <= 5e-4 * ref, (precision, got, ref)
    return x, info


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["large_cube_p3_n64", "large_vol_p3_n64_s1"])
def test_headline_size_matches_reference(name, precision):
    g = load_golden(name)
    prob = _spec_problem(name, g)
    A = _assembler(prob)
    A.assemble(precision)
    if precision == "fp64":
        d = A.diagonal()
        ds = g["diag_sample"]
        assert np.abs(d[::int(g["sample"])] - ds).max() <= REL * np.abs(ds).max()
    _check_against_reference(A, g, precision)
    A.close()


def test_headline_config_32_matches_oracle_entrywise():
    from oracle import oracle as O
    from tests.test_gpu_parity import _check_values
    g = load_golden("large_vol_p3_n32_s1")
    prob = _spec_problem("large_vol_p3_n32_s1", g)
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
    _check_against_reference(A, g, "fp64")
    A.assemble("mixed")
    _check_against_reference(A, g, "mixed")
    A.close()


def _full_range_batch():
    """20 draws of the batch generator (degree 2-4, 8-128 elements per direction, log-uniform) plus
    the corners of its range."""
    probs = P.patch_batch(count=20, seed=7, nmin=8, nmax=128)
    for j, (ne, p) in enumerate([((128, 128), 4), ((8, 8), 2), ((128, 8), 3), ((8, 128), 4), ((128, 128), 2)]):
        probs.append(P.displaced_single_patch(2, ne, (p, p), 9000 + j, 0.05, kappa_modes=16, ufreq=1 + j % 4))
    return probs


def test_batch_full_range_matches_oracle():
    from gismo_gb300.assembler import GpuPoissonBatch
    from oracle import oracle as O
    batch = _full_range_batch()
    assert max(max(pr.patches[0].nelems_dir) for pr in batch) == 128
    assert {pr.patches[0].degree[0] for pr in batch} == {2, 3, 4}
    B = GpuPoissonBatch(batch, device=0)
    B.assemble("fp64")
    ptr, col, val = B.csr()
    rhs = B.rhs()
    off = B.offsets()
    xs, info = B.solve(tol=1e-9, max_iters=20000)
    assert info["converged"], info
    its = info["per_problem"]["iterations"]
    for j, pr in enumerate(batch):
        o = O.OracleProblem(pr)
        # one thread: the oracle's scatter order, and so the last digits of its matrix and its CG
        # iteration count, do not depend on the host's thread count and scheduling (on 16 threads
        # a 172-iteration problem took 172-174 iterations from run to run)
        o.assemble(1)
        optr, ocol, oval = o.csr()
        a, b = off[j], off[j + 1]
        k0, k1 = ptr[a], ptr[b]
        assert np.array_equal(ptr[a:b + 1] - k0, optr) and np.array_equal(col[k0:k1] - a, ocol), j
        rowmax = np.maximum.reduceat(np.abs(oval), optr[:-1])
        floor = np.repeat(rowmax, np.diff(optr)) * 1e-14
        assert np.all(np.abs(val[k0:k1] - oval) <= REL * np.abs(oval) + floor), j
        orhs = o.rhs()
        assert np.abs(rhs[a:b] - orhs).max() <= REL * np.abs(orhs).max(), j
        xo, it, _, _ = o.solve_cg(1e-9, 20000)
        assert abs(int(its[j]) - it) <= 1, (j, its[j], it)
        assert np.linalg.norm(xs[j] - xo) <= 1e-7 * np.linalg.norm(xo), j
    # the mixed form of the same batch reaches the FP64 solutions
    x64, _ = B.solve(tol=1e-13, max_iters=40000)
    B.assemble("mixed")
    xm, im = B.solve(tol=1e-10, max_iters=40000, precision="mixed")
    assert im["converged"], im
    for j in range(len(batch)):
        assert np.linalg.norm(xm[j] - x64[j]) <= 1e-8 * np.linalg.norm(x64[j]), j
    B.close()


def test_cube_grid_8x8x8_layout_matches_oracle():
    from oracle import oracle as O
    from tests.test_gpu_parity import _check_values
    prob = P.cube_grid(n=8, n_elem=4, p=2, seed=3, kappa_modes=32)
    assert len(prob.patches) == 512
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
    levels, damping = 3, 0.5
    xo, it, _, _ = o.solve_mg(1e-8, 500, levels, 2, 2, damping)
    x, info = A.solve(tol=1e-8, max_iters=500, method="mg", mg_levels=levels, mg_damping=damping)
    assert info["converged"], info
    assert abs(info["iterations"] - it) <= 1, (info, it)
    assert np.linalg.norm(x - xo) <= 1e-6 * np.linalg.norm(xo)
    A.assemble("mixed")
    xm, im = A.solve(tol=1e-9, max_iters=500, method="mg", precision="mixed", mg_levels=levels, mg_damping=damping)
    assert im["converged"], im
    assert abs(im["iterations"] - it) <= 2, (im, it)
    A.close()
