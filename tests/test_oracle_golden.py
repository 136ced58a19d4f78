"""The CPU oracle against the golden fixtures produced by the G+Smo reference itself
(tests/golden/make_golden.py). This pins the oracle that every GPU parity test uses."""
import glob
import os

import numpy as np
import pytest
import scipy.sparse as sp

from gismo_gb300 import problems as P
from oracle import oracle as O
from tests.golden_cases import golden_problem, load_golden

# the full fixtures (matrix, rhs, solution); the large_* fixtures hold scalars and samples only
GOLDEN = sorted(p for p in glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz"))
                if not os.path.basename(p).startswith("large_"))


def _csr_from_csc(g):
    n = int(g["free"])
    K = sp.csc_matrix((g["csc_val"], g["csc_idx"], g["csc_ptr"]), shape=(n, n)).tocsr()
    K.sort_indices()
    return K


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_matches_reference(path):
    name = os.path.basename(path)[:-4]
    g = load_golden(name)
    prob = golden_problem(name)
    o = O.OracleProblem(prob)
    o.assemble()
    # dof map and sparsity pattern: bit-exact
    assert np.array_equal(o.dofmap(), g["dofmap"])
    ptr, idx, val = o.csr()
    Kr = _csr_from_csc(g)
    assert np.array_equal(ptr, Kr.indptr) and np.array_equal(idx, Kr.indices)
    # values: 1e-12 relative, with an absolute floor for entries that cancel to ~0
    rowmax = np.maximum.reduceat(np.abs(Kr.data), Kr.indptr[:-1])
    floor = np.repeat(rowmax, np.diff(Kr.indptr)) * 1e-14
    assert np.all(np.abs(val - Kr.data) <= 1e-12 * np.abs(Kr.data) + floor)
    rhs = o.rhs()
    assert np.abs(rhs - g["rhs"]).max() <= 1e-12 * np.abs(g["rhs"]).max()
    if len(g["ddof"]):
        assert np.abs(o.ddof() - g["ddof"]).max() <= 1e-12 * max(1.0, np.abs(g["ddof"]).max())
    if prob.solver == "mg":
        x, it, rr, _ = o.solve_mg(prob.tol, prob.maxit, prob.mg_levels, prob.mg_npre, prob.mg_npost, prob.mg_damping,
                                  prob.mg_cycles, prob.mg_cgc_damping)
    else:
        x, it, rr, _ = o.solve_cg(prob.tol, prob.maxit)
    # the element-loop scatter order varies between OpenMP runs (as in the reference), which moves
    # the stopping iteration by at most one at the tolerance boundary
    assert abs(it - int(g["iters"])) <= 1
    assert np.linalg.norm(x - g["x"]) <= 1e-9 * np.linalg.norm(g["x"])
    l2 = o.l2_error(x)
    assert abs(l2 - float(g["l2"])) <= 1e-6 * abs(float(g["l2"]))  # >= 3 significant digits
    # gsField::distanceH1 of the reference's own solution
    h1 = o.h1_error(g["x"])
    assert abs(h1 - float(g["h1"])) <= 1e-10 * float(g["h1"])


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_oracle_mass_matches_reference(path):
    """gsGenericAssembler::assembleMass with the fixture's boundary conditions: the reference's mass
    matrix has the stiffness matrix's pattern, and the oracle's restatement matches its values to
    1e-12 relative."""
    name = os.path.basename(path)[:-4]
    g = load_golden(name)
    assert "mass_val" in g, name
    n = int(g["free"])
    M = sp.csc_matrix((g["mass_val"], g["mass_idx"], g["mass_ptr"]), shape=(n, n)).tocsr()
    M.sort_indices()
    K = _csr_from_csc(g)
    assert np.array_equal(M.indptr, K.indptr) and np.array_equal(M.indices, K.indices)
    o = O.OracleProblem(golden_problem(name))
    o.assemble()
    m = o.mass()
    assert np.abs(m - M.data).max() <= 1e-12 * np.abs(M.data).max()
    assert np.all(M.diagonal() > 0)


def test_generator_reproduces_fixture_specs():
    """The seeded generator must still produce exactly the inputs the fixtures were made from."""
    import tempfile
    for path in GOLDEN:
        name = os.path.basename(path)[:-4]
        g = load_golden(name)
        with tempfile.NamedTemporaryFile("r", suffix=".txt") as fh:
            P.write_spec(golden_problem(name), fh.name)
            assert open(fh.name).read() == str(g["spec"]), name


def test_gauss_rule_exactness():
    """Gauss-Legendre with n nodes integrates x^k exactly for k <= 2n-1
    (the check of the reference's gsQuadratureRules_test)."""
    for n in range(1, 9):
        x, w = O.gauss(n)
        assert np.all(np.diff(x) > 0)
        for k in range(2 * n):
            exact = (1 - (-1) ** (k + 1)) / (k + 1)
            assert abs(np.dot(w, x ** k) - exact) < 1e-13
