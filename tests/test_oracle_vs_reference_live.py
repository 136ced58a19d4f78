"""The oracle against the reference run live (CPU; needs the G+Smo source tree, skipped where it
is absent) on input combinations beyond the committed fixtures: Neumann sides with a non-default
quadrature rule, Neumann sides together with Dirichlet values by L2 projection, and a glued cube
grid with mixed conditions solved by multigrid W-cycles. Same bars as the fixtures: dof map and
pattern bit-exact, values, rhs and eliminated values within 1e-12, iteration counts within one,
L2 and H1 errors of the reference's solution to 1e-10 (with the error norms' own quadrature rule,
p + 1 points per direction, which differs from the assembly rule when quA, quB are not 1, 1)."""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

from gismo_gb300 import problems as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MK = os.path.join(ROOT, "oracle", "ref")


def _cases():
    a = P.mixed_boundary(P.displaced_single_patch(2, (9, 7), (3, 4), 31, 0.05, ufreq=2))
    a.quA, a.quB = 1.5, 2
    b = P.mixed_boundary(P.displaced_single_patch(3, (4, 3, 5), (2, 2, 3), 33, 0.04))
    b.dirichlet_l2 = True
    c = P.mixed_boundary(P.cube_grid(n=2, n_elem=4, p=2, seed=35, kappa_modes=8))
    c.solver, c.tol, c.mg_levels, c.mg_cycles, c.mg_cgc_damping = "mg", 1e-8, 3, 2, 0.9
    return {"disp2d_neu_quad": a, "disp3d_neu_l2dir": b, "cubegrid_neu_mgw": c}


@pytest.fixture(scope="module")
def gsref():
    if shutil.which("make") is None or shutil.which("g++") is None:
        pytest.skip("no make / g++")
    ref = subprocess.run(["make", "-s", "-C", MK, "print-ref"], capture_output=True, text=True).stdout.strip()
    if not ref or not os.path.isdir(os.path.join(ref, "src", "gsAssembler")):
        pytest.skip("G+Smo source tree not available")
    r = subprocess.run(["make", "-s", "-C", MK], capture_output=True, text=True, timeout=1800)
    assert r.returncode == 0, r.stderr[-3000:]
    return os.path.join(ROOT, "oracle", "_ref", "gsref")


@pytest.mark.parametrize("name", sorted(_cases()))
def test_oracle_matches_live_reference(gsref, name):
    import importlib.util
    from oracle import oracle as O
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(ROOT, "tests", "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    prob = _cases()[name]
    with tempfile.TemporaryDirectory() as td:
        g = mg.run_reference(gsref, prob, td)
    o = O.OracleProblem(prob)
    o.assemble()
    assert np.array_equal(o.dofmap(), g["dofmap"])
    import scipy.sparse as sp
    K = sp.csc_matrix((g["csc_val"], g["csc_idx"], g["csc_ptr"])).tocsr()
    K.sort_indices()
    ptr, col, val = o.csr()
    assert np.array_equal(ptr, K.indptr) and np.array_equal(col, K.indices)
    assert np.abs(val - K.data).max() <= 1e-12 * np.abs(K.data).max()
    assert np.abs(o.rhs() - g["rhs"]).max() <= 1e-12 * np.abs(g["rhs"]).max()
    if len(g["ddof"]):
        assert np.abs(o.ddof() - g["ddof"]).max() <= 1e-12 * max(1.0, np.abs(g["ddof"]).max())
    if prob.solver == "mg":
        x, it, _, _ = o.solve_mg(prob.tol, prob.maxit, prob.mg_levels, prob.mg_npre, prob.mg_npost, prob.mg_damping,
                                 prob.mg_cycles, prob.mg_cgc_damping)
    else:
        x, it, _, _ = o.solve_cg(prob.tol, prob.maxit)
    assert abs(it - int(g["iters"])) <= 1
    # gsField::distanceL2/H1 integrate with their evaluator's default rule (p + 1 points per
    # direction), not the assembler's quA/quB
    l2, h1 = o.reference_norms(g["x"])
    assert abs(l2 - float(g["l2"])) <= 1e-10 * float(g["l2"])
    assert abs(h1 - float(g["h1"])) <= 1e-10 * float(g["h1"])
