"""Checkpoint / resume (CPU): the text spec is an exact inverse pair (every fixture's stored spec
parses back to the generator's problem, bitwise), and a saved problem + system + solution loads
back bitwise and reproduces the same host plan."""
import os

import numpy as np

from gismo_gb300 import checkpoint as K
from gismo_gb300 import problems as P
from tests.golden_cases import golden_problem, load_golden
from tests.test_oracle_golden import GOLDEN


def _same(a, b):
    assert a.dim == b.dim and len(a.patches) == len(b.patches)
    for p, q in zip(a.patches, b.patches):
        assert tuple(p.degree) == tuple(q.degree) and tuple(p.gdegree) == tuple(q.gdegree)
        assert all(np.array_equal(x, y) for x, y in zip(p.knots, q.knots))
        assert all(np.array_equal(x, y) for x, y in zip(p.gknots, q.gknots))
        assert np.array_equal(p.coefs, q.coefs)
    for f in ("interfaces", "dirichlet", "neumann"):
        assert [tuple(v) for v in getattr(a, f)] == [tuple(v) for v in getattr(b, f)], f
    for f in ("kappa_fourier", "kappa_alpha", "kappa_scale", "ufreq", "quA", "quB", "dirichlet_l2", "solver", "tol",
              "maxit", "mg_levels", "mg_npre", "mg_npost", "mg_damping", "mg_cycles", "mg_cgc_damping"):
        assert getattr(a, f) == getattr(b, f), f
    if a.kappa_fourier:
        assert np.array_equal(a.kappa_amp, b.kappa_amp) and np.array_equal(a.kappa_phase, b.kappa_phase)
        assert np.array_equal(np.asarray(a.kappa_k)[:, :3], np.asarray(b.kappa_k)[:, :3])
    else:
        assert a.kappa_const == b.kappa_const


def test_fixture_specs_parse_back():
    for path in GOLDEN:
        name = os.path.basename(path)[:-4]
        _same(P.read_spec(str(load_golden(name)["spec"])), golden_problem(name))


def test_save_and_load_state(tmp_path):
    from oracle import oracle as O
    prob = P.mixed_boundary(P.cube_grid(n=2, n_elem=3, p=2, seed=7, kappa_modes=8))
    o = O.OracleProblem(prob)
    o.assemble()
    ptr, col, val = o.csr()
    x, it, rr, _ = o.solve_cg(1e-10, 1000)
    f = str(tmp_path / "state.npz")
    K.save_state(f, prob, csr_ptr=ptr, csr_col=col, csr_val=val, rhs=o.rhs(), ddof=o.ddof(), x=x,
                 iterations=np.int64(it), relres=np.float64(rr))
    back, arr = K.load_state(f)
    _same(back, prob)
    for k, v in (("csr_ptr", ptr), ("csr_col", col), ("csr_val", val), ("rhs", o.rhs()), ("x", x)):
        assert np.array_equal(arr[k], v), k
    assert int(arr["iterations"]) == it
    # resume: the reloaded problem gives the same numbering and pattern
    o2 = O.OracleProblem(back)
    o2.assemble()
    assert np.array_equal(o2.dofmap(), o.dofmap())
    p2, c2, _ = o2.csr()
    assert np.array_equal(p2, ptr) and np.array_equal(c2, col)
    # and the stored solution solves the reloaded system to the stored residual
    import scipy.sparse as sp
    r = o2.rhs() - sp.csr_matrix((arr["csr_val"], c2, p2)) @ arr["x"]
    assert np.linalg.norm(r) <= 1.01 * float(arr["relres"]) * np.linalg.norm(o2.rhs()) + 1e-14


def test_save_assembler_contract(tmp_path):
    """save_assembler takes what an assembler exposes (prob, csr(), rhs(), fixedDofs()); an
    oracle-backed stand-in with the same methods gives a checkpoint that loads back bitwise."""
    from oracle import oracle as O

    class Stand:
        def __init__(self, prob):
            self.prob = prob
            self.o = O.OracleProblem(prob)
            self.o.assemble()

        def csr(self):
            return self.o.csr()

        def rhs(self):
            return self.o.rhs()

        def fixedDofs(self):
            return self.o.ddof()

    A = Stand(P.mixed_boundary(P.displaced_single_patch(2, (6, 5), (2, 3), 4, 0.05)))
    x, it, rr, _ = A.o.solve_cg(1e-10, 1000)
    f = str(tmp_path / "a.npz")
    K.save_assembler(f, A, x, {"iterations": it, "relres": rr})
    prob, arr = K.load_state(f)
    _same(prob, A.prob)
    assert np.array_equal(arr["x"], x) and np.array_equal(arr["ddof"], A.fixedDofs())
    assert int(arr["iterations"]) == it and float(arr["relres"]) == rr
