"""The device operators handed to a host-side solver (what a G+Smo caller passes to its own
gsConjugateGradient through gsLinearOperator adaptors): gsgpu_apply (K x) and gsgpu_mg_apply
(one V-cycle).

Bars: K x within 1e-13 relative of the host product with the exported matrix; a host PCG
preconditioned by the device V-cycle reaches the tolerance in the device MG-CG's iteration count
within one and to the same solution; the V-cycle is symmetric and positive (to the accuracy of its
coarse solve)."""
import numpy as np
import pytest

from gismo_gb300 import problems as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g
    g.build()


@pytest.fixture(scope="module")
def assembled():
    from gismo_gb300.assembler import GpuPoissonAssembler
    prob = P.cube_grid(n=3, n_elem=4, p=2, seed=5, kappa_modes=32)
    A = GpuPoissonAssembler(prob, device=0)
    A.assemble("fp64")
    yield A
    A.close()


def test_apply_matches_host_product(assembled):
    A = assembled
    K = A.matrix()
    rng = np.random.default_rng(3)
    x = rng.standard_normal(K.shape[0])
    y = A.apply(x)
    ref = K @ x
    assert np.linalg.norm(y - ref) <= 1e-13 * np.linalg.norm(ref)


def test_vcycle_preconditions_a_host_cg(assembled):
    A = assembled
    K = A.matrix()
    b = A.rhs()
    levels = 3
    xd, info = A.solve(tol=1e-8, max_iters=500, method="mg", mg_levels=levels)
    assert info["converged"]
    # gsConjugateGradient with the V-cycle as preconditioner, on the host
    x = np.zeros_like(b)
    r = b.copy()
    z = A.mg_apply(r, mg_levels=levels)
    p = z.copy()
    rz = r @ z
    bn = np.linalg.norm(b)
    its = 0
    while its < 500:
        t = A.apply(p)
        alpha = rz / (p @ t)
        x += alpha * p
        r -= alpha * t
        its += 1
        if np.linalg.norm(r) < 1e-8 * bn:
            break
        z = A.mg_apply(r, mg_levels=levels)
        rzn = r @ z
        p = z + (rzn / rz) * p
        rz = rzn
    assert abs(its - info["iterations"]) <= 1, (its, info)
    assert np.linalg.norm(b - K @ x) <= 1.01e-8 * bn
    assert np.linalg.norm(x - xd) <= 1e-6 * np.linalg.norm(xd)


def test_vcycle_is_symmetric_positive(assembled):
    A = assembled
    rng = np.random.default_rng(7)
    n = A.sizes()[0]
    r1, r2 = rng.standard_normal(n), rng.standard_normal(n)
    z1, z2 = A.mg_apply(r1, mg_levels=3), A.mg_apply(r2, mg_levels=3)
    assert abs(r2 @ z1 - r1 @ z2) <= 1e-7 * abs(r1 @ z2)
    assert r1 @ z1 > 0 and r2 @ z2 > 0


def test_wcycle_is_symmetric_positive(assembled):
    A = assembled
    rng = np.random.default_rng(9)
    n = A.sizes()[0]
    r1, r2 = rng.standard_normal(n), rng.standard_normal(n)
    kw = dict(mg_levels=3, mg_cycles=2, mg_cgc_damping=0.9)
    z1, z2 = A.mg_apply(r1, **kw), A.mg_apply(r2, **kw)
    assert abs(r2 @ z1 - r1 @ z2) <= 1e-7 * abs(r1 @ z2)
    assert r1 @ z1 > 0 and r2 @ z2 > 0
    # a W-cycle is a different operator from the V-cycle
    assert np.linalg.norm(z1 - A.mg_apply(r1, mg_levels=3)) > 1e-6 * np.linalg.norm(z1)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_fixed_dofs_from_the_caller(precision):
    """gsgpu_set_fixed_dofs: the Dirichlet lift uses the caller's eliminated-dof values (as the
    expression assembler's space setup supplies them). The rhs is affine in those values:
    rhs(2 g) = 2 rhs(g) - rhs(0); the built-in values reproduce the built-in rhs bit for bit."""
    from gismo_gb300._lib import GsGpuError
    from gismo_gb300.assembler import GpuPoissonAssembler
    prob = P.displaced_single_patch(3, (6, 7, 5), (2, 3, 2), 4, 0.04)
    A = GpuPoissonAssembler(prob, device=0)
    A.assemble(precision)
    g = A.fixedDofs()
    b1 = A.rhs()
    assert np.abs(g).max() > 0
    A.set_fixed_dofs(g)
    A.assemble(precision)
    assert np.array_equal(A.rhs(), b1) and np.array_equal(A.fixedDofs(), g)
    A.set_fixed_dofs(2 * g)
    A.assemble(precision)
    b2 = A.rhs()
    assert np.array_equal(A.fixedDofs(), 2 * g)
    A.set_fixed_dofs(np.zeros_like(g))
    A.assemble(precision)
    b0 = A.rhs()
    assert np.abs(b2 - (2 * b1 - b0)).max() <= 1e-12 * np.abs(b1).max()
    assert np.abs(b1 - b0).max() > 1e-6 * np.abs(b1).max()
    A.set_fixed_dofs(None)
    A.assemble(precision)
    assert np.array_equal(A.rhs(), b1)
    with pytest.raises(GsGpuError):
        A.set_fixed_dofs(g[:-1])
    A.close()
