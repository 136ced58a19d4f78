"""The autotuner on the GPU (gsgpu_autotune): it times every variant of the stiffness stages and of
the inner product on the problem, records the fastest in the tuning table and applies it. Every
variant forms the same sums in the same order, so the tuned context's mixed solution has the same
bits as the default variants'."""
import os

import numpy as np
import pytest

from gismo_gb300 import problems as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g
    g.build()


@pytest.fixture()
def table():
    from gismo_gb300 import _lib
    from gismo_gb300.assembler import tune_clear, tune_load
    tune_clear()
    yield
    tune_clear()
    if os.path.exists(_lib.TUNING_PATH):
        tune_load(_lib.TUNING_PATH)


@pytest.mark.parametrize("case", ["volume_p3_20", "volume_p2_24", "square_p4_96"])
def test_autotune_chooses_bitwise_neutral_variants(case, table):
    from gismo_gb300.assembler import GpuPoissonAssembler
    prob = {"volume_p3_20": lambda: P.volume_poisson(20, 3, seed=5),
            "volume_p2_24": lambda: P.volume_poisson(24, 2, seed=6),
            "square_p4_96": lambda: P.displaced_single_patch(2, (96, 90), (4, 4), 7, 0.05)}[case]()
    A = GpuPoissonAssembler(prob)
    A.assemble("mixed")
    x0, i0 = A.solve(tol=1e-11, precision="mixed", max_iters=20000)
    v0 = A.tuned_variants()
    A.close()
    A = GpuPoissonAssembler(prob)
    ms = A.autotune()
    v = A.tuned_variants()
    if prob.dim == 3:
        assert np.all(ms[[1, 2, 3, 4]] > 0)                 # the row variants always run
        assert (ms[0] > 0) == (prob.patches[0].degree[0] in (2, 3))  # tiles only for degrees 2, 3
    else:
        assert np.all(ms[:6] == -1)                         # nothing to tune in the 2D stiffness
    assert v[2] in (0, 1, 2) and ms[6] > 0 and ms[8] > 0
    x1, i1 = A.solve(tol=1e-11, precision="mixed", max_iters=20000)
    assert i1["iterations"] == i0["iterations"]
    assert np.array_equal(x1, x0), (v0, v)
    A.close()
    # a later context of the same shape takes the recorded variants
    B = GpuPoissonAssembler(prob)
    assert B.tuned_variants() == v
    B.close()
