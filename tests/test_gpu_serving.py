"""Request server with continuous batching on the GPU (gsgpu_server_*).

Bars: every request's result is the same alone (one request per batch, one slot) and in the mix
(requests arriving while others run, batched and overlapped on several slots): bitwise, since each
problem of a batch keeps its own CG scalars, stopping test and row arithmetic; each result solves its
system to the requested tolerance in FP64 (checked against the CPU oracle's matrix); requests too
large for the memory budget fail with GSGPU_ERR_BUDGET and do not block the others."""
import time

import numpy as np
import pytest

from gismo_gb300 import problems as P

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as g
    g.build()


@pytest.fixture(scope="module")
def stream():
    return P.serving_requests(18, rate=400.0, seed=5, n2d=(8, 40), n3d=(4, 10))


def _serve(reqs, slots, max_batch, budget_gb=8.0, paced=True):
    from gismo_gb300.assembler import GpuPoissonServer
    S = GpuPoissonServer(device=0, slots=slots, budget_gb=budget_gb, max_batch=max_batch)
    t0 = time.perf_counter()
    ids = []
    for t, prob in reqs:
        if paced:
            dt = t - (time.perf_counter() - t0)
            if dt > 0:
                time.sleep(dt)
        ids.append(S.submit(prob, tol=1e-9))
    out = [S.result(i) for i in ids]
    S.close()
    return out


def test_results_alone_equal_results_in_the_mix(stream):
    from oracle import oracle as O
    mix = _serve(stream, slots=3, max_batch=8)
    alone = _serve(stream, slots=1, max_batch=1, paced=False)
    assert max(info["batch_size"] for _, info in mix) > 1  # the mix really batched requests
    assert all(info["batch_size"] == 1 for _, info in alone)
    for j, ((xm, im), (xa, ia)) in enumerate(zip(mix, alone)):
        assert im["status"] == 0 and ia["status"] == 0, (j, im, ia)
        assert np.array_equal(xm, xa), j
        assert im["iterations"] == ia["iterations"] and im["relres"] == ia["relres"]
        assert im["t_submit"] <= im["t_start"] <= im["t_done"]
    # each result solves the oracle's FP64 system to the requested tolerance
    for j in (0, 3, 7, 11):
        _, prob = stream[j]
        o = O.OracleProblem(prob)
        o.assemble()
        ptr, col, val = o.csr()
        import scipy.sparse as sp
        K = sp.csr_matrix((val, col, ptr))
        b = o.rhs()
        x = mix[j][0]
        assert np.linalg.norm(b - K @ x) <= 1.01e-9 * np.linalg.norm(b), j


def test_budget_rejects_only_oversized_requests():
    from gismo_gb300.assembler import GpuPoissonServer
    small = P.displaced_single_patch(2, (8, 8), (2, 2), 3, 0.05)
    big = P.displaced_single_patch(3, (24, 24, 24), (4, 4, 4), 4, 0.04)
    S = GpuPoissonServer(device=0, slots=2, budget_gb=0.05, max_batch=4)
    ib = S.submit(big)
    i1 = S.submit(small)
    i2 = S.submit(small)
    _, infb = S.result(ib)
    x1, inf1 = S.result(i1)
    x2, inf2 = S.result(i2)
    S.close()
    from gismo_gb300._lib import ERR_BUDGET
    assert infb["status"] == ERR_BUDGET and infb["est_bytes"] > 0.05e9
    assert inf1["status"] == 0 and inf2["status"] == 0
    assert np.array_equal(x1, x2)
