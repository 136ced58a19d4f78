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


def _shape_stream(seed, count, shapes):
    """Requests cycling over a few discretisations (same knots, degree and sides), each with its own
    geometry displacement and kappa field: what a client solving on fixed meshes sends."""
    out = []
    for j in range(count):
        dim, ne, p = shapes[j % len(shapes)]
        out.append(P.displaced_single_patch(dim, (ne,) * dim, (p,) * dim, seed + 17 * j, 0.04, check=False))
    return out


def test_resident_batches_give_the_same_results():
    """A slot keeps the contexts of its recent batches resident: a later batch of the same structure
    skips refresh() (resident = 1, only control points and field constants uploaded) and gives the
    same bits as the same request on a server that keeps nothing resident."""
    from gismo_gb300.assembler import GpuPoissonServer
    reqs = _shape_stream(40, 8, [(2, 24, 3), (3, 8, 2)])
    res = {}
    for keep in (True, False):
        S = GpuPoissonServer(device=0, slots=1, budget_gb=4.0, max_batch=1)
        if not keep:
            S.set_resident(0.0)
        res[keep] = [S.result(S.submit(pr, tol=1e-9)) for pr in reqs]  # one at a time, in order
        S.close()
    flags = [info["resident"] for _, info in res[True]]
    assert flags[:2] == [0, 0] and all(f == 1 for f in flags[2:]), flags
    assert all(info["resident"] == 0 for _, info in res[False])
    for (xa, ia), (xb, ib) in zip(res[True], res[False]):
        assert ia["status"] == 0 and ib["status"] == 0
        assert np.array_equal(xa, xb)
        assert ia["iterations"] == ib["iterations"]
    # the set-up of a resident batch is an upload, not a refresh
    setup_res = np.median([info["ms_setup"] for _, info in res[True][2:]])
    setup_new = np.median([info["ms_setup"] for _, info in res[False][2:]])
    assert setup_res < setup_new, (setup_res, setup_new)


def test_resident_contexts_yield_to_the_budget():
    """Resident contexts count against the budget: a request that only fits once they are released
    still runs (nothing waits for ever), on one slot and on two (the slot that needs the memory asks
    the other to release its resident contexts)."""
    from gismo_gb300.assembler import GpuPoissonServer
    big = P.displaced_single_patch(3, (16, 16, 16), (3, 3, 3), 61, 0.04, check=False)
    S = GpuPoissonServer(device=0, slots=1, budget_gb=4.0, max_batch=1)
    _, ib = S.result(S.submit(big, tol=1e-8))
    S.close()
    eb = ib["est_bytes"]
    # three medium requests of distinct structure, about 0.4 of the big one each: resident together
    # they leave no room for the big request in a budget of 1.5 big requests
    medium = [P.displaced_single_patch(3, ne, (3, 3, 3), 62 + j, 0.04, check=False)
              for j, ne in enumerate([(12, 12, 12), (12, 12, 11), (11, 12, 12)])]
    for slots in (1, 2):
        S = GpuPoissonServer(device=0, slots=slots, budget_gb=1.5 * eb / 1e9, max_batch=1)
        S.set_resident(1.5 * eb / 1e9)
        for pr in medium:
            _, info = S.result(S.submit(pr, tol=1e-8))
            assert info["status"] == 0
            assert info["est_bytes"] < 0.5 * eb
        xb, inf = S.result(S.submit(big, tol=1e-8))
        assert inf["status"] == 0
        # and the medium ones still run afterwards
        _, info = S.result(S.submit(medium[0], tol=1e-8))
        assert info["status"] == 0
        S.close()
