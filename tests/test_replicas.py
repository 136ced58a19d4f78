"""The N > 1 path of the benchmark on CPU: two gloo ranks, each with its own replica problem
(different seed, same size), and the only cross-rank step, the timing reduction (slowest rank's
time, units of all ranks). No GPU: the replicas' host plans come from host-only contexts."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    import ctypes as C
    import numpy as np
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    from gismo_gb300 import _lib
    from gismo_gb300 import problems as P
    from gismo_gb300 import replicas as R
    from gismo_gb300.assembler import PackedProblem
    prob = P.volume_poisson(6, 3, seed=R.replica_seed(1, rank))
    L = _lib.lib()
    h = C.c_void_p()
    assert L.gsgpu_create(C.byref(h), -1) == _lib.OK
    pk = PackedProblem(prob)
    assert L.gsgpu_set_problem(h, C.byref(pk.struct)) == _lib.OK
    assert L.gsgpu_refresh(h) == _lib.OK
    nf, nnz, nb, nl = C.c_int(), C.c_longlong(), C.c_int(), C.c_int()
    L.gsgpu_sizes(h, C.byref(nf), C.byref(nnz), C.byref(nb), C.byref(nl))
    L.gsgpu_destroy(h)
    t_ms = 10.0 + 5.0 * rank  # this rank's measured time
    tmax, units = R.reduce_max_sum(dist, t_ms, nf.value, "cpu")
    out.put((rank, nf.value, float(np.abs(prob.patches[0].coefs).sum()), tmax, units))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_replicas():
    import torch.multiprocessing as mp
    import __graft_entry__ as g
    g.build()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, n0, c0, t0, u0), (r1, n1, c1, t1, u1) = res
    assert n0 == n1 > 0                # same workload size on every rank (weak scaling)
    assert c0 != c1                    # independent replicas: different control points
    assert t0 == t1 == 15.0            # slowest rank's time on every rank
    assert u0 == u1 == n0 + n1         # units of all ranks


def test_single_process_reduction_is_local():
    from gismo_gb300 import replicas as R
    assert R.reduce_max_sum(None, 12.5, 7) == (12.5, 7.0)
    assert R.replica_seed(3, 0) == 3 and R.replica_seed(3, 2) != R.replica_seed(3, 1)
