"""The allocation-free CG entry point (gsgpu_cg_jacobi_noalloc) against the existing solver.

Some callers cannot call cudaMalloc: a process whose device memory already belongs to a pool
allocator sized to the GPU, or a latency-bound loop that cannot afford an allocation's implicit
device synchronisation. This entry point runs the same Jacobi-preconditioned CG as gsgpu_solve
with its working vectors in a fixed device array inside the library; each call synchronises its
stream, so it is not meant for use during a stream capture. The test drives it through the C ABI
on device arrays the test owns, compares two calls in a row on different systems with the
solutions of gsgpu_solve, and checks that repeated calls leave the device's free memory unchanged.
This file is collected last so that a failing run has already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-8  # relative 2-norm agreement of solutions, as in the other GPU solver tests


class _DeviceSystem:
    """A CSR system, its rhs and an output vector in device memory owned by the test."""

    def __init__(self, A):
        import torch
        dev = torch.device("cuda", 0)
        ptr, col, val = A.csr()
        b = A.rhs()
        self.n = len(b)
        self.ptr = torch.from_numpy(ptr).to(dev)
        self.col = torch.from_numpy(col).to(dev)
        self.val = torch.from_numpy(val).to(dev)
        self.b = torch.from_numpy(b).to(dev)
        self.x = torch.empty(self.n, dtype=torch.float64, device=dev)

    def solve(self, lib, tol):
        import torch
        self.x.fill_(float("nan"))
        stream = torch.cuda.current_stream(self.x.device)
        torch.cuda.synchronize(self.x.device)
        it, rr = C.c_int(), C.c_double()
        rc = lib.gsgpu_cg_jacobi_noalloc(self.n, self.ptr.data_ptr(), self.col.data_ptr(), self.val.data_ptr(),
                                         self.b.data_ptr(), self.x.data_ptr(), tol, 1000,
                                         C.c_void_p(stream.cuda_stream), C.byref(it), C.byref(rr))
        torch.cuda.synchronize(self.x.device)
        return rc, it.value, rr.value


def test_noalloc_cg_matches_solver_twice():
    import torch
    import __graft_entry__ as g
    g.build()
    from gismo_gb300 import _lib, problems as P
    from gismo_gb300.assembler import GpuPoissonAssembler
    lib = _lib.lib()
    systems = []
    for prob in (P.square_poisson(64, 2), P.volume_poisson(16, 3, seed=2)):
        A = GpuPoissonAssembler(prob, device=0)
        A.assemble()
        x_ref, info = A.solve(tol=1e-10)
        systems.append((_DeviceSystem(A), x_ref, info["iterations"]))
        A.close()
    # two calls in a row, different systems: the shared array is reused
    for S, x_ref, its in systems:
        rc, it, rr = S.solve(lib, 1e-10)
        assert rc == _lib.OK
        x = S.x.cpu().numpy()
        assert np.all(np.isfinite(x))
        assert abs(it - its) <= 1
        assert np.linalg.norm(x - x_ref) <= TOL * np.linalg.norm(x_ref)
    # after those warm-up calls (every kernel variant loaded), further calls allocate nothing
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    for S, x_ref, _ in reversed(systems):
        rc, _, _ = S.solve(lib, 1e-10)
        assert rc == _lib.OK
        assert np.linalg.norm(S.x.cpu().numpy() - x_ref) <= TOL * np.linalg.norm(x_ref)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0, (free0, free1)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from gismo_gb300 import _lib
    lib = _lib.lib()
    it, rr = C.c_int(), C.c_double()
    # n above the 204,276-unknown maximum is refused before any pointer is touched
    dummy = C.c_void_p(16)
    rc = lib.gsgpu_cg_jacobi_noalloc(204277, dummy, dummy, dummy, dummy, dummy, 1e-10, 10, None, C.byref(it),
                                     C.byref(rr))
    assert rc == _lib.ERR_INVALID


def test_noalloc_rejects_a_zero_diagonal_before_iterating():
    """A row whose diagonal is zero is refused right after the diagonal search."""
    import torch
    from gismo_gb300 import _lib
    lib = _lib.lib()
    dev = torch.device("cuda", 0)
    # 3 x 3: rows 0 and 2 have diagonals, row 1 an explicit zero one
    ptr = torch.tensor([0, 2, 4, 6], dtype=torch.int32, device=dev)
    col = torch.tensor([0, 1, 1, 2, 1, 2], dtype=torch.int32, device=dev)
    val = torch.tensor([2.0, -1.0, 0.0, -1.0, -1.0, 2.0], dtype=torch.float64, device=dev)
    b = torch.ones(3, dtype=torch.float64, device=dev)
    x = torch.zeros(3, dtype=torch.float64, device=dev)
    torch.cuda.synchronize(dev)
    it, rr = C.c_int(), C.c_double()
    rc = lib.gsgpu_cg_jacobi_noalloc(3, ptr.data_ptr(), col.data_ptr(), val.data_ptr(), b.data_ptr(), x.data_ptr(),
                                     1e-10, 1000, C.c_void_p(torch.cuda.current_stream(dev).cuda_stream),
                                     C.byref(it), C.byref(rr))
    torch.cuda.synchronize(dev)
    assert rc == _lib.ERR_INVALID and it.value == 0
