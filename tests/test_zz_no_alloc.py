"""The allocation-free CG entry point (gsgpu_cg_jacobi_noalloc) against the existing solver.

Some callers cannot call cudaMalloc (code running while a CUDA graph is captured in global mode,
processes whose device memory belongs to a pool allocator, latency-bound loops); this entry
point runs the same Jacobi-preconditioned CG as gsgpu_solve with its working vectors in a fixed
device array inside the library. The test drives it through the C ABI on device arrays the
test owns and compares two calls in a row with the solutions of gsgpu_solve. This file is
collected last so that a failing run has already run every other test."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-8  # relative 2-norm agreement of solutions, as in the other GPU solver tests


def _solve_noalloc(lib, A, tol):
    import torch
    ptr, col, val = A.csr()
    b = A.rhs()
    dev = torch.device("cuda", 0)
    t_ptr = torch.from_numpy(ptr).to(dev)
    t_col = torch.from_numpy(col).to(dev)
    t_val = torch.from_numpy(val).to(dev)
    t_b = torch.from_numpy(b).to(dev)
    t_x = torch.full((len(b),), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    torch.cuda.synchronize(dev)
    it, rr = C.c_int(), C.c_double()
    rc = lib.gsgpu_cg_jacobi_noalloc(len(b), t_ptr.data_ptr(), t_col.data_ptr(), t_val.data_ptr(), t_b.data_ptr(),
                                     t_x.data_ptr(), tol, 1000, C.c_void_p(stream.cuda_stream), C.byref(it),
                                     C.byref(rr))
    torch.cuda.synchronize(dev)
    return rc, t_x.cpu().numpy(), it.value, rr.value


def test_noalloc_cg_matches_solver_twice():
    import __graft_entry__ as g
    g.build()
    from gismo_gb300 import _lib, problems as P
    from gismo_gb300.assembler import GpuPoissonAssembler
    lib = _lib.lib()
    cases = [P.square_poisson(64, 2), P.volume_poisson(16, 3, seed=2)]
    for prob in cases:  # two calls in a row, different systems: the shared array is reused
        A = GpuPoissonAssembler(prob, device=0)
        A.assemble()
        x_ref, info = A.solve(tol=1e-10)
        rc, x, it, rr = _solve_noalloc(lib, A, 1e-10)
        assert rc == _lib.OK
        assert np.all(np.isfinite(x))
        assert abs(it - info["iterations"]) <= 1
        assert np.linalg.norm(x - x_ref) <= TOL * np.linalg.norm(x_ref)
        A.close()


def test_noalloc_rejects_sizes_beyond_its_scratch():
    from gismo_gb300 import _lib
    lib = _lib.lib()
    it, rr = C.c_int(), C.c_double()
    # n above the 204,276-unknown maximum is refused before any pointer is touched
    dummy = C.c_void_p(16)
    rc = lib.gsgpu_cg_jacobi_noalloc(204277, dummy, dummy, dummy, dummy, dummy, 1e-10, 10, None, C.byref(it),
                                     C.byref(rr))
    assert rc == _lib.ERR_INVALID
