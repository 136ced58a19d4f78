"""Host plan of a batch of independent problems (no GPU): the batch's dof map and sparsity pattern
are the per-problem ones (gsDofMapper per problem, as the reference would run them one by one)
stacked block-diagonally, and the problems' free rows are contiguous in problem order."""
import ctypes as C

import numpy as np
import pytest

from gismo_gb300 import _lib
from gismo_gb300 import problems as P
from gismo_gb300.assembler import PackedProblem


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g
    g.build()
    return _lib.lib()


def _host_batch(lib, probs):
    h = C.c_void_p()
    assert lib.gsgpu_create(C.byref(h), -1) == _lib.OK
    packed = [PackedProblem(p) for p in probs]
    arr = (_lib.Problem * len(packed))(*[pp.struct for pp in packed])
    assert lib.gsgpu_set_batch(h, len(packed), C.cast(arr, C.c_void_p)) == _lib.OK, lib.gsgpu_last_error(h)
    assert lib.gsgpu_refresh(h) == _lib.OK, lib.gsgpu_last_error(h)
    return h, (packed, arr)


def test_batch_plan_is_block_diagonal(lib):
    from oracle import oracle as O
    probs = P.patch_batch(count=7, seed=11, nmin=4, nmax=12)
    h, keep = _host_batch(lib, probs)
    try:
        nf, nnz, nb, nl = C.c_int(), C.c_longlong(), C.c_int(), C.c_int()
        assert lib.gsgpu_sizes(h, C.byref(nf), C.byref(nnz), C.byref(nb), C.byref(nl)) == _lib.OK
        off = np.zeros(len(probs) + 1, np.int32)
        assert lib.gsgpu_batch_info(h, off.ctypes.data, None, None) == _lib.OK
        dm = np.empty(nl.value, np.int32)
        assert lib.gsgpu_dof_map(h, dm.ctypes.data) == _lib.OK
        ptr = np.empty(nf.value + 1, np.int32)
        col = np.empty(nnz.value, np.int32)
        assert lib.gsgpu_matrix_csr(h, ptr.ctypes.data, col.ctypes.data, None) == _lib.OK
        free_off, bnd_off, loc_off = 0, 0, 0
        for j, pr in enumerate(probs):
            o = O.OracleProblem(pr)
            f, z, b, loc = o.sizes()
            assert off[j] == free_off and off[j + 1] == free_off + f
            odm = o.dofmap()
            mine = dm[loc_off:loc_off + loc]
            expect = np.where(odm < f, odm + free_off, odm - f + nf.value + bnd_off)
            assert np.array_equal(mine, expect)
            o.assemble()
            optr, ocol, _ = o.csr()
            assert np.array_equal(ptr[free_off:free_off + f + 1] - ptr[free_off], optr)
            assert np.array_equal(col[ptr[free_off]:ptr[free_off + f]], ocol + free_off)
            free_off += f
            bnd_off += b
            loc_off += loc
        assert free_off == nf.value and bnd_off == nb.value
    finally:
        lib.gsgpu_destroy(h)


def test_batch_rejects_coupled_problems(lib):
    h = C.c_void_p()
    assert lib.gsgpu_create(C.byref(h), -1) == _lib.OK
    try:
        grid = P.cube_grid(n=2, n_elem=2, p=2, check=False)
        pk = PackedProblem(grid)
        arr = (_lib.Problem * 1)(pk.struct)
        assert lib.gsgpu_set_batch(h, 1, C.cast(arr, C.c_void_p)) == _lib.ERR_INVALID
        assert b"single patch" in lib.gsgpu_last_error(h)
    finally:
        lib.gsgpu_destroy(h)
