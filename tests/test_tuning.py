"""The tuning table of the kernel variants (gsgpu_tune_load / gsgpu_tune_save / gsgpu_tuned_variants)
on host-only contexts: no GPU. The table decides, per (kernel group, dimension, degree, Gauss
points), which variant of the stiffness stages and of the inner product a context uses."""
import ctypes as C
import os

import numpy as np
import pytest

from gismo_gb300 import problems as P


@pytest.fixture()
def lib():
    import __graft_entry__ as g
    g.build()
    from gismo_gb300 import _lib
    L = _lib.lib()
    L.gsgpu_tune_clear()
    yield L
    # back to the committed table
    L.gsgpu_tune_clear()
    if os.path.exists(_lib.TUNING_PATH):
        assert L.gsgpu_tune_load(_lib.TUNING_PATH.encode()) == _lib.OK


def _variants(L, prob):
    from gismo_gb300 import _lib
    from gismo_gb300.assembler import PackedProblem
    h = C.c_void_p()
    assert L.gsgpu_create(C.byref(h), -1) == _lib.OK
    pk = PackedProblem(prob)
    assert L.gsgpu_set_problem(h, C.byref(pk.struct)) == _lib.OK
    assert L.gsgpu_refresh(h) == _lib.OK
    v = np.empty(3, np.int32)
    assert L.gsgpu_tuned_variants(h, v.ctypes.data) == _lib.OK
    L.gsgpu_destroy(h)
    return tuple(int(a) for a in v)


def test_defaults_without_a_table(lib):
    # degree 3: stage-1 tiles (0), stage 2 with 4 output fields (0), load-based inner product with
    # four rows per thread (2)
    assert _variants(lib, P.volume_poisson(8, 3, seed=1, check=False)) == (0, 0, 2)
    # degree 4 has no stage-1 tiles: rows with 4 output fields (1); a glued grid has no half-diagonal
    # inner operator (-1)
    assert _variants(lib, P.displaced_single_patch(3, (9, 9, 9), (4, 4, 4), 2, 0.04, check=False))[0] == 1
    assert _variants(lib, P.cube_grid(n=2, n_elem=3, p=2, seed=1, kappa_modes=4, check=False))[2] == -1


def test_table_round_trip_and_lookup(lib, tmp_path):
    from gismo_gb300 import _lib
    f = tmp_path / "t.txt"
    f.write_text("# comment\n31 3 3 4 2 1.25\n32 3 3 4 1 1.25\n1 3 3 4 1 0.061\n31 3 2 3 1 0.5\n")
    assert lib.gsgpu_tune_load(str(f).encode()) == _lib.OK
    assert _variants(lib, P.volume_poisson(8, 3, seed=1, check=False)) == (2, 1, 1)
    # other degrees keep their defaults
    assert _variants(lib, P.displaced_single_patch(3, (9, 9, 9), (4, 4, 4), 2, 0.04, check=False)) == (1, 0, 2)
    g = tmp_path / "u.txt"
    assert lib.gsgpu_tune_save(str(g).encode()) == _lib.OK
    rows = sorted(tuple(ln.split()) for ln in g.read_text().splitlines() if ln and not ln.startswith("#"))
    want = sorted(tuple(ln.split()) for ln in f.read_text().splitlines() if ln and not ln.startswith("#"))
    assert [r[:5] for r in rows] == [w[:5] for w in want]
    assert all(abs(float(r[5]) - float(w[5])) < 1e-12 for r, w in zip(rows, want))


@pytest.mark.parametrize("bad", ["31 3 3 4 7 1.0\n", "32 5 3 4 1 1.0\n", "31 3 3\n", "9 3 3 4 0 1.0\n"])
def test_invalid_tables_are_rejected(lib, tmp_path, bad):
    from gismo_gb300 import _lib
    f = tmp_path / "bad.txt"
    f.write_text(bad)
    assert lib.gsgpu_tune_load(str(f).encode()) == _lib.ERR_INVALID
    assert _variants(lib, P.volume_poisson(8, 3, seed=1, check=False)) == (0, 0, 2)  # nothing was taken
