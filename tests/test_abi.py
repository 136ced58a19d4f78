"""The C-ABI library (CPU checks): it loads, exports every entry point include/gsgpu.h declares,
and its host-side plan (gsDofMapper numbering, sparsity pattern) matches the reference fixtures.
No numerical call is made here: host-only contexts refuse them."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from gismo_gb300 import _lib
from gismo_gb300.assembler import PackedProblem
from tests.golden_cases import golden_problem, load_golden
from tests.test_oracle_golden import GOLDEN, _csr_from_csc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    txt = open(os.path.join(ROOT, "include", "gsgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(gsgpu_[a-z0-9_]+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g
    g.build()
    return _lib.lib()


def test_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(lib, s), s
    assert sorted(_lib.EXPORTS) == syms


def _host_ctx(lib, prob):
    h = C.c_void_p()
    assert lib.gsgpu_create(C.byref(h), -1) == _lib.OK
    pk = PackedProblem(prob)
    assert lib.gsgpu_set_problem(h, C.byref(pk.struct)) == _lib.OK
    assert lib.gsgpu_refresh(h) == _lib.OK
    return h, pk


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_host_plan_matches_reference(lib, path):
    name = os.path.basename(path)[:-4]
    g = load_golden(name)
    h, pk = _host_ctx(lib, golden_problem(name))
    try:
        nf, nnz, nb, nl = C.c_int(), C.c_longlong(), C.c_int(), C.c_int()
        assert lib.gsgpu_sizes(h, C.byref(nf), C.byref(nnz), C.byref(nb), C.byref(nl)) == _lib.OK
        assert nf.value == int(g["free"]) and nnz.value == int(g["nnz"])
        dm = np.empty(nl.value, np.int32)
        assert lib.gsgpu_dof_map(h, dm.ctypes.data) == _lib.OK
        assert np.array_equal(dm, g["dofmap"])
        ptr = np.empty(nf.value + 1, np.int32)
        col = np.empty(nnz.value, np.int32)
        assert lib.gsgpu_matrix_csr(h, ptr.ctypes.data, col.ctypes.data, None) == _lib.OK
        K = _csr_from_csc(g)
        assert np.array_equal(ptr, K.indptr) and np.array_equal(col, K.indices)
        # eliminated-dof values of the problem's Dirichlet strategy (interpolation or L2
        # projection), computed on the host: the reference's own values
        dd = np.empty(nb.value, np.float64)
        assert lib.gsgpu_fixed_dofs(h, dd.ctypes.data) == _lib.OK
        if nb.value:
            assert np.abs(dd - g["ddof"]).max() <= 1e-12 * max(1.0, np.abs(g["ddof"]).max()), name
        # numerical calls are refused without a device
        assert lib.gsgpu_assemble(h, 0) == _lib.ERR_STATE
    finally:
        lib.gsgpu_destroy(h)


def test_invalid_problem_is_rejected(lib):
    from gismo_gb300 import problems as P
    prob = P.square_poisson(4, 2)
    prob.dirichlet = [(0, 9)]  # no side 9 on a 2D patch
    h = C.c_void_p()
    assert lib.gsgpu_create(C.byref(h), -1) == _lib.OK
    pk = PackedProblem(prob)
    assert lib.gsgpu_set_problem(h, C.byref(pk.struct)) == _lib.ERR_INVALID
    assert b"dirichlet" in lib.gsgpu_last_error(h)
    assert lib.gsgpu_refresh(h) == _lib.ERR_STATE
    lib.gsgpu_destroy(h)


def test_dropin_headers_compile_against_reference():
    """include/gsGpuPoissonAssembler.h and include/gsGpuExprAssembler.h compile against the G+Smo
    headers as a user's driver would use them (oracle/ref/adaptor_check.cpp), and the expression
    recogniser classifies the Poisson, diffusion and source forms (and not a mass matrix) at
    compile time. Needs the G+Smo source tree; skipped where it is absent."""
    import shutil
    import subprocess
    mk = os.path.join(ROOT, "oracle", "ref")
    if shutil.which("make") is None or shutil.which("g++") is None:
        pytest.skip("no make / g++")
    ref = subprocess.run(["make", "-s", "-C", mk, "print-ref"], capture_output=True, text=True).stdout.strip()
    if not ref or not os.path.isdir(os.path.join(ref, "src", "gsAssembler")):
        pytest.skip("G+Smo source tree not available")
    r = subprocess.run(["make", "-s", "-C", mk, "dropin-syntax"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]


def test_dropin_pack_matches_reference_mapper(lib):
    """The C++ drop-in packs glued multipatch grids built by the reference (its own interface
    orientation flags) with Dirichlet and Neumann sides from gsBoundaryConditions; a host-only
    context's dof map equals the reference's gsDofMapper (oracle/ref/pack_check.cpp). Needs the
    G+Smo source tree; skipped where it is absent."""
    import shutil
    import subprocess
    mk = os.path.join(ROOT, "oracle", "ref")
    if shutil.which("make") is None or shutil.which("g++") is None:
        pytest.skip("no make / g++")
    ref = subprocess.run(["make", "-s", "-C", mk, "print-ref"], capture_output=True, text=True).stdout.strip()
    if not ref or not os.path.isdir(os.path.join(ref, "src", "gsAssembler")):
        pytest.skip("G+Smo source tree not available")
    r = subprocess.run(["make", "-s", "-C", mk, "packcheck"], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-3000:])
    assert r.stdout.strip().endswith("ok")


@pytest.mark.parametrize("bad", ["dirichlet", "interface", "index", "duplicate"])
def test_invalid_neumann_sides_are_rejected(lib, bad):
    """One condition per boundary side (gsBoundaryConditions): a Neumann side that is also
    Dirichlet, an interface side, a side index out of range or a repeated side is an input error."""
    from gismo_gb300 import problems as P
    if bad == "interface":
        prob = P.mixed_boundary(P.cube_grid(n=2, n_elem=2, p=2, seed=1, kappa_modes=0))
        prob.neumann.append(tuple(prob.interfaces[0][:2]))
    else:
        prob = P.mixed_boundary(P.square_poisson(4, 2))
        prob.neumann.append({"dirichlet": prob.dirichlet[0], "index": (0, 7), "duplicate": prob.neumann[0]}[bad])
    h = C.c_void_p()
    assert lib.gsgpu_create(C.byref(h), -1) == _lib.OK
    pk = PackedProblem(prob)
    assert lib.gsgpu_set_problem(h, C.byref(pk.struct)) == _lib.ERR_INVALID
    assert b"neumann" in lib.gsgpu_last_error(h)
    lib.gsgpu_destroy(h)


def test_ctypes_structs_match_the_header(tmp_path):
    """The ctypes mirrors of the C-ABI structs (gismo_gb300/_lib.py, and the oracle's problem
    struct) have the headers' field offsets and sizes: a C program compiled against
    include/gsgpu.h and oracle/gsoracle.h prints offsetof / sizeof for every field."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    from oracle import oracle as O
    structs = {"gsgpu_problem": _lib.Problem, "gsgpu_solver_opts": _lib.SolverOpts,
               "gsgpu_solve_info": _lib.SolveInfo, "gsgpu_request_info": _lib.RequestInfo,
               "orc_problem": O._Problem}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gsgpu.h"', '#include "gsoracle.h"',
             "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    r = subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "oracle"), str(src), "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {tuple(ln.split()[:2]): int(ln.split()[2]) for ln in out if ln}
    for cname, py in structs.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert got[(cname, fname)] == getattr(py, fname).offset, (cname, fname)


@pytest.mark.parametrize("name", ["large_vol_p3_n32_s1", "large_cube_p3_n64"])
def test_host_plan_sizes_match_large_reference_runs(lib, name):
    """The reference's free-dof and non-zero counts at the benchmark's sizes, from the host plan of a
    host-only context (no GPU)."""
    from tests.golden_cases import golden_module, load_golden
    g = load_golden(name)
    prob = golden_module().large_cases()[name]
    h, pk = _host_ctx(lib, prob)
    nf, nnz, nb, nl = C.c_int(), C.c_longlong(), C.c_int(), C.c_int()
    assert lib.gsgpu_sizes(h, C.byref(nf), C.byref(nnz), C.byref(nb), C.byref(nl)) == _lib.OK
    assert (nf.value, nnz.value) == (int(g["free"]), int(g["nnz"]))
    lib.gsgpu_destroy(h)


def test_dropin_checks_caller_functions(lib):
    """The C++ drop-in compares the caller's rhs, Dirichlet and Neumann functions with the closed
    forms the device evaluates and throws on a mismatch (oracle/ref/dropin_check.cpp, host-only
    contexts, no GPU). Needs the G+Smo source tree; skipped where it is absent."""
    import shutil
    import subprocess
    mk = os.path.join(ROOT, "oracle", "ref")
    if shutil.which("make") is None or shutil.which("g++") is None:
        pytest.skip("no make / g++")
    ref = subprocess.run(["make", "-s", "-C", mk, "print-ref"], capture_output=True, text=True).stdout.strip()
    if not ref or not os.path.isdir(os.path.join(ref, "src", "gsAssembler")):
        pytest.skip("G+Smo source tree not available")
    r = subprocess.run(["make", "-s", "-C", mk, "dropincheck"], capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-3000:])
    assert r.stdout.strip().endswith("ok")
