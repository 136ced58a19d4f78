"""The C++ layer of the drop-ins (include/gsgpu.hpp) on the GPU: tests/cpp/system_check.cpp is
compiled with g++ against libgsgpu.so (no G+Smo needed) and run on the 2D degree-2 64 x 64 unit
square, the reference's own CPU-runnable configuration. Its CSR arrays (read straight into
compressed-storage arrays), rhs, CG iteration count and L2 / H1 errors are compared with the
reference fixture square_p2_n64; the mixed-precision solve of the same system reaches the FP64
solution; an out-of-order call throws gsgpu::Error with the state code."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from tests.golden_cases import load_golden
from tests.test_oracle_golden import _csr_from_csc

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_system_layer_matches_reference_fixture(tmp_path):
    import __graft_entry__ as g
    g.build()
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "system_check")
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "system_check.cpp"), "-L", os.path.join(ROOT, "gismo_gb300"),
                    "-lgsgpu", "-Wl,-rpath," + os.path.join(ROOT, "gismo_gb300"), "-o", exe], check=True)
    out = subprocess.run([exe, "64", "2", str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    f = out.stdout.split()
    nfree, nnz, its, relres, l2, h1 = int(f[0]), int(f[1]), int(f[2]), float(f[3]), float(f[4]), float(f[5])
    converged, mixed_err, threw = int(f[6]), float(f[7]), int(f[8])
    g = load_golden("square_p2_n64")
    K = _csr_from_csc(g)
    assert (nfree, nnz) == (int(g["free"]), int(g["nnz"]))
    ptr = np.fromfile(str(tmp_path / "ptr.i32"), np.int32)
    col = np.fromfile(str(tmp_path / "col.i32"), np.int32)
    val = np.fromfile(str(tmp_path / "val.f64"), np.float64)
    assert np.array_equal(ptr, K.indptr) and np.array_equal(col, K.indices)
    assert np.abs(val - K.data).max() <= 1e-12 * np.abs(K.data).max()
    rhs = np.fromfile(str(tmp_path / "rhs.f64"), np.float64)
    assert np.abs(rhs - g["rhs"]).max() <= 1e-12 * np.abs(g["rhs"]).max()
    assert converged == 1 and relres < 1e-10 and abs(its - int(g["iters"])) <= 1
    x = np.fromfile(str(tmp_path / "x.f64"), np.float64)
    assert np.linalg.norm(x - g["x"]) <= 1e-8 * np.linalg.norm(g["x"])
    assert abs(l2 - float(g["l2"])) <= 5e-4 * float(g["l2"])
    assert abs(h1 - float(g["h1"])) <= 5e-4 * float(g["h1"])
    assert mixed_err <= 1e-8
    assert threw == 1
