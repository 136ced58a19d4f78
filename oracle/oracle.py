"""ctypes binding of the CPU oracle (oracle/gsoracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg, never by the product package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "gsoracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-o", LIB_PATH, src])
    return LIB_PATH


class _Problem(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("npatches", C.c_int),
        ("degree", C.POINTER(C.c_int)), ("nknots", C.POINTER(C.c_int)), ("knots", C.POINTER(C.c_double)),
        ("gdegree", C.POINTER(C.c_int)), ("gnknots", C.POINTER(C.c_int)), ("gknots", C.POINTER(C.c_double)),
        ("coefs", C.POINTER(C.c_double)),
        ("ninterfaces", C.c_int), ("interfaces", C.POINTER(C.c_int)),
        ("ndirichlet", C.c_int), ("dirichlet", C.POINTER(C.c_int)),
        ("kappa_fourier", C.c_int), ("kappa_const", C.c_double), ("kappa_alpha", C.c_double),
        ("kappa_scale", C.c_double), ("kappa_nmodes", C.c_int), ("kappa_amp", C.POINTER(C.c_double)),
        ("kappa_k", C.POINTER(C.c_int)), ("kappa_phase", C.POINTER(C.c_double)),
        ("ufreq", C.c_int), ("quA", C.c_double), ("quB", C.c_int), ("dirichlet_l2", C.c_int),
        ("nneumann", C.c_int), ("neumann", C.POINTER(C.c_int)),
    ]


def _lib():
    lib = C.CDLL(build())
    vp = C.c_void_p
    lib.orc_create.restype = vp
    lib.orc_create.argtypes = [C.POINTER(_Problem)]
    lib.orc_destroy.argtypes = [vp]
    lib.orc_assemble.restype = C.c_double
    lib.orc_assemble.argtypes = [vp, C.c_int, C.c_longlong]
    lib.orc_sizes.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_longlong), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.orc_dofmap.argtypes = [vp, C.c_void_p]
    lib.orc_csr.argtypes = [vp, C.c_void_p, C.c_void_p, C.c_void_p]
    lib.orc_rhs.argtypes = [vp, C.c_void_p]
    lib.orc_ddof.argtypes = [vp, C.c_void_p]
    lib.orc_solve_cg.restype = C.c_double
    lib.orc_solve_cg.argtypes = [vp, C.c_double, C.c_int, C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    lib.orc_solve_mg.restype = C.c_double
    lib.orc_solve_mg.argtypes = [vp, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int,
                                 C.c_double, C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    lib.orc_l2_error.restype = C.c_double
    lib.orc_l2_error.argtypes = [vp, C.c_void_p]
    lib.orc_mass.restype = None
    lib.orc_mass.argtypes = [vp, C.c_void_p]
    lib.orc_h1_error.restype = C.c_double
    lib.orc_h1_error.argtypes = [vp, C.c_void_p]
    lib.orc_error_evaluator_rule.restype = C.c_double
    lib.orc_error_evaluator_rule.argtypes = [vp, C.c_void_p, C.c_int]
    lib.orc_gauss.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
    return lib


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        _LIB = _lib()
    return _LIB


def _ptr(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class OracleProblem:
    """Owns the packed arrays of a gismo_gb300.problems.Problem and the oracle handle."""

    def __init__(self, prob):
        d = prob.dim
        deg, nk, kn, gdeg, gnk, gkn, co = [], [], [], [], [], [], []
        for pt in prob.patches:
            for k in range(3):
                if k < d:
                    deg.append(pt.degree[k]); nk.append(len(pt.knots[k])); kn.extend(pt.knots[k])
                    gdeg.append(pt.gdegree[k]); gnk.append(len(pt.gknots[k])); gkn.extend(pt.gknots[k])
                else:
                    deg.append(0); nk.append(0); gdeg.append(0); gnk.append(0)
            co.append(np.ascontiguousarray(pt.coefs, dtype=np.float64).ravel())
        self._a = dict(
            degree=np.array(deg, np.int32), nknots=np.array(nk, np.int32), knots=np.array(kn, np.float64),
            gdegree=np.array(gdeg, np.int32), gnknots=np.array(gnk, np.int32), gknots=np.array(gkn, np.float64),
            coefs=np.concatenate(co), ifaces=np.array(prob.interfaces, np.int32).reshape(-1),
            dirichlet=np.array(prob.dirichlet, np.int32).reshape(-1),
            neumann=np.array(getattr(prob, "neumann", []), np.int32).reshape(-1),
            amp=np.ascontiguousarray(prob.kappa_amp, np.float64), kk=np.ascontiguousarray(prob.kappa_k, np.int32).reshape(-1),
            phase=np.ascontiguousarray(prob.kappa_phase, np.float64),
        )
        a = self._a
        s = _Problem()
        s.dim = d
        s.npatches = len(prob.patches)
        s.degree = _ptr(a["degree"], C.c_int); s.nknots = _ptr(a["nknots"], C.c_int); s.knots = _ptr(a["knots"], C.c_double)
        s.gdegree = _ptr(a["gdegree"], C.c_int); s.gnknots = _ptr(a["gnknots"], C.c_int); s.gknots = _ptr(a["gknots"], C.c_double)
        s.coefs = _ptr(a["coefs"], C.c_double)
        s.ninterfaces = len(prob.interfaces); s.interfaces = _ptr(a["ifaces"], C.c_int)
        s.ndirichlet = len(prob.dirichlet); s.dirichlet = _ptr(a["dirichlet"], C.c_int)
        s.kappa_fourier = int(prob.kappa_fourier); s.kappa_const = prob.kappa_const
        s.kappa_alpha = prob.kappa_alpha; s.kappa_scale = prob.kappa_scale
        s.kappa_nmodes = len(prob.kappa_amp) if prob.kappa_fourier else 0
        s.kappa_amp = _ptr(a["amp"], C.c_double); s.kappa_k = _ptr(a["kk"], C.c_int); s.kappa_phase = _ptr(a["phase"], C.c_double)
        s.ufreq = prob.ufreq; s.quA = prob.quA; s.quB = prob.quB
        s.dirichlet_l2 = 1 if getattr(prob, "dirichlet_l2", False) else 0
        s.nneumann = len(a["neumann"]) // 2; s.neumann = _ptr(a["neumann"], C.c_int)
        self._s = s
        self.prob = prob
        self.h = lib().orc_create(C.byref(s))
        if not self.h:
            raise ValueError("oracle rejected the problem")

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def assemble(self, nthreads: int = 0, max_elements: int = -1) -> float:
        return lib().orc_assemble(self.h, nthreads, max_elements)

    def sizes(self):
        nf, nnz, nb, nl = C.c_int(), C.c_longlong(), C.c_int(), C.c_int()
        lib().orc_sizes(self.h, C.byref(nf), C.byref(nnz), C.byref(nb), C.byref(nl))
        return nf.value, nnz.value, nb.value, nl.value

    def dofmap(self):
        nl = self.sizes()[3]
        out = np.empty(nl, np.int32)
        lib().orc_dofmap(self.h, out.ctypes.data)
        return out

    def csr(self):
        nf, nnz, _, _ = self.sizes()
        ptr = np.empty(nf + 1, np.int32); idx = np.empty(nnz, np.int32); val = np.empty(nnz, np.float64)
        lib().orc_csr(self.h, ptr.ctypes.data, idx.ctypes.data, val.ctypes.data)
        return ptr, idx, val

    def rhs(self):
        out = np.empty(self.sizes()[0], np.float64)
        lib().orc_rhs(self.h, out.ctypes.data)
        return out

    def ddof(self):
        out = np.empty(self.sizes()[2], np.float64)
        lib().orc_ddof(self.h, out.ctypes.data)
        return out

    def solve_cg(self, tol=1e-10, maxit=1000):
        x = np.zeros(self.sizes()[0])
        it, rr = C.c_int(), C.c_double()
        t = lib().orc_solve_cg(self.h, tol, maxit, x.ctypes.data, C.byref(it), C.byref(rr))
        return x, it.value, rr.value, t

    def solve_mg(self, tol=1e-8, maxit=1000, levels=4, npre=2, npost=2, damping=0.6, cycles=1, cgc_damping=1.0):
        x = np.zeros(self.sizes()[0])
        it, rr = C.c_int(), C.c_double()
        t = lib().orc_solve_mg(self.h, tol, maxit, levels, npre, npost, damping, cycles, cgc_damping, x.ctypes.data,
                               C.byref(it), C.byref(rr))
        return x, it.value, rr.value, t

    def mass(self):
        """gsGenericAssembler::assembleMass on the free dofs: values in the CSR pattern of csr()."""
        val = np.empty(self.sizes()[1], np.float64)
        lib().orc_mass(self.h, val.ctypes.data)
        return val

    def l2_error(self, x):
        x = np.ascontiguousarray(x, np.float64)
        return lib().orc_l2_error(self.h, x.ctypes.data)

    def h1_error(self, x):
        x = np.ascontiguousarray(x, np.float64)
        return lib().orc_h1_error(self.h, x.ctypes.data)

    def reference_norms(self, x):
        """(L2, H1 seminorm) errors with gsField::distanceL2/H1's own rule (p + 1 Gauss points per
        direction, whatever quA/quB the problem assembles with)."""
        x = np.ascontiguousarray(x, np.float64)
        return (lib().orc_error_evaluator_rule(self.h, x.ctypes.data, 0),
                lib().orc_error_evaluator_rule(self.h, x.ctypes.data, 1))


def gauss(n: int):
    x = np.empty(n); w = np.empty(n)
    lib().orc_gauss(n, x.ctypes.data, w.ctypes.data)
    return x, w
