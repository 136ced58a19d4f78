"""Python mirror of G+Smo's gsPoissonAssembler / gsConjugateGradient interface over libgsgpu.

    A = GpuPoissonAssembler(problem)          # gsPoissonAssembler(mp, mb, bc, f) + refresh()
    A.assemble()                              # gsPoissonAssembler::assemble()
    K, b = A.matrix(), A.rhs()                # gsAssembler::matrix() / rhs()
    x, info = A.solve(tol=1e-10)              # gsConjugateGradient(K, gsJacobiOp(K)).solve(b, x)

(src/gsAssembler/gsPoissonAssembler.h:35-142, src/gsAssembler/gsAssembler.h:538-639,
src/gsSolver/gsConjugateGradient.hpp). Errors raise GsGpuError (G+Smo raises std::runtime_error
from GISMO_ENSURE); non-convergence is reported in the info like gsIterativeSolver::error().
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib
from ._lib import GsGpuError, Problem as _CProblem, SolverOpts, SolveInfo


def _ptr(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class PackedProblem:
    """The C-ABI problem struct (include/gsgpu.h gsgpu_problem) plus the arrays it points to."""

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
        self.arrays = dict(
            degree=np.array(deg, np.int32), nknots=np.array(nk, np.int32), knots=np.array(kn, np.float64),
            gdegree=np.array(gdeg, np.int32), gnknots=np.array(gnk, np.int32), gknots=np.array(gkn, np.float64),
            coefs=np.concatenate(co), ifaces=np.array(prob.interfaces, np.int32).reshape(-1),
            dirichlet=np.array(prob.dirichlet, np.int32).reshape(-1),
            neumann=np.array(getattr(prob, "neumann", []), np.int32).reshape(-1),
            amp=np.ascontiguousarray(prob.kappa_amp, np.float64),
            kk=np.ascontiguousarray(prob.kappa_k, np.int32).reshape(-1),
            phase=np.ascontiguousarray(prob.kappa_phase, np.float64),
        )
        a = self.arrays
        s = _CProblem()
        s.dim = d
        s.npatches = len(prob.patches)
        s.degree = _ptr(a["degree"], C.c_int); s.nknots = _ptr(a["nknots"], C.c_int); s.knots = _ptr(a["knots"], C.c_double)
        s.gdegree = _ptr(a["gdegree"], C.c_int); s.gnknots = _ptr(a["gnknots"], C.c_int)
        s.gknots = _ptr(a["gknots"], C.c_double)
        s.coefs = _ptr(a["coefs"], C.c_double)
        s.ninterfaces = len(prob.interfaces); s.interfaces = _ptr(a["ifaces"], C.c_int)
        s.ndirichlet = len(prob.dirichlet); s.dirichlet = _ptr(a["dirichlet"], C.c_int)
        s.kappa_fourier = int(prob.kappa_fourier); s.kappa_const = prob.kappa_const
        s.kappa_alpha = prob.kappa_alpha; s.kappa_scale = prob.kappa_scale
        s.kappa_nmodes = len(prob.kappa_amp) if prob.kappa_fourier else 0
        s.kappa_amp = _ptr(a["amp"], C.c_double); s.kappa_k = _ptr(a["kk"], C.c_int)
        s.kappa_phase = _ptr(a["phase"], C.c_double)
        s.ufreq = prob.ufreq; s.quA = prob.quA; s.quB = prob.quB
        s.dirichlet_strategy = 1 if getattr(prob, "dirichlet_l2", False) else 0
        s.nneumann = len(a["neumann"]) // 2; s.neumann = _ptr(a["neumann"], C.c_int)
        self.struct = s


class GpuPoissonAssembler:
    """gsPoissonAssembler on the GPU: one context per problem (device memory is owned here)."""

    def __init__(self, prob, device: int = 0, refresh: bool = True):
        self.L = _lib.lib()
        self.prob = prob
        self.h = C.c_void_p()
        rc = self.L.gsgpu_create(C.byref(self.h), device)
        if rc != _lib.OK:
            raise GsGpuError(rc, "could not create a context on CUDA device %d" % device)
        self._packed = PackedProblem(prob)
        self._check(self.L.gsgpu_set_problem(self.h, C.byref(self._packed.struct)))
        if refresh:
            self.refresh()

    def _check(self, rc: int) -> int:
        if rc != _lib.OK:
            raise GsGpuError(rc, self.L.gsgpu_last_error(self.h).decode())
        return rc

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.gsgpu_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- gsAssembler interface ----
    def refresh(self):
        self._check(self.L.gsgpu_refresh(self.h))

    def set_coefs(self, coefs: np.ndarray):
        c = np.ascontiguousarray(coefs, np.float64)
        self._check(self.L.gsgpu_set_coefs(self.h, c.ctypes.data))

    def assemble(self, precision: str = "fp64"):
        prec = _lib.PREC_FP64 if precision == "fp64" else _lib.PREC_MIXED
        self._check(self.L.gsgpu_assemble(self.h, prec))

    def sizes(self):
        nf, nnz, nb, nl = C.c_int(), C.c_longlong(), C.c_int(), C.c_int()
        self._check(self.L.gsgpu_sizes(self.h, C.byref(nf), C.byref(nnz), C.byref(nb), C.byref(nl)))
        return nf.value, nnz.value, nb.value, nl.value

    def numDofs(self) -> int:
        return self.sizes()[0]

    def csr(self):
        nf, nnz, _, _ = self.sizes()
        ptr = np.empty(nf + 1, np.int32)
        col = np.empty(nnz, np.int32)
        val = np.empty(nnz, np.float64)
        self._check(self.L.gsgpu_matrix_csr(self.h, ptr.ctypes.data, col.ctypes.data, val.ctypes.data))
        return ptr, col, val

    def matrix(self):
        import scipy.sparse as sp
        ptr, col, val = self.csr()
        n = len(ptr) - 1
        return sp.csr_matrix((val, col, ptr), shape=(n, n))

    def mass_csr(self) -> np.ndarray:
        """gsGenericAssembler::assembleMass on the device: the mass matrix's values in the CSR
        pattern of csr() (gsgpu_mass_csr); the next solve or matrix read needs a new assemble()."""
        val = np.empty(self.sizes()[1], np.float64)
        self._check(self.L.gsgpu_mass_csr(self.h, val.ctypes.data))
        return val

    def diagonal(self) -> np.ndarray:
        """matrix().diagonal() (gsSparseMatrix::diagonal), from the downloaded CSR arrays."""
        ptr, col, val = self.csr()
        rows = np.repeat(np.arange(len(ptr) - 1, dtype=np.int32), np.diff(ptr))
        on = col == rows
        d = np.zeros(len(ptr) - 1)
        d[rows[on]] = val[on]
        return d

    def rhs(self) -> np.ndarray:
        out = np.empty(self.sizes()[0], np.float64)
        self._check(self.L.gsgpu_rhs(self.h, out.ctypes.data))
        return out

    def fixedDofs(self) -> np.ndarray:
        out = np.empty(self.sizes()[2], np.float64)
        self._check(self.L.gsgpu_fixed_dofs(self.h, out.ctypes.data))
        return out

    def dofMapper(self) -> np.ndarray:
        out = np.empty(self.sizes()[3], np.int32)
        self._check(self.L.gsgpu_dof_map(self.h, out.ctypes.data))
        return out

    def apply(self, x: np.ndarray) -> np.ndarray:
        """gsMatrixOp::apply on the device: K x with the assembled FP64 matrix."""
        x = np.ascontiguousarray(x, np.float64)
        y = np.empty_like(x)
        self._check(self.L.gsgpu_apply(self.h, x.ctypes.data, y.ctypes.data))
        return y

    def mg_apply(self, r: np.ndarray, mg_levels: int = 4, mg_npre: int = 2, mg_npost: int = 2,
                 mg_damping: float = 0.6, mg_cycles: int = 1, mg_cgc_damping: float = 1.0) -> np.ndarray:
        """gsMultiGridOp as a preconditioner: one FP64 cycle (V for mg_cycles=1, W for 2) on r
        from a zero start."""
        o = SolverOpts()
        o.method, o.precision = _lib.SOLVER_CG_MG, _lib.PREC_FP64
        o.mg_levels, o.mg_npre, o.mg_npost, o.mg_damping = mg_levels, mg_npre, mg_npost, mg_damping
        o.mg_cycles, o.mg_cgc_damping = mg_cycles, mg_cgc_damping
        r = np.ascontiguousarray(r, np.float64)
        z = np.empty_like(r)
        self._check(self.L.gsgpu_mg_apply(self.h, C.byref(o), r.ctypes.data, z.ctypes.data))
        return z

    def set_fixed_dofs(self, ddof):
        """Eliminated-dof values for the next assembles (e.g. the caller's own interpolation or
        L2 projection of the Dirichlet data); None restores the built-in interpolation."""
        if ddof is None:
            self._check(self.L.gsgpu_set_fixed_dofs(self.h, None, 0))
            return
        self._fixed = np.ascontiguousarray(ddof, np.float64)
        self._check(self.L.gsgpu_set_fixed_dofs(self.h, self._fixed.ctypes.data, len(self._fixed)))

    def l2_error(self) -> float:
        """gsField::distanceL2 of the last solution against the manufactured solution."""
        v = C.c_double()
        self._check(self.L.gsgpu_l2_error(self.h, C.byref(v)))
        return v.value

    def h1_error(self) -> float:
        """gsField::distanceH1 (H1 seminorm of the error) of the last solution."""
        v = C.c_double()
        self._check(self.L.gsgpu_h1_error(self.h, C.byref(v)))
        return v.value

    def min_jacobian(self) -> float:
        v = C.c_double()
        self._check(self.L.gsgpu_min_jacobian(self.h, C.byref(v)))
        return v.value

    def assemble_times(self) -> np.ndarray:
        out = np.zeros(7)
        self._check(self.L.gsgpu_assemble_times(self.h, out.ctypes.data))
        return out

    def stream_handle(self) -> int:
        v = C.c_void_p()
        self._check(self.L.gsgpu_stream(self.h, C.byref(v)))
        return v.value or 0

    def autotune(self):
        """Time every kernel variant on this problem, record the fastest in the process-wide tuning
        table and apply it (gsgpu_autotune). Returns the measured milliseconds: six stiffness
        combinations and three inner products (-1 where not applicable)."""
        ms = np.empty(9, np.float64)
        self._check(self.L.gsgpu_autotune(self.h, ms.ctypes.data))
        return ms

    def tuned_variants(self):
        """(stage 1, stage 2, inner product) variants of this context (gsgpu_tuned_variants)."""
        v = np.empty(3, np.int32)
        self._check(self.L.gsgpu_tuned_variants(self.h, v.ctypes.data))
        return tuple(int(a) for a in v)

    def set_profiling(self, on: bool):
        self._check(self.L.gsgpu_set_profiling(self.h, int(on)))

    def spmv_stats(self):
        n, ms, b = C.c_longlong(), C.c_double(), C.c_double()
        self._check(self.L.gsgpu_spmv_stats(self.h, C.byref(n), C.byref(ms), C.byref(b)))
        return n.value, ms.value, b.value

    # ---- gsConjugateGradient ----
    def solve(self, tol: float = 1e-10, max_iters: int = 1000, method: str = "jacobi", precision: str = "fp64",
              mg_levels: int = 4, mg_npre: int = 2, mg_npost: int = 2, mg_damping: float = 0.6,
              inner_tol: float = 1e-4, download: bool = True, mg_cycles: int = 1, mg_cgc_damping: float = 1.0,
              out: Optional[np.ndarray] = None):
        """`out`: a caller-owned contiguous float64 array of numDofs() entries (for instance a view of
        pinned host memory) that receives the solution instead of a new array."""
        o = SolverOpts()
        o.method = _lib.SOLVER_CG_JACOBI if method == "jacobi" else _lib.SOLVER_CG_MG
        o.precision = _lib.PREC_FP64 if precision == "fp64" else _lib.PREC_MIXED
        o.tol, o.max_iters = tol, max_iters
        o.mg_levels, o.mg_npre, o.mg_npost, o.mg_damping = mg_levels, mg_npre, mg_npost, mg_damping
        o.mg_cycles, o.mg_cgc_damping = mg_cycles, mg_cgc_damping
        o.inner_tol = inner_tol
        info = SolveInfo()
        if out is not None:
            if out.dtype != np.float64 or not out.flags["C_CONTIGUOUS"] or out.size != self.sizes()[0]:
                raise ValueError("out must be a contiguous float64 array of numDofs() entries")
            x, download = out, True
        else:
            x = np.empty(self.sizes()[0], np.float64) if download else None
        rc = self.L.gsgpu_solve(self.h, C.byref(o), x.ctypes.data if download else None, C.byref(info))
        if rc not in (_lib.OK, _lib.ERR_NOT_CONVERGED):
            self._check(rc)
        return x, dict(iterations=info.iterations, relres=info.relres, refinements=info.refinements,
                       t_solve_ms=info.t_solve_ms, converged=(rc == _lib.OK))


class GpuPoissonBatch(GpuPoissonAssembler):
    """A batch of independent single-patch problems in one context: what G+Smo runs as one
    gsPoissonAssembler + gsConjugateGradient per problem, assembled by the same launches and solved
    by a segmented CG with per-problem scalars and stopping tests (include/gsgpu.h gsgpu_set_batch)."""

    def __init__(self, problems, device: int = 0, refresh: bool = True):
        self.L = _lib.lib()
        self.problems = list(problems)
        self.prob = None
        self.h = C.c_void_p()
        rc = self.L.gsgpu_create(C.byref(self.h), device)
        if rc != _lib.OK:
            raise GsGpuError(rc, "could not create a context on CUDA device %d" % device)
        self._packed = [PackedProblem(p) for p in self.problems]
        arr = (_CProblem * len(self._packed))(*[pp.struct for pp in self._packed])
        self._structs = arr
        self._check(self.L.gsgpu_set_batch(self.h, len(self._packed), C.cast(arr, C.c_void_p)))
        if refresh:
            self.refresh()

    def offsets(self) -> np.ndarray:
        out = np.zeros(len(self.problems) + 1, np.int32)
        self._check(self.L.gsgpu_batch_info(self.h, out.ctypes.data, None, None))
        return out

    def solve(self, tol: float = 1e-10, max_iters: int = 1000, precision: str = "fp64", inner_tol: float = 1e-5,
              download: bool = True, **_unused):
        """Per problem: solution, iterations and relative residual (info['per_problem'])."""
        x, info = super().solve(tol=tol, max_iters=max_iters, method="jacobi", precision=precision,
                                inner_tol=inner_tol, download=download)
        n = len(self.problems)
        its = np.zeros(n, np.int32)
        rr = np.zeros(n, np.float64)
        self._check(self.L.gsgpu_batch_info(self.h, None, its.ctypes.data, rr.ctypes.data))
        info["per_problem"] = dict(iterations=its, relres=rr)
        if download:
            off = self.offsets()
            x = [x[off[j]:off[j + 1]] for j in range(n)]
        return x, info

    def l2_errors(self) -> np.ndarray:
        out = np.zeros(len(self.problems), np.float64)
        self._check(self.L.gsgpu_batch_l2_error(self.h, out.ctypes.data))
        return out

    def h1_errors(self) -> np.ndarray:
        out = np.zeros(len(self.problems), np.float64)
        self._check(self.L.gsgpu_batch_h1_error(self.h, out.ctypes.data))
        return out


class GpuPoissonServer:
    """Request server with continuous batching (include/gsgpu.h gsgpu_server_*): submit() queues a
    copy of a single-patch problem and returns at once; result() blocks until it is solved. Worker
    slots batch the queued requests of one dimension under a device-memory budget."""

    def __init__(self, device: int = 0, slots: int = 4, budget_gb: float = 120.0, max_batch: int = 64,
                 precision: str = "mixed"):
        self.L = _lib.lib()
        self.h = C.c_void_p()
        prec = _lib.PREC_FP64 if precision == "fp64" else _lib.PREC_MIXED
        rc = self.L.gsgpu_server_create(C.byref(self.h), device, slots, budget_gb * 1e9, max_batch, prec)
        if rc != _lib.OK:
            raise GsGpuError(rc, "could not create the server")
        self._sizes = {}

    def submit(self, prob, tol: float = 1e-8) -> int:
        pk = PackedProblem(prob)
        rid = C.c_longlong()
        rc = self.L.gsgpu_server_submit(self.h, C.byref(pk.struct), tol, C.byref(rid))
        if rc != _lib.OK:
            raise GsGpuError(rc, self.L.gsgpu_server_last_error(self.h).decode())
        n = 1
        for pt in prob.patches:
            for k in range(prob.dim):
                n *= len(pt.knots[k]) - pt.degree[k] - 1
        self._sizes[rid.value] = n
        return rid.value

    def result(self, rid: int):
        """(x, info) of request rid; info['status'] is the request's status code."""
        cap = self._sizes.pop(rid, 0)
        x = np.empty(cap, np.float64)
        info = _lib.RequestInfo()
        rc = self.L.gsgpu_server_wait(self.h, rid, x.ctypes.data, cap, C.byref(info))
        d = {f: getattr(info, f) for f, _ in _lib.RequestInfo._fields_}
        if rc not in (_lib.OK, _lib.ERR_NOT_CONVERGED, _lib.ERR_BUDGET):
            raise GsGpuError(rc, self.L.gsgpu_server_last_error(self.h).decode())
        return x[:info.nfree], d

    def set_resident(self, gb: float):
        """Device memory (GB) that resident batch contexts may hold (gsgpu_server_set_resident)."""
        self._check_rc(self.L.gsgpu_server_set_resident(self.h, gb * 1e9))

    def _check_rc(self, rc):
        if rc != _lib.OK:
            raise GsGpuError(rc, self.L.gsgpu_server_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            self.L.gsgpu_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tune_save(path: str) -> None:
    """Write the process-wide tuning table (gsgpu_tune_save)."""
    if _lib.lib().gsgpu_tune_save(path.encode()) != _lib.OK:
        raise GsGpuError(_lib.ERR_INVALID, f"could not write the tuning table {path}")


def tune_load(path: str) -> None:
    """Add the entries of a tuning table file to the process-wide table (gsgpu_tune_load)."""
    if _lib.lib().gsgpu_tune_load(path.encode()) != _lib.OK:
        raise GsGpuError(_lib.ERR_INVALID, f"could not read the tuning table {path}")


def tune_clear() -> None:
    _lib.lib().gsgpu_tune_clear()
