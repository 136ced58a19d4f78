"""Seeded synthetic inputs for the isogeometric Poisson / diffusion path.

Every configuration the benchmark and the parity tests use is built here, from a seed, so that
the GPU path, the CPU oracle and the reference (through the text spec written by
:func:`write_spec`) all see bit-identical knots, control points and coefficient parameters.

Conventions follow G+Smo:
  * open knot vectors as built by ``gsKnotVector(a, b, interior, p+1)``
    (src/gsNurbs/gsKnotVector.h:457): p+1 end repetitions and uniform interior knots;
  * control points are stored lexicographically with the first parametric direction fastest
    (gsTensorBasis::index, src/gsTensor/gsTensorBasis.h);
  * the identity map uses the Greville abscissae as control points
    (gsBasis::anchors, src/gsNurbs/gsKnotVector.hpp:991-1026);
  * box sides are numbered west=1, east=2, south=3, north=4, front=5, back=6
    (src/gsCore/gsBoundary.h); side s fixes direction (s-1)//2 at parameter (s-1)%2.

Closed-form fields (the same formulas are evaluated on the device and in the oracle):
  g(x)   = scale * sum_m amp_m cos(pi k_m . x + phase_m)
  kappa  = exp(alpha * g)              (or a constant)
  u(x)   = prod_i sin(freq * pi * x_i)  (manufactured solution, also the Dirichlet data)
  f      = -div(kappa grad u)
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence, Tuple

import numpy as np

SIDE_WEST, SIDE_EAST, SIDE_SOUTH, SIDE_NORTH, SIDE_FRONT, SIDE_BACK = 1, 2, 3, 4, 5, 6


def side_direction(side: int) -> int:
    return (side - 1) // 2


def side_parameter(side: int) -> int:
    return (side - 1) % 2


def open_uniform_knots(n_elem: int, p: int, a: float = 0.0, b: float = 1.0) -> np.ndarray:
    """Open uniform knot vector with ``n_elem`` elements on [a, b] and end multiplicity p+1."""
    interior = [a + (b - a) * i / n_elem for i in range(1, n_elem)]
    return np.array([a] * (p + 1) + interior + [b] * (p + 1), dtype=np.float64)


def greville(knots: np.ndarray, p: int) -> np.ndarray:
    n = len(knots) - p - 1
    if p == 0:
        return 0.5 * (knots[:-1] + knots[1:])
    return np.array([knots[i + 1:i + p + 1].sum() / p for i in range(n)], dtype=np.float64)


def bspline_basis_matrix(knots: np.ndarray, p: int, pts: np.ndarray, deriv: int = 0) -> np.ndarray:
    """Dense (len(pts) x n) matrix of B-spline values (deriv=0) or first derivatives (deriv=1).

    Cox-de Boor recursion, vectorised over points. Used by the input generator only (the
    Jacobian-positivity check); the product path evaluates bases on the device.
    """
    pts = np.asarray(pts, dtype=np.float64)
    n = len(knots) - p - 1
    m = len(knots)
    # degree-0 indicator with the right end included in the last non-empty span
    last = np.max(np.nonzero(knots[:-1] < knots[1:])[0])
    N = np.zeros((len(pts), m - 1))
    for i in range(m - 1):
        if knots[i] < knots[i + 1]:
            hi = (pts <= knots[i + 1]) if i == last else (pts < knots[i + 1])
            N[:, i] = ((pts >= knots[i]) & hi).astype(np.float64)
    for k in range(1, p + 1):
        Nk = np.zeros((len(pts), m - 1 - k))
        for i in range(m - 1 - k):
            d1 = knots[i + k] - knots[i]
            d2 = knots[i + k + 1] - knots[i + 1]
            if deriv == 1 and k == p:
                t = np.zeros(len(pts))
                if d1 > 0:
                    t += k / d1 * N[:, i]
                if d2 > 0:
                    t -= k / d2 * N[:, i + 1]
                Nk[:, i] = t
            else:
                t = np.zeros(len(pts))
                if d1 > 0:
                    t += (pts - knots[i]) / d1 * N[:, i]
                if d2 > 0:
                    t += (knots[i + k + 1] - pts) / d2 * N[:, i + 1]
                Nk[:, i] = t
        N = Nk
    return N[:, :n]


def gauss_legendre(n: int) -> Tuple[np.ndarray, np.ndarray]:
    x, w = np.polynomial.legendre.leggauss(n)
    return x, w


@dataclasses.dataclass
class Patch:
    dim: int
    degree: Tuple[int, ...]
    knots: List[np.ndarray]
    gdegree: Tuple[int, ...]
    gknots: List[np.ndarray]
    coefs: np.ndarray  # (ncoef, dim), first parametric direction fastest

    @property
    def ndofs_dir(self) -> Tuple[int, ...]:
        return tuple(len(k) - p - 1 for k, p in zip(self.knots, self.degree))

    @property
    def ndofs(self) -> int:
        return int(np.prod(self.ndofs_dir))

    @property
    def nelems_dir(self) -> Tuple[int, ...]:
        return tuple(int(np.count_nonzero(np.diff(np.unique(k)) > 0)) for k in self.knots)


@dataclasses.dataclass
class Problem:
    dim: int
    patches: List[Patch]
    interfaces: List[Tuple[int, int, int, int]] = dataclasses.field(default_factory=list)
    dirichlet: List[Tuple[int, int]] = dataclasses.field(default_factory=list)
    kappa_fourier: bool = False
    kappa_const: float = 1.0
    kappa_alpha: float = 0.0
    kappa_scale: float = 0.0
    kappa_amp: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    kappa_k: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros((0, 3), dtype=np.int32))
    kappa_phase: np.ndarray = dataclasses.field(default_factory=lambda: np.zeros(0))
    ufreq: int = 1
    quA: float = 1.0
    quB: int = 1
    solver: str = "cg"
    tol: float = 1e-10
    maxit: int = 1000
    mg_levels: int = 4
    mg_npre: int = 2
    mg_npost: int = 2
    mg_damping: float = 0.6
    mg_cycles: int = 1            # gsMultiGridOp "NumCycles" (1 = V-cycle, 2 = W-cycle)
    mg_cgc_damping: float = 1.0   # gsMultiGridOp "CoarseGridCorrectionDamping"
    dirichlet_l2: bool = False    # Dirichlet values by L2 projection (dirichlet::l2Projection)
    # Neumann sides (patch, side), data h = sgn kappa du/dx_k on side s of direction k = (s-1)//2
    # (sgn -1 on the lower side, +1 on the upper): the flux of u where the side is a plane x_k = c
    neumann: List[Tuple[int, int]] = dataclasses.field(default_factory=list)
    name: str = ""

    # ---- closed forms (numpy, used by the generator's checks and by the host tests) ----
    def fields(self, x: np.ndarray):
        """kappa, f, u at physical points x (N x dim)."""
        d = self.dim
        w = self.ufreq * math.pi
        sn = np.sin(w * x)
        cs = np.cos(w * x)
        u = np.prod(sn, axis=1)
        gu = np.empty_like(x)
        for j in range(d):
            t = w * cs[:, j]
            for i in range(d):
                if i != j:
                    t = t * sn[:, i]
            gu[:, j] = t
        if self.kappa_fourier:
            th = self.kappa_phase[None, :] + math.pi * x @ self.kappa_k[:, :d].T.astype(np.float64)
            g = self.kappa_scale * (np.cos(th) @ self.kappa_amp)
            gg = -self.kappa_scale * ((np.sin(th) * self.kappa_amp[None, :]) @ (math.pi * self.kappa_k[:, :d].astype(np.float64)))
            kappa = np.exp(self.kappa_alpha * g)
        else:
            kappa = np.full(len(x), self.kappa_const)
            gg = np.zeros_like(x)
        f = kappa * (d * w * w * u - self.kappa_alpha * np.sum(gg * gu, axis=1))
        return kappa, f, u

    @property
    def total_local_dofs(self) -> int:
        return sum(p.ndofs for p in self.patches)


# ------------------------------------------------------------------------------------------
# geometry construction


def identity_patch(dim: int, n_elem: Sequence[int], p: Sequence[int],
                   lo: Sequence[float] = (0.0, 0.0, 0.0), hi: Sequence[float] = (1.0, 1.0, 1.0)) -> Patch:
    knots = [open_uniform_knots(n_elem[k], p[k]) for k in range(dim)]
    gv = [greville(knots[k], p[k]) for k in range(dim)]
    grids = np.meshgrid(*[lo[k] + (hi[k] - lo[k]) * gv[k] for k in range(dim)], indexing="ij")
    # first direction fastest: flatten in Fortran order over (i0, i1, i2)
    coefs = np.stack([g.ravel(order="F") for g in grids], axis=1)
    return Patch(dim, tuple(p), knots, tuple(p), [k.copy() for k in knots], coefs)


@dataclasses.dataclass
class Displacement:
    amp: float
    k: np.ndarray      # (M, 3) integer wave vectors in {1,2,3}
    phase: np.ndarray  # (M,)
    comp: np.ndarray   # (M,) component index

    def __call__(self, x: np.ndarray) -> np.ndarray:
        d = x.shape[1]
        out = np.zeros_like(x)
        m = len(self.phase)
        th = self.phase[None, :] + math.pi * x @ self.k[:, :d].T.astype(np.float64)
        s = np.sin(th) * (self.amp / m)
        for j in range(m):
            out[:, self.comp[j]] += s[:, j]
        return out


def make_displacement(rng: np.random.Generator, dim: int, amp: float, nmodes: int = 8) -> Displacement:
    k = rng.integers(1, 4, size=(nmodes, 3)).astype(np.int32)
    phase = rng.uniform(0.0, 2.0 * math.pi, size=nmodes)
    comp = rng.integers(0, dim, size=nmodes).astype(np.int32)
    return Displacement(amp, k, phase, comp)


def set_kappa_fourier(prob: Problem, rng: np.random.Generator, nmodes: int, alpha: float = 0.5,
                      scale: float = 0.25, kmax: int = 4) -> None:
    prob.kappa_fourier = True
    prob.kappa_alpha = alpha
    prob.kappa_scale = scale
    prob.kappa_amp = rng.standard_normal(nmodes)
    k = np.zeros((nmodes, 3), dtype=np.int32)
    k[:, :prob.dim] = rng.integers(0, kmax + 1, size=(nmodes, prob.dim))
    prob.kappa_k = k
    prob.kappa_phase = rng.uniform(0.0, 2.0 * math.pi, size=nmodes)


def min_jacobian_det(patch: Patch, quA: float = 1.0, quB: int = 1, slab: int = 16) -> float:
    """Minimum of det(J) of the geometry map over all Gauss points of the patch."""
    d = patch.dim
    pts, Bv, Bd = [], [], []
    for k in range(d):
        kn = patch.knots[k]
        br = np.unique(kn)
        q = int(quA * patch.degree[k] + quB + 0.5)
        xr, _ = gauss_legendre(q)
        gp = ((br[:-1, None] + br[1:, None]) + (br[1:, None] - br[:-1, None]) * xr[None, :]) * 0.5
        gp = gp.ravel()
        pts.append(gp)
        Bv.append(bspline_basis_matrix(patch.gknots[k], patch.gdegree[k], gp, 0))
        Bd.append(bspline_basis_matrix(patch.gknots[k], patch.gdegree[k], gp, 1))
    ng = tuple(len(kn) - p - 1 for kn, p in zip(patch.gknots, patch.gdegree))
    C = patch.coefs.reshape(ng[::-1] + (d,))  # (n_{d-1}, ..., n_0, d)
    if d == 2:
        # C[i1, i0, m]
        J = np.empty((len(pts[1]), len(pts[0]), 2, 2))
        for n in range(2):
            B0 = Bd[0] if n == 0 else Bv[0]
            B1 = Bd[1] if n == 1 else Bv[1]
            J[:, :, :, n] = np.einsum("ai,bj,jim->bam", B0, B1, C, optimize=True)
        det = J[..., 0, 0] * J[..., 1, 1] - J[..., 0, 1] * J[..., 1, 0]
        return float(det.min())
    best = np.inf
    n2 = len(pts[2])
    # stage over direction 0 and 1 once, slab over direction 2
    T = {}
    for a0 in (0, 1):
        B0 = Bd[0] if a0 else Bv[0]
        t0 = np.tensordot(C, B0, axes=([2], [1]))  # (n2, n1, d, Q0)
        for a1 in (0, 1):
            if a0 + a1 > 1:
                continue
            B1 = Bd[1] if a1 else Bv[1]
            T[(a0, a1)] = np.tensordot(t0, B1, axes=([1], [1]))  # (n2, d, Q0, Q1)
    for s0 in range(0, n2, slab):
        s1 = min(n2, s0 + slab)
        J = np.empty((s1 - s0, len(pts[1]), len(pts[0]), 3, 3))
        for n in range(3):
            a = (1 if n == 0 else 0, 1 if n == 1 else 0)
            B2 = (Bd[2] if n == 2 else Bv[2])[s0:s1]
            v = np.tensordot(B2, T[a], axes=([1], [0]))  # (S, d, Q0, Q1)
            J[..., :, n] = np.transpose(v, (0, 3, 2, 1))
        det = (J[..., 0, 0] * (J[..., 1, 1] * J[..., 2, 2] - J[..., 1, 2] * J[..., 2, 1])
               - J[..., 0, 1] * (J[..., 1, 0] * J[..., 2, 2] - J[..., 1, 2] * J[..., 2, 0])
               + J[..., 0, 2] * (J[..., 1, 0] * J[..., 2, 1] - J[..., 1, 1] * J[..., 2, 0]))
        best = min(best, float(det.min()))
    return best


def _displaced(patch: Patch, disp: Optional[Displacement]) -> Patch:
    if disp is None:
        return patch
    c = patch.coefs + disp(patch.coefs)
    return dataclasses.replace(patch, coefs=c)


def all_sides(dim: int) -> List[int]:
    return list(range(1, 2 * dim + 1))


def square_grid_mms(n_elem: int, p: int = 1) -> Problem:
    """The set-up of the reference's gsPoissonSolver_test (unittests/gsPoissonSolver_test.cpp:
    BSplineSquareGrid(2, 2, 0.5), Galerkin with iFace::glue): the unit square as four identity
    patches of side 0.5 (patch 2i + j at (0.5 i, 0.5 j)), Dirichlet on the west sides of patches 0, 1
    and the north sides of 1, 3, Neumann (the exact flux) on the east sides of 2, 3 and the south
    sides of 0, 2; u = sin(pi x) sin(pi y); ``n_elem`` elements per patch and direction."""
    patches = []
    for i in range(2):
        for j in range(2):
            patches.append(identity_patch(2, (n_elem, n_elem), (p, p), lo=(0.5 * i, 0.5 * j), hi=(0.5 * i + 0.5, 0.5 * j + 0.5)))
    ifaces = [(0, SIDE_EAST, 2, SIDE_WEST), (1, SIDE_EAST, 3, SIDE_WEST),
              (0, SIDE_NORTH, 1, SIDE_SOUTH), (2, SIDE_NORTH, 3, SIDE_SOUTH)]
    return Problem(2, patches, interfaces=ifaces,
                   dirichlet=[(0, SIDE_WEST), (1, SIDE_WEST), (1, SIDE_NORTH), (3, SIDE_NORTH)],
                   neumann=[(3, SIDE_EAST), (2, SIDE_EAST), (0, SIDE_SOUTH), (2, SIDE_SOUTH)],
                   name=f"squaregrid_mms_p{p}_n{n_elem}")


def mixed_boundary(prob: Problem) -> Problem:
    """Turn the upper boundary sides (east, north, back) of a problem's Dirichlet list into Neumann
    sides: Dirichlet on the lower sides, Neumann on the upper ones (the gsPoissonSolver_test
    set-up of mixed conditions). Returns the problem."""
    keep, neu = [], []
    for (pt, sd) in prob.dirichlet:
        (neu if side_parameter(sd) == 1 else keep).append((pt, sd))
    prob.dirichlet, prob.neumann = keep, neu
    prob.name = prob.name + "_neu"
    return prob


# ------------------------------------------------------------------------------------------
# the configurations


def square_poisson(n_elem: int = 64, p: int = 2) -> Problem:
    """2D Poisson on the unit square as an identity B-spline map, homogeneous Dirichlet on all
    sides, f = 2 pi^2 sin(pi x) sin(pi y), CG + Jacobi to 1e-10."""
    patch = identity_patch(2, (n_elem, n_elem), (p, p))
    prob = Problem(2, [patch], dirichlet=[(0, s) for s in all_sides(2)], name=f"square_p{p}_n{n_elem}")
    return prob


def displaced_single_patch(dim: int, n_elem: Sequence[int], p: Sequence[int], seed: int, amp: float,
                           kappa_modes: int = 16, ufreq: int = 1, min_det: float = 0.2,
                           check: bool = True) -> Problem:
    """Identity map plus a seeded smooth control-point displacement (8 random-phase sines),
    kappa = exp(0.5 g) with a seeded Fourier field g, manufactured u = prod sin(ufreq pi x_i),
    Dirichlet u on all sides. A draw whose Jacobian determinant drops to ``min_det`` or below at
    any Gauss point is rejected and the next seed is drawn."""
    base = identity_patch(dim, n_elem, p)
    s = seed
    while True:
        rng = np.random.default_rng(s)
        disp = make_displacement(rng, dim, amp)
        patch = _displaced(base, disp)
        if not check or min_jacobian_det(patch) > min_det:
            break
        s += 1_000_003
    prob = Problem(dim, [patch], dirichlet=[(0, sd) for sd in all_sides(dim)], ufreq=ufreq,
                   name=f"disp{dim}d_p{p[0]}_n{n_elem[0]}_s{seed}")
    if kappa_modes > 0:
        set_kappa_fourier(prob, rng, kappa_modes)
    return prob


def volume_poisson(n_elem: int = 64, p: int = 3, seed: int = 1, check: bool = True) -> Problem:
    """3D single volume patch, degree p, n_elem^3 elements, displacement amplitude 0.04,
    16-mode kappa field, Dirichlet u on all sides."""
    return displaced_single_patch(3, (n_elem,) * 3, (p,) * 3, seed, 0.04, kappa_modes=16, check=check)


def patch_batch(count: int = 4096, seed: int = 7, nmin: int = 8, nmax: int = 128,
                check: bool = True) -> List[Problem]:
    """Independent 2D patches of uneven size: degree in {2,3,4}, elements per direction
    log-uniform in [nmin, nmax] per direction, displacement amplitude 0.05, 16-mode kappa,
    u = sin(k pi x) sin(k pi y) with k in {1..4}."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        p = int(rng.integers(2, 5))
        ne = tuple(int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax))))) for _ in range(2))
        k = int(rng.integers(1, 5))
        out.append(displaced_single_patch(2, ne, (p, p), seed * 100003 + i, 0.05, kappa_modes=16,
                                          ufreq=k, check=check))
    return out


def cube_grid(n: int = 8, n_elem: int = 16, p: int = 2, seed: int = 3, amp: float = 0.03,
              kappa_modes: int = 32, check: bool = True) -> Problem:
    """n x n x n conforming cube patches of the unit cube (each degree p with n_elem^3 elements),
    C0 interface coupling, a displacement of the global map evaluated at global coordinates so
    that interfaces stay conforming, kappa from a ``kappa_modes``-mode Fourier field, CG with a
    4-level h-multigrid V-cycle (2+2 damped Jacobi sweeps, omega=0.6)."""
    h = 1.0 / n
    s = seed
    while True:
        rng = np.random.default_rng(s)
        disp = make_displacement(rng, 3, amp)
        patches = []
        for kz in range(n):
            for ky in range(n):
                for kx in range(n):
                    base = identity_patch(3, (n_elem,) * 3, (p,) * 3, lo=(kx * h, ky * h, kz * h),
                                          hi=((kx + 1) * h, (ky + 1) * h, (kz + 1) * h))
                    patches.append(_displaced(base, disp))
        # the determinant criterion is relative to the undisplaced patch map (det = h^3)
        if not check or all(min_jacobian_det(pt) > 0.2 * h ** 3 for pt in patches):
            break
        s += 1_000_003
    idx = lambda x, y, z: (z * n + y) * n + x
    ifaces, dirichlet = [], []
    for kz in range(n):
        for ky in range(n):
            for kx in range(n):
                me = idx(kx, ky, kz)
                if kx + 1 < n:
                    ifaces.append((me, SIDE_EAST, idx(kx + 1, ky, kz), SIDE_WEST))
                if ky + 1 < n:
                    ifaces.append((me, SIDE_NORTH, idx(kx, ky + 1, kz), SIDE_SOUTH))
                if kz + 1 < n:
                    ifaces.append((me, SIDE_BACK, idx(kx, ky, kz + 1), SIDE_FRONT))
                if kx == 0:
                    dirichlet.append((me, SIDE_WEST))
                if kx == n - 1:
                    dirichlet.append((me, SIDE_EAST))
                if ky == 0:
                    dirichlet.append((me, SIDE_SOUTH))
                if ky == n - 1:
                    dirichlet.append((me, SIDE_NORTH))
                if kz == 0:
                    dirichlet.append((me, SIDE_FRONT))
                if kz == n - 1:
                    dirichlet.append((me, SIDE_BACK))
    prob = Problem(3, patches, interfaces=ifaces, dirichlet=dirichlet, solver="mg",
                   name=f"cubegrid{n}_p{p}_n{n_elem}_s{seed}")
    set_kappa_fourier(prob, rng, kappa_modes)
    return prob


def serving_requests(count: int, rate: float, seed: int = 11, check: bool = False, n2d=(16, 256), n3d=(8, 48)):
    """Poisson-process arrivals at ``rate`` req/s; 60 % 2D (``n2d`` elements/dir, log-uniform), 40 % 3D
    (``n3d`` elements/dir), degree in {2,3,4}; geometry and kappa as in the other configs.
    Returns a list of (arrival_time_s, Problem)."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for i in range(count):
        t += rng.exponential(1.0 / rate)
        p = int(rng.integers(2, 5))
        if rng.uniform() < 0.6:
            ne = int(round(math.exp(rng.uniform(math.log(n2d[0]), math.log(n2d[1])))))
            prob = displaced_single_patch(2, (ne, ne), (p, p), seed * 7919 + i, 0.05, check=check)
        else:
            ne = int(round(math.exp(rng.uniform(math.log(n3d[0]), math.log(n3d[1])))))
            prob = displaced_single_patch(3, (ne,) * 3, (p,) * 3, seed * 7919 + i, 0.04, check=check)
        prob.tol = 1e-8
        out.append((t, prob))
    return out


# ------------------------------------------------------------------------------------------
# text spec for the reference driver (oracle/ref/ref_driver.cpp)


def read_spec(text: str) -> Problem:
    """The Problem of a text spec written by :func:`write_spec` (its exact inverse: every number is
    written with repr, so the arrays come back bitwise)."""
    toks = [ln.split() for ln in text.splitlines() if ln.strip()]
    if not toks or toks[0][:2] != ["GSGPU-SPEC", "1"]:
        raise ValueError("not a GSGPU-SPEC 1 text")
    dim = int(toks[1][1])
    i = 2
    patches = []
    prob = Problem(dim, patches)
    modes = 0
    while i < len(toks):
        w = toks[i]
        key = w[0]
        if key == "patch":
            deg = tuple(int(v) for v in toks[i + 1])
            knots = [np.array([float(v) for v in toks[i + 2 + k][1:]]) for k in range(dim)]
            gdeg = tuple(int(v) for v in toks[i + 2 + dim])
            gknots = [np.array([float(v) for v in toks[i + 3 + dim + k][1:]]) for k in range(dim)]
            nc = int(toks[i + 3 + 2 * dim][0])
            rows = toks[i + 4 + 2 * dim:i + 4 + 2 * dim + nc]
            coefs = np.array([[float(v) for v in r] for r in rows], dtype=np.float64).reshape(nc, dim)
            patches.append(Patch(dim, deg, knots, gdeg, gknots, coefs))
            i += 4 + 2 * dim + nc
            continue
        if key == "interface":
            prob.interfaces.append(tuple(int(v) for v in w[1:5]))
        elif key == "dirichlet":
            prob.dirichlet.append((int(w[1]), int(w[2])))
        elif key == "neumann":
            prob.neumann.append((int(w[1]), int(w[2])))
        elif key == "kappa_fourier":
            prob.kappa_fourier = True
            prob.kappa_alpha, prob.kappa_scale, modes = float(w[1]), float(w[2]), int(w[3])
            rows = toks[i + 1:i + 1 + modes]
            prob.kappa_amp = np.array([float(r[0]) for r in rows])
            prob.kappa_k = np.array([[int(r[1]), int(r[2]), int(r[3])] for r in rows], dtype=np.int32).reshape(-1, 3)
            prob.kappa_phase = np.array([float(r[4]) for r in rows])
            i += 1 + modes
            continue
        elif key == "kappa_const":
            prob.kappa_const = float(w[1])
        elif key == "ufreq":
            prob.ufreq = int(w[1])
        elif key == "quad":
            prob.quA, prob.quB = float(w[1]), int(w[2])
        elif key == "dirichlet_values":
            prob.dirichlet_l2 = w[1] == "l2"
        elif key == "solver":
            prob.solver, prob.tol, prob.maxit = w[1], float(w[2]), int(w[3])
        elif key == "mg":
            prob.mg_levels, prob.mg_npre, prob.mg_npost, prob.mg_damping = int(w[1]), int(w[2]), int(w[3]), float(w[4])
        elif key == "mgcycle":
            prob.mg_cycles, prob.mg_cgc_damping = int(w[1]), float(w[2])
        elif key == "end":
            break
        else:
            raise ValueError(f"unknown spec line {key!r}")
        i += 1
    return prob


def write_spec(prob: Problem, path: str) -> None:
    def fmt(v):
        return repr(float(v))

    lines = ["GSGPU-SPEC 1", f"dim {prob.dim}"]
    for pt in prob.patches:
        lines.append("patch")
        lines.append(" ".join(str(int(v)) for v in pt.degree))
        for kn in pt.knots:
            lines.append(f"{len(kn)} " + " ".join(fmt(v) for v in kn))
        lines.append(" ".join(str(int(v)) for v in pt.gdegree))
        for kn in pt.gknots:
            lines.append(f"{len(kn)} " + " ".join(fmt(v) for v in kn))
        lines.append(str(len(pt.coefs)))
        for row in pt.coefs:
            lines.append(" ".join(fmt(v) for v in row))
    for f in prob.interfaces:
        lines.append("interface " + " ".join(str(int(v)) for v in f))
    for dsd in prob.dirichlet:
        lines.append(f"dirichlet {dsd[0]} {dsd[1]}")
    for nsd in prob.neumann:
        lines.append(f"neumann {nsd[0]} {nsd[1]}")
    if prob.kappa_fourier:
        lines.append(f"kappa_fourier {fmt(prob.kappa_alpha)} {fmt(prob.kappa_scale)} {len(prob.kappa_amp)}")
        for a, k, ph in zip(prob.kappa_amp, prob.kappa_k, prob.kappa_phase):
            lines.append(f"{fmt(a)} {int(k[0])} {int(k[1])} {int(k[2])} {fmt(ph)}")
    else:
        lines.append(f"kappa_const {fmt(prob.kappa_const)}")
    lines.append(f"ufreq {prob.ufreq}")
    lines.append(f"quad {fmt(prob.quA)} {prob.quB}")
    if prob.dirichlet_l2:
        lines.append("dirichlet_values l2")
    lines.append(f"solver {prob.solver} {fmt(prob.tol)} {prob.maxit}")
    lines.append(f"mg {prob.mg_levels} {prob.mg_npre} {prob.mg_npost} {fmt(prob.mg_damping)}")
    if prob.mg_cycles != 1 or prob.mg_cgc_damping != 1.0:
        lines.append(f"mgcycle {prob.mg_cycles} {fmt(prob.mg_cgc_damping)}")
    lines.append("end")
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")
