"""Generate the golden parity fixtures from the G+Smo reference itself.

Builds the reference's own FP64 assembler/solver from its sources (oracle/ref/Makefile, output in
oracle/_ref/), runs it on seeded problems from gismo_gb300.problems and stores what it returns
(dof map, CSC matrix, rhs, eliminated-dof values, solution, iterations, L2 error, H1 seminorm error, and the
mass matrix of gsGenericAssembler::assembleMass with the same boundary conditions) as compressed
.npz files next to this script. Run from the repository root, in a container that has the G+Smo
source tree:

    python tests/golden/make_golden.py --ref /path/to/gismo

The fixtures are committed; the GPU tests only read them.
"""
from __future__ import annotations

import argparse
import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from gismo_gb300 import problems as P  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def cases():
    """name -> Problem. Kept small so the fixtures stay a few MB in total."""
    out = {}
    out["square_p2_n4"] = P.square_poisson(4, 2)
    out["square_p2_n64"] = P.square_poisson(64, 2)  # the reference's CPU-runnable config, full size
    pr = P.displaced_single_patch(2, (7, 9), (3, 2), 5, 0.05, ufreq=2)
    out["disp2d_p3x2_7x9"] = pr
    pr = P.displaced_single_patch(2, (12, 10), (4, 4), 17, 0.05, ufreq=3)
    out["disp2d_p4_12x10"] = pr
    out["disp3d_p232_4x5x6"] = P.displaced_single_patch(3, (4, 5, 6), (2, 3, 2), 5, 0.04)
    out["disp3d_p3_8"] = P.volume_poisson(8, 3, seed=1)
    pr = P.cube_grid(n=2, n_elem=4, p=2, seed=3, kappa_modes=8)
    pr.mg_levels = 3
    pr.tol = 1e-8
    out["cubegrid2_p2_n4_mg"] = pr
    pr = P.displaced_single_patch(2, (32, 24), (2, 2), 9, 0.05, ufreq=2)
    pr.solver = "mg"
    pr.mg_levels, pr.mg_cycles, pr.mg_cgc_damping = 4, 2, 0.8  # W-cycle, damped coarse correction
    pr.tol = 1e-8
    out["disp2d_p2_32x24_mgw"] = pr
    pr = P.displaced_single_patch(3, (4, 5, 3), (2, 3, 2), 7, 0.04, ufreq=2)
    pr.dirichlet_l2 = True  # dirichlet::l2Projection
    out["disp3d_p232_4x5x3_l2dir"] = pr
    pr = P.cube_grid(n=2, n_elem=3, p=2, seed=4, kappa_modes=8)
    pr.dirichlet_l2 = True
    out["cubegrid2_p2_n3_l2dir"] = pr
    pr = P.cube_grid(n=2, n_elem=4, p=2, seed=3, kappa_modes=8)
    pr.solver = "cg"
    pr.tol = 1e-8
    out["cubegrid2_p2_n4_cg"] = pr
    # mixed boundary conditions: Dirichlet on the lower sides, Neumann (gsVisitorNeumann) on the
    # upper ones
    out["square_p2_n16_neu"] = P.mixed_boundary(P.square_poisson(16, 2))
    out["disp2d_p3_10x8_neu"] = P.mixed_boundary(P.displaced_single_patch(2, (10, 8), (3, 3), 21, 0.05, ufreq=2))
    out["disp3d_p232_4x5x3_neu"] = P.mixed_boundary(P.displaced_single_patch(3, (4, 5, 3), (2, 3, 2), 8, 0.04))
    pr = P.mixed_boundary(P.cube_grid(n=2, n_elem=3, p=2, seed=6, kappa_modes=8))
    pr.solver = "cg"
    pr.tol = 1e-8
    out["cubegrid2_p2_n3_neu"] = pr
    return out


def large_cases():
    """name -> Problem at the benchmark's sizes. The full matrices (87M non-zeros at 64^3) are too
    large to commit: these fixtures keep the reference's scalars (sizes, CG iterations, residual,
    L2 and H1 errors), every SAMPLE-th entry of its solution, rhs and diagonal, the norms of its
    rhs and solution, and the SHA-256 of the problem's spec text."""
    out = {}
    # the headline shape (3D, p=3, 64^3) with kappa = 1 on the undisplaced unit cube
    cube = P.Problem(3, [P.identity_patch(3, (64, 64, 64), (3, 3, 3))],
                     dirichlet=[(0, s) for s in P.all_sides(3)], name="cube_p3_n64")
    out["large_cube_p3_n64"] = cube
    # the headline configuration itself (displacement 0.04, 16-mode kappa field), and at 32^3
    out["large_vol_p3_n64_s1"] = P.volume_poisson(64, 3, seed=1)
    out["large_vol_p3_n32_s1"] = P.volume_poisson(32, 3, seed=1)
    return out


SAMPLE = 97


def run_reference(exe: str, prob, workdir: str) -> dict:
    spec = os.path.join(workdir, "spec.txt")
    P.write_spec(prob, spec)
    subprocess.check_call([exe, spec, workdir])
    ld = lambda n, t: np.fromfile(os.path.join(workdir, n), dtype=t)
    info = dict(line.split() for line in open(os.path.join(workdir, "info.txt")))
    with open(spec) as fh:
        spec_text = fh.read()
    extra = {}
    if os.path.exists(os.path.join(workdir, "mass_val.f64")):  # gsGenericAssembler::assembleMass
        extra = dict(mass_ptr=ld("mass_ptr.i32", np.int32), mass_idx=ld("mass_idx.i32", np.int32),
                     mass_val=ld("mass_val.f64", np.float64))
    return dict(**extra,
        dofmap=ld("dofmap.i32", np.int32), csc_ptr=ld("csc_ptr.i32", np.int32), csc_idx=ld("csc_idx.i32", np.int32),
        csc_val=ld("csc_val.f64", np.float64), rhs=ld("rhs.f64", np.float64), ddof=ld("ddof.f64", np.float64),
        x=ld("x.f64", np.float64), free=np.int64(info["free"]), nnz=np.int64(info["nnz"]),
        iters=np.int64(info["iters"]), relres=np.float64(info["error"]), l2=np.float64(info["l2"]),
        h1=np.float64(info["h1"]),
        spec=np.array(spec_text),
    )


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("GISMO_REF", ""))
    ap.add_argument("--only", default="")
    args = ap.parse_args()
    mk = ["make", "-C", os.path.join(ROOT, "oracle", "ref"), "-j8"]
    if args.ref:
        mk.append(f"REF={args.ref}")
    subprocess.check_call(mk)
    exe = os.path.join(ROOT, "oracle", "_ref", "gsref")
    for name, prob in cases().items():
        if args.only and name != args.only:
            continue
        with tempfile.TemporaryDirectory() as td:
            res = run_reference(exe, prob, td)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
        print(name, "free", int(res["free"]), "nnz", int(res["nnz"]), "iters", int(res["iters"]), "l2", float(res["l2"]))
    for name, prob in large_cases().items():
        if args.only and name != args.only:
            continue
        with tempfile.TemporaryDirectory() as td:
            res = run_reference(exe, prob, td)
        keep = {k: res[k] for k in ("free", "nnz", "iters", "relres", "l2", "h1")}
        res.pop("mass_ptr", None), res.pop("mass_idx", None), res.pop("mass_val", None)
        # the spec text of a 64^3 displaced patch is tens of MB: keep its digest, the tests rebuild
        # the problem with large_cases() and compare digests
        keep["spec_sha256"] = np.array(hashlib.sha256(str(res["spec"]).encode()).hexdigest())
        keep["sample"] = np.int64(SAMPLE)
        keep["x_sample"] = res["x"][::SAMPLE]
        keep["rhs_sample"] = res["rhs"][::SAMPLE]
        keep["rhs_norm"] = np.float64(np.linalg.norm(res["rhs"]))
        keep["x_norm"] = np.float64(np.linalg.norm(res["x"]))
        keep["diag_sample"] = _csc_diagonal(res)[::SAMPLE]
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **keep)
        print(name, "free", int(res["free"]), "nnz", int(res["nnz"]), "iters", int(res["iters"]), "l2", float(res["l2"]),
              flush=True)


def _csc_diagonal(res) -> np.ndarray:
    """Diagonal of the reference's compressed ColMajor matrix."""
    ptr, idx, val = res["csc_ptr"], res["csc_idx"], res["csc_val"]
    n = len(ptr) - 1
    colof = np.repeat(np.arange(n, dtype=np.int64), np.diff(ptr))
    on = idx == colof
    d = np.zeros(n)
    d[colof[on]] = val[on]
    return d


if __name__ == "__main__":
    main()
