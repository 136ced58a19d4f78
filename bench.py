#!/usr/bin/env python3
"""Benchmark: assembled + solved DoF/s of the isogeometric Poisson / diffusion path on one GB300.

Workload (the configuration the headline metric is quoted on, fits one GPU): 3D single volume
patch, degree 3, 64^3 uniform elements (274,625 free dofs, 86,938,307 non-zeros), 4^3 Gauss
points, identity map plus a seeded smooth control-point displacement (amplitude 0.04), diffusion
kappa = exp(0.5 g) with a seeded 16-mode Fourier field, manufactured u = prod sin(pi x_i),
Dirichlet u on all sides. A step is one assemble() + one solve() to 1e-10 relative residual through
the C ABI. Headline (--mode mixed): double-float (two-FP32) assembly, FP32 CG + Jacobi inner
iteration with FP64-accurate residual replacement; the plain FP64 path (FP64 assembly, FP64
CG + Jacobi) is timed in the same run, and the mixed solution is checked against a tightly
converged (1e-13) FP64 solution: relative 2-norm error must stay <= 1e-8.

  value  device-resident inputs (control points already in HBM), solution left on the device
  e2e    per step: control points host->device from pinned memory, assemble, solve, solution
         device->host into pinned memory
The working set (coefficient fields, contraction intermediates, CSR) is several GB, far larger
than the 126 MB L2, so no extra L2 flush is done between steps.

--impl reference times the reference algorithm's CPU implementation (the oracle port of G+Smo's
OpenMP assembler + CG) on the same workload with all host threads, every step a whole assemble +
solve (no sampling, no scaling).
Under torchrun with N GPUs each rank runs an independent replica (no data exchange).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "assembled+solved DoF/s @1e-8 rel err vs plain FP64 GPU; p50/p99 latency"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--p", type=int, default=3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="volume", choices=["volume", "batch", "multigrid", "serving"],
                    help="volume: the headline configuration; the others are in gismo_gb300/bench_workloads.py")
    ap.add_argument("--mg-damping", type=float, default=0.5)
    ap.add_argument("--mg-grid", type=int, default=8, help="multigrid workload: patches per direction")
    ap.add_argument("--mg-elems", type=int, default=16, help="multigrid workload: elements per patch and direction")
    ap.add_argument("--requests", type=int, default=200)
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            if len(r) < 9:
                continue
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def workload(args):
    from gismo_gb300 import problems as P
    return P.volume_poisson(args.n, args.p, seed=args.seed)


def config(args, nfree, nnz, extra=None):
    c = {"workload": f"volume_poisson_p{args.p}_{args.n}^3", "dim": 3, "degree": args.p, "elements": args.n ** 3,
         "free_dofs": nfree, "nnz": nnz, "gauss_points_per_dir": args.p + 1, "kappa": "exp(0.5 g), 16-mode Fourier",
         "solver": "CG+Jacobi", "tol": args.tol, "precision": args.mode,
         "l2_flush": "none needed: per-step working set (fields, intermediates, CSR) is several GB > L2"}
    if extra:
        c.update(extra)
    return c


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(kernel: str):
    """dram bytes per launch of the roofline kernel from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as fh:
            return json.load(fh).get(kernel)
    except Exception:
        return None


def cpu_full_step(o, tol: float, nthreads: int):
    """One whole step of the reference algorithm on the host: every element assembled by the
    OpenMP element loop with the serialised scatter (gsAssembler::apply, gsAssembler.h:666-722),
    then CG + Jacobi to `tol` (gsConjugateGradient, gsConjugateGradient.hpp:19-84; single-threaded
    like the reference's Eigen SpMV). Returns (wall seconds, assembly s, solve s, iterations)."""
    t0 = time.perf_counter()
    t_asm = o.assemble(nthreads)
    _, it, _, t_cg = o.solve_cg(tol, 1000)
    return time.perf_counter() - t0, t_asm, t_cg, it


def cpu_baseline(prob, tol: float, nthreads: int):
    """The oracle port of the reference algorithm on the host cores, one whole step (no sampling,
    no scaling): the symbolic set-up once untimed (as refresh() is on the GPU), then one timed
    assemble + solve of the full workload."""
    from oracle import oracle as O
    o = O.OracleProblem(prob)
    o.assemble(nthreads, 0)  # symbolic pattern and Dirichlet set-up, untimed
    wall, t_asm, t_cg, it = cpu_full_step(o, tol, nthreads)
    nfree = o.sizes()[0]
    return {"value": nfree / wall, "unit": "DoF/s", "cores": nthreads, "kind": "port",
            "cpu": cpu_model(),
            "sample": f"one whole step: all {int(np.prod(prob.patches[0].nelems_dir))} elements assembled (OpenMP element "
                      f"loop, serialised scatter) in {t_asm:.1f} s + CG+Jacobi to {tol:g} on the full {nfree}-dof matrix, "
                      f"{it} iterations in {t_cg:.1f} s (single-threaded, as the reference's Eigen SpMV); "
                      f"wall {wall:.1f} s; symbolic set-up excluded"}


def cpu_model() -> str:
    try:
        with open("/proc/cpuinfo") as fh:
            for line in fh:
                if line.lower().startswith(("model name", "cpu part", "hardware")):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.machine()


def run_reference(args):
    """The reference algorithm's CPU implementation (the oracle port: the reference itself is built
    only where its sources are, not on the GPU machine) on the same workload, every step a whole
    assemble + solve, timed on the wall clock with all host threads."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    prob = workload(args)
    nthreads = os.cpu_count() or 1
    from oracle import oracle as O
    o = O.OracleProblem(prob)
    o.assemble(nthreads, 0)  # symbolic set-up once, untimed
    times, its, asm, cg = [], [], [], []
    for k in range(args.warmup + args.steps):
        wall, t_asm, t_cg, it = cpu_full_step(o, args.tol, nthreads)
        if k >= args.warmup:
            times.append(wall)
            its.append(it)
            asm.append(t_asm)
            cg.append(t_cg)
    nfree, nnz, _, _ = o.sizes()
    total = float(np.sum(times))
    value = nfree * len(times) / total
    cfg = config(args, nfree, nnz, {"precision": "fp64 (the reference algorithm on the host)"})
    line = {"metric": METRIC, "value": value, "unit": "DoF/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total / len(times) * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator, same inputs as --impl ours)",
            "impl": "reference", "config": cfg,
            "cpu_baseline": {"value": value, "unit": "DoF/s", "cores": nthreads, "kind": "port", "cpu": cpu_model(),
                             "sample": f"every step the whole workload: all {args.n ** 3} elements assembled by the "
                                       f"OpenMP element loop with serialised scatter (mean {np.mean(asm):.1f} s), CG+Jacobi "
                                       f"to {args.tol:g} (iterations {min(its)}-{max(its)}, mean {np.mean(cg):.1f} s, "
                                       f"single-threaded like the reference's Eigen SpMV); wall-clock time per step"},
            "e2e": {"value": value, "unit": "DoF/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.workload != "volume" and args.impl == "ours":
        from gismo_gb300 import bench_workloads as BW
        import __graft_entry__ as g
        g.build()
        fn = {"batch": BW.run_batch, "multigrid": BW.run_multigrid, "serving": BW.run_serving}[args.workload]
        return fn(args, lambda: ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))))
    if args.impl == "reference":
        return run_reference(args)
    ws, rank, local = dist_env()
    import torch
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from gismo_gb300.assembler import GpuPoissonAssembler
    from gismo_gb300 import replicas as R

    args.seed = R.replica_seed(args.seed, rank)  # independent replica per rank
    prob = workload(args)
    A = GpuPoissonAssembler(prob, device=local)
    nfree, nnz, _, _ = A.sizes()
    stream = torch.cuda.ExternalStream(A.stream_handle(), device=torch.device("cuda", local))

    def step(download=None):
        A.assemble(args.mode)
        x, info = A.solve(tol=args.tol, precision=args.mode, download=download is not None)
        return x, info

    for _ in range(max(3, args.warmup)):
        _, info = step()
    gpu_iters = info["iterations"]

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    # ---- device-resident timing ----
    clk = ClockSampler(local)
    barrier()
    clk.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    infos = []
    asm_ms = []
    for _ in range(args.steps):
        _, info = step()
        infos.append(info)
        asm_ms.append(A.assemble_times())
    e1.record(stream)
    e1.synchronize()
    t_ms = e0.elapsed_time(e1)
    barrier()
    clocks = clk.stop()
    # slowest rank's time, dofs of all ranks' replicas
    t_ms, units = R.reduce_max_sum(dist, t_ms, nfree, "cuda")
    ms_per_step = t_ms / args.steps
    value = units / (ms_per_step * 1e-3)

    # ---- the plain FP64 path on the same workload, and the accuracy of the headline path ----
    fp64_line = None
    err_vs_fp64 = None
    if args.mode == "mixed":
        A.assemble("fp64")
        x_ref, info_ref = A.solve(tol=1e-13, max_iters=20000)
        A.assemble("mixed")
        x_m, info_m = A.solve(tol=args.tol, precision="mixed")
        err_vs_fp64 = float(np.linalg.norm(x_m - x_ref) / np.linalg.norm(x_ref))
        for _ in range(2):
            A.assemble("fp64")
            A.solve(tol=args.tol, download=False)
        barrier()
        g0 = torch.cuda.Event(enable_timing=True)
        g1 = torch.cuda.Event(enable_timing=True)
        g0.record(stream)
        fp_infos = []
        fp_asm = []
        for _ in range(args.steps):
            A.assemble("fp64")
            fp_asm.append(A.assemble_times())
            _, fi = A.solve(tol=args.tol, download=False)
            fp_infos.append(fi)
        g1.record(stream)
        g1.synchronize()
        t64 = g0.elapsed_time(g1) / args.steps
        fa = np.mean(np.array(fp_asm), axis=0)
        fp64_line = {"value": ws * nfree / (t64 * 1e-3), "unit": "DoF/s", "ms_per_step": t64,
                     "iterations": fp_infos[-1]["iterations"], "speedup_mixed_over_fp64": t64 / ms_per_step,
                     "t_solve_ms": float(np.mean([f["t_solve_ms"] for f in fp_infos])),
                     "assemble_ms": {"geometry_fields": fa[2], "stiffness": fa[3], "load": fa[4],
                                     "scatter": fa[5], "total": fa[6]}}
        for _ in range(2):
            step()

    # ---- end to end through the C ABI with pinned host buffers ----
    coefs_h = torch.from_numpy(np.ascontiguousarray(prob.patches[0].coefs, np.float64).ravel()).pin_memory()
    x_h = torch.empty(nfree, dtype=torch.float64).pin_memory()
    xv = x_h.numpy()

    def e2e_step():
        A.set_coefs(coefs_h.numpy())
        A.assemble(args.mode)
        _, info = A.solve(tol=args.tol, precision=args.mode, out=xv)  # straight into pinned memory
        return info

    for _ in range(max(3, args.warmup)):
        e2e_step()
    import gc
    gc.collect()
    gc.disable()  # no collector pause inside the timed host loop
    barrier()
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    lat = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        e2e_step()
        lat.append((time.perf_counter() - t0) * 1e3)
    f1.record(stream)
    f1.synchronize()
    gc.enable()
    te_ms = f0.elapsed_time(f1)
    barrier()
    te_ms, units = R.reduce_max_sum(dist, te_ms, nfree, "cuda")
    e2e_value = units / (te_ms / args.steps * 1e-3)

    # ---- roofline of the dominant HBM kernel: the CG SpMV, timed per launch with events ----
    A.set_profiling(True)
    A.solve(tol=args.tol, precision=args.mode, download=False)
    nl, sp_ms, sp_bytes = A.spmv_stats()
    A.set_profiling(False)
    peak, peak_kind = measured_peak()
    achieved = sp_bytes / (sp_ms / nl * 1e-3) / 1e9 if nl else None
    nh = 1 + ((2 * args.p + 1) ** 3 - 1) // 2
    if args.mode == "mixed" and sp_bytes == nh * nfree * 4 + 8 * nfree:
        inner = A.tuned_variants()[2]
        kbase = {0: "k_sdia32_dot", 1: "k_sdia32_tma", 2: "k_sdia32_g4"}.get(inner, "k_sdia32_dot")
        traffic = profiled_traffic(kbase + "_volume_p3_64")
        kname = (kbase + " (FP32 inner operator in half-diagonal storage: the lexicographically "
                 "non-negative half of the 7^3 neighbour box as 172 diagonals, each stored value read by "
                 "its row and by its mirror row; " + ("four rows per thread, 16-byte loads; " if inner == 2 else "")
                 + "+ block partials of p.Ap)")
    elif args.mode == "mixed":
        traffic = profiled_traffic("k_spmv32_dot_volume_p3_64")
        kname = ("k_spmv32_dot (CSR SpMV + p.Ap of the FP32 inner operator; box rows take their column "
                 "offsets from shared memory, the other rows int16 offsets)")
    else:
        traffic = profiled_traffic("k_spmv_dot_fp64_volume_p3_64")
        kname = "k_spmv_dot (CSR SpMV + p.Ap, FP64 values)"
    roofline = {"kernel": kname, "bound": "hbm",
                "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak if achieved else None, "peak_source": peak_kind,
                "traffic": traffic, "algorithmic_bytes_per_launch": sp_bytes, "launches_timed": nl,
                "avg_launch_ms": sp_ms / nl if nl else None}

    it = infos[-1]["iterations"]
    chunks = math.ceil(it / 16) + 1 if it else 1
    if args.mode == "mixed" and kname.startswith("k_sdia32"):
        # counted in the launch list of one step (profiles/launches_volume_p3_64_mixed.md): assemble 24
        # (basis 2, pair 1, to_df 3, geo 2, point 1, contraction 9 with the tuned stage-2 width, load 3,
        # gather 1, half-diagonal build 1, rhs 1); solve: dinv 1, init 2, per graph chunk 16 x 4 iteration
        # kernels (product, alpha, update with beta, direction) + 5 replacement kernels; 12 chunks for
        # 155 iterations with 5 replacements
        chunks = math.ceil(it / 16) + 2 if it else 1
        launches_per_step = 24 + 3 + (16 * 4 + 5) * chunks
    elif args.mode == "mixed":
        # assemble: basis 2, pair 1, to_df 2, geo 2, point 1, contraction 7 (stage 1: two tile
        # launches + two boundary-row launches; stage 2: interior + boundary rows; stage 3), load 3,
        # gather 1, rhs 1; solve: dinv 1, init 2, per graph chunk 16 x 5 iteration kernels + 5
        # replacement kernels
        launches_per_step = 20 + 3 + (16 * 5 + 5) * chunks
    else:
        # assemble 13; solve: dinv 1, init 2, per graph chunk 16 x 3 iteration kernels (alpha and beta
        # are formed by the last block of the SpMV and of the update)
        launches_per_step = 13 + 3 + 3 * 16 * chunks
    amean = np.mean(np.array(asm_ms), axis=0)
    line = {"metric": METRIC, "value": value, "unit": "DoF/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.mode == "fp64" else "f32+f64",
            "data": "synthetic (seeded generator: displacement, kappa field, manufactured solution)",
            "config": config(args, nfree, nnz),
            "e2e": {"value": e2e_value, "unit": "DoF/s", "h2d_bytes_per_step": int(coefs_h.numel() * 8),
                    "d2h_bytes_per_step": int(nfree * 8), "latency_ms_p50": float(np.percentile(lat, 50)),
                    "latency_ms_p99": float(np.percentile(lat, 99))},
            "roofline": roofline, "clocks": clocks, "gpu_launches": launches_per_step * args.steps,
            "solve": {"iterations": it, "relres": infos[-1]["relres"], "t_solve_ms": infos[-1]["t_solve_ms"],
                      "residual_replacements": infos[-1]["refinements"]},
            "rel_err_vs_fp64": err_vs_fp64, "plain_fp64": fp64_line,
            "assemble_ms": {"dirichlet_host": amean[0], "basis": amean[1], "geometry_fields": amean[2],
                            "stiffness": amean[3], "load": amean[4], "scatter": amean[5], "total": amean[6]}}
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(prob, args.tol, os.cpu_count() or 1)
    if rank == 0:
        print(json.dumps(line), flush=True)
    A.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
