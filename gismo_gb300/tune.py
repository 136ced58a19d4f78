"""Tuning run: gsgpu_autotune on representative problems of the benchmark configurations, then
the table written to a file (by default gismo_gb300/tuning.txt, which the library loads).

    python -m gismo_gb300.tune [--out PATH]

Keys are (kernel group, dimension, degree, Gauss points); the problems below cover the degrees
2-4 of the volume, batch and multigrid configurations at sizes large enough (working sets above
the 126 MB L2) for the timings to be representative."""
from __future__ import annotations

import argparse
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def problems():
    from . import problems as P
    out = []
    for p in (2, 3, 4):
        out.append((f"volume_p{p}", P.volume_poisson({2: 72, 3: 64, 4: 48}[p], p, seed=1, check=False)))
    for p in (2, 3, 4):
        out.append((f"square_p{p}", P.displaced_single_patch(2, (512, 512), (p, p), 3, 0.05, check=False)))
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "tuning.txt"))
    args = ap.parse_args(argv)
    from .assembler import GpuPoissonAssembler, tune_clear, tune_save
    tune_clear()
    for name, prob in problems():
        A = GpuPoissonAssembler(prob, device=0)
        ms = A.autotune()
        print(name, "stiffness ms", [round(float(v), 3) for v in ms[:6]], "inner ms", [round(float(v), 4) for v in ms[6:]],
              "variants", A.tuned_variants(), flush=True)
        A.close()
    tune_save(args.out)
    print("wrote", args.out)
    return 0


if __name__ == "__main__":
    sys.exit(main())
