"""Checkpoint / resume of a problem, its assembled system and its solution: one compressed .npz
holding the problem as its text spec (problems.write_spec / read_spec, bitwise round trip) and
any of the CSR arrays, rhs, eliminated-dof values, solution and solver figures. The reference
has no solver checkpoints; gsFileData::save stores XML (for the patches alone, gismo_gb300.xmlio
writes and reads that format)."""
from __future__ import annotations

import os
import tempfile
from typing import Dict, Optional, Tuple

import numpy as np

from . import problems as P

_ARRAYS = ("csr_ptr", "csr_col", "csr_val", "rhs", "ddof", "x")


def save_state(path: str, prob: "P.Problem", **arrays) -> None:
    """Write the problem and the given arrays (csr_ptr, csr_col, csr_val, rhs, ddof, x) and scalars
    (e.g. iterations, relres) to ``path`` (.npz), atomically (a temporary file renamed into place)."""
    with tempfile.TemporaryDirectory() as td:
        spec = os.path.join(td, "spec.txt")
        P.write_spec(prob, spec)
        with open(spec) as fh:
            text = fh.read()
    out = {"spec": np.array(text)}
    for k, v in arrays.items():
        if v is None:
            continue
        out[k] = np.asarray(v)
    d = os.path.dirname(os.path.abspath(path))
    fd, tmp = tempfile.mkstemp(suffix=".npz", dir=d)
    os.close(fd)
    try:
        np.savez_compressed(tmp, **out)
        os.replace(tmp, path)
    finally:
        if os.path.exists(tmp):
            os.remove(tmp)


def load_state(path: str) -> Tuple["P.Problem", Dict[str, np.ndarray]]:
    """The problem and the stored arrays / scalars of a checkpoint written by :func:`save_state`."""
    with np.load(path, allow_pickle=False) as z:
        prob = P.read_spec(str(z["spec"]))
        rest = {k: z[k] for k in z.files if k != "spec"}
    return prob, rest


def save_assembler(path: str, A, x: Optional[np.ndarray] = None, info: Optional[dict] = None) -> None:
    """Checkpoint of a GpuPoissonAssembler after assemble() (and optionally a solve): its problem,
    CSR system, rhs, eliminated-dof values and the solution with its iteration count / residual."""
    ptr, col, val = A.csr()
    extra = {}
    if info is not None:
        extra = {"iterations": np.int64(info.get("iterations", -1)), "relres": np.float64(info.get("relres", np.nan))}
    save_state(path, A.prob, csr_ptr=ptr, csr_col=col, csr_val=val, rhs=A.rhs(), ddof=A.fixedDofs(), x=x, **extra)
