"""Runs the reference libcugpe engine (built by build_ref.py) on given inputs.

TEST INFRASTRUCTURE ONLY: used by the GPU parity tests, the golden-vector
generator and the reference timing.  Needs a CUDA device.
"""
from __future__ import annotations

import os
import subprocess
import tempfile

import numpy as np

from . import build_ref


def available() -> bool:
    return build_ref.prepare()


def run(shape, interactions, alpha, beta, dt, npart, params, psi0, cmds, qf=0.0, timeout=600, vext=0):
    """Executes `cmds` (see oracle/ref_runner.cpp) and returns the parsed results.

    Returns dict with 'psi' (list of dumps), 'energy' (list of (t, ekin, eint, eext)),
    'mu' (list), 'time_ms' (list).
    """
    nx, ny, nz = shape
    exe = build_ref.build_one(nx, ny, nz, interactions, vext=vext)
    p = list(params) + [0.0] * (4 - len(params))
    with tempfile.TemporaryDirectory() as d:
        inp = os.path.join(d, "psi0.bin")
        np.ascontiguousarray(psi0, dtype=np.complex128).tofile(inp)
        args = [exe, inp, d, repr(float(alpha)), repr(float(beta)), repr(float(dt)), repr(float(npart)),
                repr(float(qf)), *[repr(float(x)) for x in p[:4]], ",".join(cmds)]
        r = subprocess.run(args, capture_output=True, text=True, timeout=timeout)
        if r.returncode != 0:
            raise RuntimeError(f"reference run failed ({r.returncode}): {r.stderr[-2000:]}")
        out = {"psi": [], "energy": [], "mu": [], "time_ms": [], "t": [], "currents": [], "edip": []}
        for line in r.stdout.splitlines():
            f = line.split()
            if not f:
                continue
            if f[0] == "E":
                out["energy"].append(tuple(float(x) for x in f[1:5]))
            elif f[0] == "W":
                out["edip"].append(float(f[2]))
            elif f[0] == "MU":
                out["mu"].append(float(f[1]))
            elif f[0] == "TIME":
                out["time_ms"].append(float(f[1]))
            elif f[0] == "D":
                out["t"].append(float(f[1]))
        k = 0
        while os.path.isfile(os.path.join(d, f"psi_{k}.bin")):
            out["psi"].append(np.fromfile(os.path.join(d, f"psi_{k}.bin"), dtype=np.complex128).reshape(shape))
            k += 1
        k = 0
        while os.path.isfile(os.path.join(d, f"cur_{k}.bin")):
            j = np.fromfile(os.path.join(d, f"cur_{k}.bin"), dtype=np.float64).reshape((3,) + tuple(shape))
            out["currents"].append((j[0], j[1], j[2]))
            k += 1
        return out
