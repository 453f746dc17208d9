"""A seeded FP32-mixed run on any lattice, for kernel profilers.

    python -m libcugpe_gb300.profile_case --lattice 512,512,128 --warm 3 --steps 1

Unitary Fermi gas, quantum friction 0.1, real time, a random seeded state:
`--warm` steps (the first step runs 8 fused passes, every later one 7), then
`--steps` more, so that `ncu -k regex:pass_kernel -s 7*warm+1 -c 7*steps`
captures whole steady steps.  Prints the wall time of the measured
steps; it is not a benchmark (see bench.py).
"""
from __future__ import annotations

import argparse
import time

import libcugpe_gb300 as g
from libcugpe_gb300 import configs


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--lattice", default="512,512,128")
    ap.add_argument("--warm", type=int, default=3)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    args = ap.parse_args(argv)
    shape = tuple(int(x) for x in args.lattice.split(","))
    e = g.Engine(shape, 0, 1.0, 0.0, 0.02, 1e5, precision=g.FP32 if args.precision == "fp32" else g.FP64)
    e.set_user_params([0.002, 0.002, 0.003, 0.0])
    e.set_quantum_friction_coeff(0.1)
    e.set_psi(0.0, configs.random_state(shape, seed=3, npart=1e5, gamma=2.0))
    e.evolve_qf(args.warm)
    e.synchronize()
    t0 = time.perf_counter()
    e.evolve_qf(args.steps)
    e.synchronize()
    print(f"{shape} {args.precision}: {args.steps} steps in {time.perf_counter() - t0:.4f} s")
    e.close()


if __name__ == "__main__":
    main()
