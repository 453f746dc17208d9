"""Records golden vectors from the reference libcugpe engine.

Runs on a machine with a GPU and the edited reference sources
(oracle/build_ref.py).  For each case it builds the reference for the
lattice/functional, feeds it a seeded state (libcugpe_gb300.configs.random_state)
and stores the reference's own wavefunction after each checkpoint, its
chemical potential and its energies:

    python tests/golden/make_golden.py      # writes tests/golden/<case>.{json,npz}

The CPU oracle is pinned against these files (tests/test_oracle.py).
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from libcugpe_gb300 import configs  # noqa: E402
from oracle import ref_run  # noqa: E402

CASES = [
    # name, shape, interactions, alpha, beta, dt, npart, params, qf, steps per checkpoint, seed
    ("bec_ite_16", (16, 16, 16), -1, 0.0, 1.0, 0.05, 1.0, [0.0625, 0.0625, 0.0625, 31.83], 0.0, [1, 6], 1),
    ("bec_rte_32x16x8", (32, 16, 8), -1, 1.0, 0.0, 0.05, 1.0, [0.0625, 0.05, 0.07, 31.83], 0.0, [1, 9], 2),
    ("ufg_rte_qf_16", (16, 16, 16), 0, 1.0, 0.0, 0.05, 1000.0, [0.04, 0.04, 0.06, 0.0], 0.1, [1, 6], 3),
    ("ufg_ite_qf_8x32x16", (8, 32, 16), 0, 0.0, 1.0, 0.05, 1000.0, [0.04, 0.04, 0.06, 0.0], 0.1, [1, 6], 4),
    ("becside_ite_16", (16, 16, 16), 1, 0.0, 1.0, 0.05, 100.0, [0.05, 0.05, 0.05, 2.0], 0.0, [1, 6], 5),
    ("ufg_rte_currents_16x8x32", (16, 8, 32), 0, 1.0, 0.0, 0.05, 1000.0, [0.04, 0.05, 0.06, 0.0], 0.1, [1, 4], 6),
    # dipolar BEC (gpe_evolve_dipolar), fifth user parameter A_DIP
    ("dipolar_rte_16x8x32", (16, 8, 32), -2, 1.0, 0.0, 0.05, 1.0, [0.0625, 0.0625, 0.05, 2.0, 1.5], 0.0, [1, 6], 7),
    ("dipolar_ite_16", (16, 16, 16), -2, 0.0, 1.0, 0.05, 1.0, [0.0625, 0.0625, 0.05, 2.0, 1.5], 0.0, [1, 6], 8),
]


def main(outdir=HERE, only=None):
    os.makedirs(outdir, exist_ok=True)
    for name, shape, inter, alpha, beta, dt, npart, params, qf, steps, seed in CASES:
        if only and name not in only:
            continue
        gamma = 1.0 if inter < 0 else 2.0
        dipolar = inter == -2
        currents = "currents" in name
        psi0 = configs.random_state(shape, seed=seed, npart=npart, gamma=gamma)
        cmds = (["N"] if beta != 0 else [])
        if dipolar:
            cmds += [f"A{params[4]!r}"]
        for s in steps:
            cmds += [f"Y{s}" if dipolar else f"S{s}", "D"]
        if currents:
            cmds += ["J"]
        if dipolar:
            cmds += ["W"]
        cmds += ["E"]
        out = ref_run.run(shape, inter, alpha, beta, dt, npart, params[:4], psi0, cmds, qf=qf)
        arrays = {"psi0": psi0}
        for k, p in enumerate(out["psi"]):
            arrays[f"psi_{k}"] = p
        if currents:
            for a, j in zip("xyz", out["currents"][0]):
                arrays["j" + a] = j
        np.savez_compressed(os.path.join(outdir, name + ".npz"), **arrays)
        meta = {"shape": list(shape), "interactions": inter, "alpha": alpha, "beta": beta, "dt": dt,
                "npart": npart, "params": params, "qf": qf, "steps": steps, "seed": seed,
                "normalize_first": beta != 0, "mu": out["mu"], "energy": list(out["energy"][-1][1:]),
                "evolve": "dipolar" if dipolar else "qf", "currents": currents,
                "tol_psi": 1e-12, "source": "reference libcugpe dev/ engine built for sm_103a by oracle/build_ref.py"}
        if dipolar:
            meta["edip"] = out["edip"][-1]
        with open(os.path.join(outdir, name + ".json"), "w") as fh:
            json.dump(meta, fh, indent=1)
        print(name, "written")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE, set(sys.argv[2:]) or None)
