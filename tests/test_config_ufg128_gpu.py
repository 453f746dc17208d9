"""The timed workload itself, at its own size: 128^3 unitary Fermi gas, real time with quantum friction.

Workload: 128^3 lattice, dx = 0.2, trap omega = (1, 1, 1.5), UFG dimers (INTERACTIONS 0), real time
(alpha = 1, beta = 0) with quantum friction 0.1, dt = 5e-3 (lattice dt' = 0.125), npart = 1000, starting
from a Thomas-Fermi state relaxed by 200 imaginary-time steps with the vortex phase atan2(y, x) imprinted.

* FP64 drop-in against the reference engine built for this lattice (dev/gpe_engine.cu:1030-1109, friction
  potential :893-933): <= 1e-12 relative L2 per step over 3 steps (each step restarted from the
  reference's state), then energy, density, norm and psi after 100 steps.
* FP32-mixed form against the FP64 form over the workload's full 10,000 steps: relative energy error
  <= 1e-6; the density's relative L2 error is reported beside it (a loose bound only catches a
  divergence).
"""
import numpy as np
import pytest

import libcugpe_gb300 as g
from libcugpe_gb300 import configs
from oracle import build_ref, ref_run

pytestmark = pytest.mark.gpu

N = 128


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def start(cuda_device, gpe_lib):
    w = configs.ufg_vortex_rte_qf(n=N)
    e = g.Engine(w.shape, w.interactions, 0.0, 1.0, w.dt, w.npart, precision=g.FP64)
    e.set_user_params(w.params)
    e.set_psi(0.0, np.abs(w.psi0))
    e.evolve_qf(200)
    _, psi = e.get_psi()
    e.close()
    X, Y, _ = configs.grid(w.shape)
    psi = np.abs(psi) * np.exp(1j * np.arctan2(Y + 0.5, X + 0.5))
    return w, configs.normalise(psi, w.npart, w.gamma)


def engine(w, psi, precision=g.FP64):
    e = g.Engine(w.shape, w.interactions, w.alpha, w.beta, w.dt, w.npart, precision=precision)
    e.set_user_params(w.params)
    e.set_quantum_friction_coeff(w.qf)
    e.set_psi(0.0, psi)
    return e


@pytest.fixture(scope="module")
def reference(cuda_device):
    if not ref_run.available():
        pytest.skip("reference sources not available on this machine")
    build_ref.build_one(N, N, N, 0)
    return True


def test_fp64_per_step_parity_with_reference(reference, start):
    w, psi = start
    out = ref_run.run(w.shape, w.interactions, w.alpha, w.beta, w.dt, w.npart, w.params, psi,
                      ["S1", "D", "S1", "D", "S1", "D"], qf=w.qf)
    prev = psi
    errs = []
    for k, ref in enumerate(out["psi"]):
        e = engine(w, prev)
        e.evolve_qf(1)
        _, ours = e.get_psi()
        e.close()
        errs.append(rel(ours, ref))
        assert errs[-1] <= 1e-12, (k, errs)
        prev = ref
    print("per-step relative L2 vs reference:", errs)


def test_fp64_after_100_steps_matches_reference(reference, start):
    w, psi = start
    out = ref_run.run(w.shape, w.interactions, w.alpha, w.beta, w.dt, w.npart, w.params, psi,
                      ["E", "S100", "E", "D"], qf=w.qf)
    e = engine(w, psi)
    e0 = e.energy()
    e.evolve_qf(100)
    e1 = e.energy()
    _, ours = e.get_psi()
    norm = e.get_norm()
    e.close()
    ref = out["psi"][0]
    assert rel(ours, ref) <= 1e-11, rel(ours, ref)
    for ours_e, ref_e in ((e0, out["energy"][0]), (e1, out["energy"][1])):
        assert ours_e[0] == pytest.approx(ref_e[0], abs=1e-12)
        for a, b in zip(ours_e[1:], ref_e[1:]):
            assert abs(a - b) <= 1e-10 * max(1.0, abs(b)), (a, b)
    dens_ours = w.gamma * np.abs(ours) ** 2
    dens_ref = w.gamma * np.abs(ref) ** 2
    assert rel(dens_ours, dens_ref) <= 1e-11, rel(dens_ours, dens_ref)
    norm_ref = float(dens_ref.sum())
    assert abs(norm - norm_ref) <= 1e-12 * norm_ref, (norm, norm_ref)


def test_fp32_mixed_energy_error_over_full_run(start):
    """FP32-mixed against FP64 over the workload's 10,000 steps: |E32 - E64| / |E64| <= 1e-6."""
    w, psi = start
    assert w.steps == 10000
    a = engine(w, psi, g.FP32)
    b = engine(w, psi, g.FP64)
    a.evolve_qf(w.steps)
    b.evolve_qf(w.steps)
    ta, *ea = a.energy()
    tb, *eb = b.energy()
    assert ta == pytest.approx(tb, rel=1e-12)
    Ea, Eb = sum(ea), sum(eb)
    _, da = a.get_density()
    _, db = b.get_density()
    a.close()
    b.close()
    de = abs(Ea - Eb) / abs(Eb)
    dd = rel(da, db)
    print(f"after {w.steps} steps: dE/E = {de:.3e}, density relative L2 = {dd:.3e}")
    assert np.isfinite(Ea) and np.isfinite(Eb)
    assert de <= 1e-6, (de, dd)
    # the density error is reported, not bounded by the workload; measured 1.06e-3 after 10,000 steps
    # (the vortex core's position drifts with the accumulated FP32 phase error); the bound only
    # catches a divergence
    assert dd <= 1e-2, dd
