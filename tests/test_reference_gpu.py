"""GPU engine against the reference libcugpe engine built for this GPU.

The reference (dev/ engine, cuFFT Z2Z, FP64) is compiled by
oracle/build_ref.py, one binary per lattice and functional, and driven by
oracle/ref_runner.cpp through its own public API.  Both engines get the same
seeded state; the FP64 drop-in must agree to <= 1e-12 relative L2 per step,
and in energy, chemical potential and density after several steps.
"""
import numpy as np
import pytest

import libcugpe_gb300 as g
from libcugpe_gb300 import configs
from oracle import build_ref, ref_run

pytestmark = pytest.mark.gpu

CASES = [
    # shape, interactions, alpha, beta, dt, npart, params, qf
    ((16, 16, 16), -1, 0.0, 1.0, 0.05, 1.0, [0.0625, 0.0625, 0.0625, 31.83], 0.0),
    ((32, 16, 8), -1, 1.0, 0.0, 0.05, 1.0, [0.0625, 0.05, 0.07, 31.83], 0.0),
    ((16, 16, 16), 0, 1.0, 0.0, 0.05, 1000.0, [0.04, 0.04, 0.06, 0.0], 0.1),
    ((8, 32, 16), 0, 0.0, 1.0, 0.05, 1000.0, [0.04, 0.04, 0.06, 0.0], 0.1),
    ((16, 16, 16), 0, 1.0, 0.0, 0.05, 1000.0, [0.04, 0.04, 0.06, 0.0], 0.0),
    ((32, 32, 32), 0, 1.0, 0.0, 0.125, 1000.0, [0.04, 0.04, 0.06, 0.0], 0.1),
    # BEC side of the crossover (INTERACTIONS 1), a_scat = 2
    ((16, 16, 16), 1, 0.0, 1.0, 0.05, 100.0, [0.05, 0.05, 0.05, 2.0], 0.0),
    ((16, 8, 32), 1, 1.0, 0.0, 0.05, 100.0, [0.05, 0.06, 0.04, 2.0], 0.1),
]


@pytest.fixture(scope="module")
def reference(cuda_device):
    if not ref_run.available():
        pytest.skip("reference sources not available on this machine")
    build_ref.build(sorted({(c[0][0], c[0][1], c[0][2], c[1]) for c in CASES} | {(64, 64, 64, -1)}))
    return True


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def engine_for(shape, inter, alpha, beta, dt, npart, params, qf, psi):
    e = g.Engine(shape, inter, alpha, beta, dt, npart)
    e.set_user_params(params)
    if qf:
        e.set_quantum_friction_coeff(qf)
    e.set_psi(0.0, psi)
    return e


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}_i{c[1]}_b{c[3]}_qf{c[7]}")
def test_per_step_parity_with_reference(reference, gpe_lib, case):
    shape, inter, alpha, beta, dt, npart, params, qf = case
    gamma = 1.0 if inter < 0 else 2.0
    psi = configs.random_state(shape, seed=21, npart=npart, gamma=gamma)
    # reference: 1 step, dump, 1 step, dump, ... ; ours restarts from the reference's psi each step
    cmds = []
    for _ in range(3):
        cmds += ["S1", "D"]
    out = ref_run.run(shape, inter, alpha, beta, dt, npart, params, psi, cmds, qf=qf)
    prev = psi
    for k, ref in enumerate(out["psi"]):
        e = engine_for(shape, inter, alpha, beta, dt, npart, params, qf, prev)
        mu = e.evolve_qf(1)
        _, ours = e.get_psi()
        assert rel(ours, ref) <= 1e-12, (k, rel(ours, ref))
        if beta != 0.0:
            assert abs(mu - out["mu"][k]) <= 1e-10 * max(1.0, abs(out["mu"][k]))
        prev = ref


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}_i{c[1]}_b{c[3]}_qf{c[7]}")
def test_energy_density_after_n_steps(reference, gpe_lib, case):
    shape, inter, alpha, beta, dt, npart, params, qf = case
    gamma = 1.0 if inter < 0 else 2.0
    psi = configs.random_state(shape, seed=22, npart=npart, gamma=gamma)
    n = 40
    out = ref_run.run(shape, inter, alpha, beta, dt, npart, params, psi, ["E", f"S{n}", "E", "D"], qf=qf)
    e = engine_for(shape, inter, alpha, beta, dt, npart, params, qf, psi)
    e0 = e.energy()
    mu = e.evolve_qf(n)
    e1 = e.energy()
    _, ours = e.get_psi()
    ref = out["psi"][0]
    assert rel(ours, ref) <= 1e-11, rel(ours, ref)
    for ours_e, ref_e in ((e0, out["energy"][0]), (e1, out["energy"][1])):
        assert ours_e[0] == pytest.approx(ref_e[0], abs=1e-12)
        for a, b in zip(ours_e[1:], ref_e[1:]):
            assert abs(a - b) <= 1e-10 * max(1.0, abs(b)), (a, b)
    if beta != 0.0:
        assert abs(mu - out["mu"][0]) <= 1e-9 * max(1.0, abs(out["mu"][0]))
    dens_ours = gamma * np.abs(ours) ** 2
    dens_ref = gamma * np.abs(ref) ** 2
    assert rel(dens_ours, dens_ref) <= 2e-11


def test_bec_64_ite_matches_reference(reference, gpe_lib):
    """The 64^3 contact-BEC imaginary-time workload, 200 steps."""
    w = configs.bec_ground_state_ite(n=64, steps=200)
    out = ref_run.run(w.shape, -1, 0.0, 1.0, w.dt, w.npart, w.params, w.psi0, ["N", "S200", "E", "D"])
    e = engine_for(w.shape, -1, 0.0, 1.0, w.dt, w.npart, w.params, 0.0, w.psi0)
    e.normalize_psi()
    mu = e.evolve_qf(200)
    en = e.energy()
    _, ours = e.get_psi()
    assert rel(ours, out["psi"][0]) <= 1e-11
    assert abs(mu - out["mu"][0]) <= 1e-9 * abs(out["mu"][0])
    etot, etot_ref = sum(en[1:]), sum(out["energy"][0][1:])
    assert abs(etot - etot_ref) <= 1e-11 * abs(etot_ref)


def test_compare_harness_ite_then_rte_matches_reference(reference, gpe_lib):
    """The reference's own regression harness (test_compare/gpe_imag.c, gpe_real.c, compared by
    test_compare/compare.py) on its lattice: 256x32x32 UFG, dt = 0.025, npart = 1000, omega = (0.01,
    0.10, 0.11), psi = 1.  Imaginary time in blocks of 100 steps until the energy per particle changes
    by < 1e-5 (gpe_imag.c:125-144), then real time from t = 0 to t > 10 (gpe_real.c:145-163).  Same
    number of blocks, energies after every block and both final states as the reference engine."""
    shape, dt, npart, params = (256, 32, 32), 0.025, 1000.0, [0.01, 0.10, 0.11, 0.0]
    build_ref.build([(256, 32, 32, 0)])
    psi0 = np.ones(shape, dtype=np.complex128)
    out = ref_run.run(shape, 0, 0.0, 1.0, dt, npart, params, psi0,
                      ["N", "E", "C100/1e-5", "D", "R", "Z", "E", "T100/10.0", "D"], timeout=1200)
    e = g.Engine(shape, 0, 0.0, 1.0, dt, npart)
    e.set_user_params(params)
    e.set_psi(0.0, psi0)
    e.normalize_psi()
    ours = [e.energy()]
    while True:
        e.evolve_qf(100)
        ours.append(e.energy())
        if abs(sum(ours[-2][1:]) - sum(ours[-1][1:])) / npart < 1e-5:
            break
    n_ite = len(ours)
    _, psi_ite = e.get_psi()
    e.set_rte_evolution()
    e.set_psi(0.0, psi_ite)
    ours.append(e.energy())
    while True:
        e.evolve_qf(100)
        ours.append(e.energy())
        if ours[-1][0] > 10.0:
            break
    _, psi_rte = e.get_psi()
    ref = out["energy"]
    assert len(ours) == len(ref), (len(ours), len(ref), n_ite)
    for a, r in zip(ours, ref):
        assert a[0] == pytest.approx(r[0], abs=1e-9)
        for x, y in zip(a[1:], r[1:]):
            assert abs(x - y) <= 1e-9 * max(1.0, abs(y)), (a, r)
    assert rel(psi_ite, out["psi"][0]) <= 1e-9
    assert rel(psi_rte, out["psi"][1]) <= 1e-9


@pytest.mark.parametrize("beta", [1.0, 0.0])
@pytest.mark.parametrize("method", [1, 2, 3, "P"])
def test_phase_enforcing_evolves_match_reference(reference, gpe_lib, beta, method):
    shape, inter, npart, params, qf = (16, 16, 16), -1, 1.0, [0.0625, 0.0625, 0.0625, 31.83], 0.0
    alpha = 1.0 - beta
    psi = configs.random_state(shape, seed=23, npart=npart)
    e = engine_for(shape, inter, alpha, beta, 0.05, npart, params, qf, psi)
    if method == "P":
        cmds = ["G", "P4", "D"]
        e.get_phase()
        mu = e.evolve_enforced_phase(4)
    else:
        cmds = ["X0.5/-0.5/1", f"V{method}_4", "D"]
        e.set_vortex(0.5, -0.5, 1)
        mu = e.evolve_vortex(4, method)
    out = ref_run.run(shape, inter, alpha, beta, 0.05, npart, params, psi, cmds, qf=qf)
    _, ours = e.get_psi()
    assert rel(ours, out["psi"][0]) <= 3e-12, rel(ours, out["psi"][0])
    if beta != 0.0:
        assert abs(mu - out["mu"][0]) <= 1e-10 * max(1.0, abs(out["mu"][0]))


@pytest.mark.parametrize("case", [CASES[0], CASES[3]], ids=["bec", "ufg_qf"])
def test_currents_match_reference(reference, gpe_lib, case):
    """gpe_get_currents against the reference's own on the reference's state after 3 RTE steps."""
    shape, inter, alpha, beta, dt, npart, params, qf = case
    gamma = 1.0 if inter < 0 else 2.0
    psi = configs.random_state(shape, seed=24, npart=npart, gamma=gamma)
    out = ref_run.run(shape, inter, 1.0, 0.0, dt, npart, params, psi, ["S3", "J", "D"], qf=qf)
    e = engine_for(shape, inter, 1.0, 0.0, dt, npart, params, qf, out["psi"][0])
    _, jx, jy, jz = e.get_currents()
    for ours, ref in zip((jx, jy, jz), out["currents"][0]):
        assert rel(ours, ref) <= 1e-12, rel(ours, ref)


@pytest.mark.parametrize("ab", [(1.0, 0.0), (0.0, 1.0)], ids=["rte", "ite"])
def test_dipolar_matches_reference(reference, gpe_lib, ab):
    """gpe_evolve_dipolar and gpe_energy_dipolar2 of the reference built with INTERACTIONS=-2."""
    shape = (16, 16, 16)
    build_ref.build([(16, 16, 16, -2)])
    params = [0.0625, 0.0625, 0.05, 2.0]
    psi = configs.random_state(shape, seed=25, npart=1.0, gamma=1.0)
    out = ref_run.run(shape, -2, ab[0], ab[1], 0.05, 1.0, params, psi, ["A1.5", "W", "Y1", "D", "Y4", "W", "D"])
    e = g.Engine(shape, -2, ab[0], ab[1], 0.05, 1.0)
    e.set_user_params(params + [1.5])
    e.set_psi(0.0, psi)
    assert e.energy_dipolar()[1] == pytest.approx(out["edip"][0], rel=1e-12)
    mu = e.evolve_dipolar(1)
    assert rel(e.get_psi()[1], out["psi"][0]) <= 1e-12
    if ab[1] != 0.0:
        assert abs(mu - out["mu"][0]) <= 1e-10 * max(1.0, abs(out["mu"][0]))
    e.evolve_dipolar(4)
    assert rel(e.get_psi()[1], out["psi"][1]) <= 1e-11
    assert e.energy_dipolar()[1] == pytest.approx(out["edip"][1], rel=1e-11)
