"""yz-plane passes (gpe_plane.cuh) against the CPU FP64 oracle and against the pencil passes.

Real-time FP32 steps on lattices with 128 x 128 yz-planes run as four launches (two yz-plane passes,
two x-pencil passes) instead of seven pencil passes: the same step (dev/gpe_engine.cu:1030-1109), with
the y and z kinetic factors applied by one 2D transform pair per plane and the friction Laplacian's
y + z part taken by one more.  FP32 tolerances as for the pencil passes: <= 2e-5 relative L2 per step
against the oracle, energies to 1e-5.
"""
import numpy as np
import pytest

import oracle
import libcugpe_gb300 as g
from libcugpe_gb300 import configs

pytestmark = pytest.mark.gpu

CASES = {
    # name: shape, interactions, qf, params, npart
    "ufg_rte_qf": ((16, 128, 128), 0, 0.1, [0.04, 0.04, 0.06, 0.0], 1000.0),
    "bec_rte": ((8, 128, 128), -1, 0.0, [0.0625, 0.05, 0.07, 31.83], 1.0),
    "bec_rte_qf": ((32, 128, 128), -1, 0.3, [0.0625, 0.0625, 0.0625, 31.83], 1.0),
}


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def engine(case, psi, plane=True, dt=0.05):
    shape, inter, qf, params, npart = CASES[case]
    e = g.Engine(shape, inter, 1.0, 0.0, dt, npart, precision=g.FP32)
    e.set_plane_passes(plane)
    e.set_user_params(params)
    if qf:
        e.set_quantum_friction_coeff(qf)
    e.set_psi(0.0, psi)
    return e


def start(case, seed=11):
    shape, inter, qf, params, npart = CASES[case]
    return configs.random_state(shape, seed=seed, npart=npart, gamma=1.0 if inter < 0 else 2.0)


@pytest.mark.parametrize("case", list(CASES))
def test_plane_passes_are_used(cuda_device, gpe_lib, case):
    e = engine(case, start(case))
    kinds = [p["kind"] for p in e.profile_passes(1)]
    assert kinds.count("plane") == 2 and len(kinds) == 4, kinds
    e.set_plane_passes(False)
    kinds = [p["kind"] for p in e.profile_passes(1)]
    assert "plane" not in kinds and len(kinds) in (6, 7), kinds
    e.close()


@pytest.mark.parametrize("case", list(CASES))
def test_plane_per_step_against_oracle(cuda_device, gpe_lib, case):
    shape, inter, qf, params, npart = CASES[case]
    psi = start(case)
    o = oracle.Oracle(shape, inter, 1.0, 0.0, 0.05, npart, threads=8)
    o.set_user_params(params)
    o.set_quantum_friction_coeff(qf)
    prev = psi
    for step in range(3):
        o.set_psi(0.0, prev)
        o.evolve_qf(1)
        _, ref = o.get_psi()
        e = engine(case, prev)
        e.evolve_qf(1)
        _, ours = e.get_psi()
        e.close()
        assert rel(ours, ref) <= 2e-5, (step, rel(ours, ref))
        prev = ref


@pytest.mark.parametrize("case", list(CASES))
def test_plane_matches_pencil_passes_over_many_steps(cuda_device, gpe_lib, case):
    """20 steps (graph replay) with plane passes and with pencil passes, energies against the oracle."""
    shape, inter, qf, params, npart = CASES[case]
    psi = start(case, seed=12)
    a, b = engine(case, psi, True), engine(case, psi, False)
    a.evolve_qf(20)
    b.evolve_qf(20)
    pa, pb = a.get_psi()[1], b.get_psi()[1]
    assert rel(pa, pb) <= 5e-5, rel(pa, pb)
    o = oracle.Oracle(shape, inter, 1.0, 0.0, 0.05, npart, threads=8)
    o.set_user_params(params)
    o.set_quantum_friction_coeff(qf)
    o.set_psi(0.0, psi)
    o.evolve_qf(20)
    _, po = o.get_psi()
    assert rel(pa, po) <= 1e-4, rel(pa, po)
    ea, eo = a.energy(), o.energy()
    assert ea[0] == pytest.approx(eo[0], abs=1e-12)
    for x, y in zip(ea[1:], eo[1:]):
        assert abs(x - y) <= 1e-5 * max(1.0, abs(y)), (x, y)
    a.close()
    b.close()


def test_plane_graph_replay_is_bit_identical_to_direct_launches(cuda_device, gpe_lib):
    case = "ufg_rte_qf"
    psi = start(case, seed=13)
    a, b = engine(case, psi), engine(case, psi)
    b.use_graphs(False)
    a.evolve_qf(12)
    b.evolve_qf(12)
    assert np.array_equal(a.get_psi()[1], b.get_psi()[1])
    a.close()
    b.close()


def test_switch_between_layouts_mid_run(cuda_device, gpe_lib):
    """Switching the pass layout between evolve calls, or going through imaginary time (pencil passes),
    continues the same evolution."""
    case = "ufg_rte_qf"
    psi = start(case, seed=14)
    a, b = engine(case, psi, True), engine(case, psi, False)
    a.evolve_qf(5)
    a.set_plane_passes(False)
    a.evolve_qf(5)
    a.set_plane_passes(True)
    a.evolve_qf(5)
    b.evolve_qf(15)
    assert rel(a.get_psi()[1], b.get_psi()[1]) <= 5e-5
    a.close()
    b.close()


def test_plane_layout_with_alternative_radix_plan_and_autotuner(cuda_device, gpe_lib):
    """The x-pencil passes may run the alternative radix plan (by hand or chosen by the autotuner) while
    the plane passes keep theirs; the autotuner restores the state."""
    case = "ufg_rte_qf"
    shape, inter, qf, params, npart = CASES[case]
    psi = start(case, seed=15)
    e = engine(case, psi)
    e.set_fft_plan(1)
    e.evolve_qf(4)
    o = oracle.Oracle(shape, inter, 1.0, 0.0, 0.05, npart, threads=8)
    o.set_user_params(params)
    o.set_quantum_friction_coeff(qf)
    o.set_psi(0.0, psi)
    o.evolve_qf(4)
    assert rel(e.get_psi()[1], o.get_psi()[1]) <= 4 * 2e-5
    e.set_fft_plan(0)
    before = e.get_psi()
    choice = e.autotune(8)
    assert choice["ms_per_step"] > 0 and choice["fft_plan"] in (0, 1, 2)
    after = e.get_psi()
    assert after[0] == before[0] and np.array_equal(after[1], before[1])
    kinds = [p["kind"] for p in e.profile_passes(1)]
    assert kinds.count("plane") == 2, kinds
    e.close()


@pytest.mark.parametrize("what", ["vortex", "slices"])
def test_plane_layout_with_enforced_phase_and_time_sliced_potential(cuda_device, gpe_lib, what):
    """The plane passes under the phase-enforcing evolution (gpe_evolve_vortex, method 1) and with a
    time-sliced additive potential, against the FP64 oracle."""
    case = "bec_rte_qf"
    shape, inter, qf, params, npart = CASES[case]
    psi = start(case, seed=16)
    e = engine(case, psi)
    o = oracle.Oracle(shape, inter, 1.0, 0.0, 0.05, npart, threads=8)
    o.set_user_params(params)
    o.set_quantum_friction_coeff(qf)
    o.set_psi(0.0, psi)
    if what == "vortex":
        e.set_vortex(0.5, -0.5, 1)
        o.set_vortex(0.5, -0.5, 1)
        e.evolve_vortex(3, 1)
        o.evolve_vortex(3, 1)
    else:
        rng = np.random.default_rng(17)
        fields = 0.002 * rng.standard_normal((3,) + shape)
        e.set_potential_slices(fields, 2)
        o.set_vextra(fields, 2)
        e.evolve_qf(6)
        o.evolve_qf(6)
    assert rel(e.get_psi()[1], o.get_psi()[1]) <= 6 * 2e-5
    kinds = [p["kind"] for p in e.profile_passes(1)]  # (steps further: after the comparison)
    assert kinds.count("plane") == 2, kinds
    e.close()


def test_plane_layout_on_lattices_with_the_real_corrector_buffer(cuda_device, gpe_lib):
    """Above 2^21 points the corrector keeps the real potential V' instead of exp(c3 V') (the Vstep3 plane
    pass recomputes the phase): 256 x 128 x 128 with friction against the pencil passes after 20 steps and
    against the oracle after one."""
    shape, inter, qf, params, npart = (256, 128, 128), 0, 0.1, [0.04, 0.04, 0.06, 0.0], 1000.0
    psi = configs.random_state(shape, seed=18, npart=npart, gamma=2.0)

    def make(plane):
        e = g.Engine(shape, inter, 1.0, 0.0, 0.05, npart, precision=g.FP32)
        e.set_plane_passes(plane)
        e.set_user_params(params)
        e.set_quantum_friction_coeff(qf)
        e.set_psi(0.0, psi)
        return e

    a = make(True)
    assert [p["kind"] for p in a.profile_passes(1)].count("plane") == 2
    a.close()
    a, b = make(True), make(False)
    a.evolve_qf(1)
    o = oracle.Oracle(shape, inter, 1.0, 0.0, 0.05, npart, threads=8)
    o.set_user_params(params)
    o.set_quantum_friction_coeff(qf)
    o.set_psi(0.0, psi)
    o.evolve_qf(1)
    assert rel(a.get_psi()[1], o.get_psi()[1]) <= 2e-5
    a.evolve_qf(19)
    b.evolve_qf(20)
    assert rel(a.get_psi()[1], b.get_psi()[1]) <= 5e-5
    a.close()
    b.close()
