"""GPU engine against the CPU FP64 oracle, through the C ABI.

FP64 plain form: <= 1e-12 relative L2 per step (both start each step from the
same psi), drift after several steps, mu and energies.  FP32-mixed form:
relative L2 <= 2e-5 per step and energies to 1e-5."""
import numpy as np
import pytest

import oracle
import libcugpe_gb300 as g
from libcugpe_gb300 import configs

pytestmark = pytest.mark.gpu

TOL_FP64_STEP = 1e-12
TOL_FP32_STEP = 2e-5

CASES = {
    # name: interactions, alpha, beta, qf, params, npart
    "bec_ite": (-1, 0.0, 1.0, 0.0, [0.0625, 0.0625, 0.0625, 31.83], 1.0),
    "bec_rte": (-1, 1.0, 0.0, 0.0, [0.0625, 0.05, 0.07, 31.83], 1.0),
    "ufg_rte": (0, 1.0, 0.0, 0.0, [0.04, 0.04, 0.06, 0.0], 1000.0),
    "ufg_rte_qf": (0, 1.0, 0.0, 0.1, [0.04, 0.04, 0.06, 0.0], 1000.0),
    "ufg_ite_qf": (0, 0.0, 1.0, 0.1, [0.04, 0.04, 0.06, 0.0], 1000.0),
    "bec_ite_qf": (-1, 0.0, 1.0, 0.2, [0.0625, 0.0625, 0.0625, 31.83], 1.0),
    "bec_rte_qf": (-1, 1.0, 0.0, 0.3, [0.0625, 0.0625, 0.0625, 31.83], 1.0),
    "becside_ite": (1, 0.0, 1.0, 0.0, [0.05, 0.05, 0.05, 2.0], 100.0),
}
SHAPES = [(16, 16, 16), (32, 16, 8), (8, 32, 16), (16, 8, 64), (128, 16, 8), (8, 256, 8), (512, 8, 16)]


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def make_pair(shape, case, precision=g.FP64, dt=0.05, seed=7):
    inter, alpha, beta, qf, params, npart = CASES[case]
    gamma = 1.0 if inter == -1 else 2.0
    psi = configs.random_state(shape, seed=seed, npart=npart, gamma=gamma)
    e = g.Engine(shape, inter, alpha, beta, dt, npart, precision=precision)
    e.set_user_params(params)
    o = oracle.Oracle(shape, inter, alpha, beta, dt, npart, threads=4)
    o.set_user_params(params)
    if qf:
        e.set_quantum_friction_coeff(qf)
        o.set_quantum_friction_coeff(qf)
    e.set_psi(0.0, psi)
    o.set_psi(0.0, psi)
    return e, o, psi


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("shape", SHAPES[:3])
def test_fp64_per_step_parity(cuda_device, gpe_lib, case, shape):
    e, o, psi = make_pair(shape, case)
    beta = CASES[case][2]
    for step in range(4):
        mu_e = e.evolve_qf(1)
        mu_o = o.evolve_qf(1)
        _, pe = e.get_psi()
        _, po = o.get_psi()
        assert rel(pe, po) <= TOL_FP64_STEP, (step, rel(pe, po))
        if beta != 0.0:
            assert abs(mu_e - mu_o) <= 1e-10 * max(1.0, abs(mu_o))
        e.set_psi(0.0, po)  # next step starts from the same psi again
        o.set_psi(0.0, po)


@pytest.mark.parametrize("shape", SHAPES[3:])
@pytest.mark.parametrize("case", ["bec_ite", "ufg_rte_qf"])
def test_fp64_parity_all_pencil_lengths(cuda_device, gpe_lib, case, shape):
    e, o, _ = make_pair(shape, case)
    e.evolve_qf(1)
    o.evolve_qf(1)
    assert rel(e.get_psi()[1], o.get_psi()[1]) <= TOL_FP64_STEP


@pytest.mark.parametrize("case", ["bec_ite", "ufg_rte", "ufg_rte_qf", "ufg_ite_qf"])
def test_fp64_multi_step_drift_and_energy(cuda_device, gpe_lib, case):
    shape = (32, 16, 16)
    e, o, _ = make_pair(shape, case)
    for _ in range(3):
        mu_e = e.evolve_qf(10)
        mu_o = o.evolve_qf(10)
    t_e, pe = e.get_psi()
    t_o, po = o.get_psi()
    assert t_e == pytest.approx(t_o, abs=1e-12)
    assert rel(pe, po) <= 3e-11
    if CASES[case][2] != 0.0:
        assert abs(mu_e - mu_o) <= 1e-9 * max(1.0, abs(mu_o))
    en_e, en_o = e.energy(), o.energy()
    for a, b in zip(en_e[1:], en_o[1:]):
        assert abs(a - b) <= 1e-10 * max(1.0, abs(b))
    # the RTE energy call normalises psi in place on both sides
    assert rel(e.get_psi()[1], o.get_psi()[1]) <= 3e-11
    _, de = e.get_density()
    _, do = o.get_density()
    assert rel(de, do) <= 3e-11
    assert e.get_norm() == pytest.approx(o.get_norm(), rel=1e-12)


@pytest.mark.parametrize("case", ["bec_ite", "ufg_rte_qf", "ufg_ite_qf", "bec_rte"])
def test_fp32_mixed_against_fp64_oracle(cuda_device, gpe_lib, case):
    shape = (32, 16, 16)
    e, o, _ = make_pair(shape, case, precision=g.FP32)
    e.evolve_qf(1)
    o.evolve_qf(1)
    assert rel(e.get_psi()[1], o.get_psi()[1]) <= TOL_FP32_STEP
    e.evolve_qf(20)
    o.evolve_qf(20)
    assert rel(e.get_psi()[1], o.get_psi()[1]) <= 20 * TOL_FP32_STEP
    en_e, en_o = e.energy(), o.energy()
    etot_e, etot_o = sum(en_e[1:]), sum(en_o[1:])
    assert abs(etot_e - etot_o) <= 1e-5 * abs(etot_o)


def test_graph_replay_is_bit_identical(cuda_device, gpe_lib):
    shape = (16, 16, 32)
    e1, _, psi = make_pair(shape, "ufg_ite_qf")
    e2, _, _ = make_pair(shape, "ufg_ite_qf")
    e2.use_graphs(False)
    m1 = e1.evolve_qf(37)
    m2 = e2.evolve_qf(37)
    assert m1 == m2
    assert np.array_equal(e1.get_psi()[1], e2.get_psi()[1])
    n0 = e1.kernel_launches()
    e1.evolve_qf(16)
    assert e1.kernel_launches() - n0 >= 16 * 7  # 7 fused passes per quantum-friction step


def test_normalize_and_norm(cuda_device, gpe_lib):
    shape = (16, 16, 16)
    e, o, psi = make_pair(shape, "bec_rte")
    e.set_psi(0.0, 3.0 * psi)
    assert e.get_norm() == pytest.approx(9.0 * float(np.sum(np.abs(psi) ** 2)), rel=1e-13)
    e.normalize_psi()
    assert e.get_norm() == pytest.approx(1.0, rel=1e-13)


def test_time_and_step_counter(cuda_device, gpe_lib):
    shape = (16, 16, 16)
    e, o, psi = make_pair(shape, "bec_ite", dt=0.02)
    e.evolve_qf(5)
    t, _ = e.get_psi()
    assert t == pytest.approx(0.1)
    e.set_time(1.0)
    t, _ = e.get_psi()
    assert t == pytest.approx(1.0)
    e.set_psi(2.5, psi)
    assert e.get_psi()[0] == 2.5


def test_error_codes_on_gpu(cuda_device, gpe_lib):
    e = g.Engine((16, 16, 16), -1, 0.0, 1.0, 0.1, 1.0)
    with pytest.raises(g.GPEError) as ex:
        e.set_user_params(np.zeros(33))
    assert ex.value.code == g.ERR_TOO_MANY_PARAMS
    with pytest.raises(g.GPEError) as ex:
        g.Engine((16, 12, 16), -1, 0.0, 1.0, 0.1, 1.0)
    assert ex.value.code == g.ERR_LATTICE


def test_time_sliced_potential_matches_oracle(cuda_device, gpe_lib):
    shape = (16, 16, 16)
    e, o, _ = make_pair(shape, "bec_rte", dt=0.02)
    rng = np.random.default_rng(11)
    fields = 0.05 * rng.standard_normal((3,) + shape)
    e.set_potential_slices(fields, 4)
    o.set_vextra(fields, 4)
    e.evolve_qf(10)
    o.evolve_qf(10)
    assert rel(e.get_psi()[1], o.get_psi()[1]) <= 1e-11
    en_e, en_o = e.energy(), o.energy()
    for a, b in zip(en_e[1:], en_o[1:]):
        assert abs(a - b) <= 1e-10 * max(1.0, abs(b))


@pytest.mark.parametrize("case", ["bec_ite", "ufg_ite_qf", "bec_rte", "ufg_rte_qf"])
@pytest.mark.parametrize("method", [1, 2, 3, 4])
def test_phase_enforcing_evolves_match_oracle(cuda_device, gpe_lib, case, method):
    """gpe_evolve_vortex{,2,3} (methods 1-3) and gpe_evolve_enforced_phase (4)."""
    shape = (16, 16, 16)
    e, o, psi = make_pair(shape, case)
    if method == 4:
        rng = np.random.default_rng(5)
        ph = rng.uniform(-np.pi, np.pi, shape)
        e.set_phase(ph)
        o.set_phase(ph)
        mu_e, mu_o = e.evolve_enforced_phase(3), o.evolve_enforced_phase(3)
    else:
        e.set_vortex(0.5, -0.5, 1)
        o.set_vortex(0.5, -0.5, 1)
        mu_e, mu_o = e.evolve_vortex(3, method), o.evolve_vortex(3, method)
    assert rel(e.get_psi()[1], o.get_psi()[1]) <= 3e-12
    if CASES[case][2] != 0.0:
        assert abs(mu_e - mu_o) <= 1e-10 * max(1.0, abs(mu_o))
    np.testing.assert_allclose(e.get_phase(), o.get_phase(), atol=1e-9)


@pytest.mark.parametrize("shape", [(16, 16, 16), (32, 16, 8), (8, 256, 8), (512, 8, 16)])
def test_currents_match_oracle(cuda_device, gpe_lib, shape):
    """gpe_get_currents: one axis pass per component (FFT_a, x k_a/(Gamma N_a), inverse,
    Re(conj(psi) .)) against the oracle's 3D-FFT restatement; FP64 <= 1e-12, FP32 <= 5e-5 (the
    currents of a random-phase state are small differences of large products)."""
    e, o, _ = make_pair(shape, "ufg_rte_qf")
    o.evolve_qf(3)
    t, p = o.get_psi()
    e.set_psi(t, p)
    o.set_psi(t, p)
    ref = o.get_currents()
    got = e.get_currents()
    assert got[0] == pytest.approx(ref[0])
    for a in range(1, 4):
        assert rel(got[a], ref[a]) <= 1e-12, (a, rel(got[a], ref[a]))
    # currents leave the evolution untouched: the next steps still match
    e.evolve_qf(2)
    o.evolve_qf(2)
    assert rel(e.get_psi()[1], o.get_psi()[1]) <= 5e-12
    e32, o32, _ = make_pair(shape, "bec_rte", precision=g.FP32)
    ref = o32.get_currents()
    got = e32.get_currents()
    for a in range(1, 4):
        assert rel(got[a], ref[a]) <= 5e-5, (a, rel(got[a], ref[a]))


WZ = {"ufg_rte_qf": 0.25, "ufg_ite_qf": 0.25, "ufg_rte": 0.25, "bec_ite": 0.5}


def make_wz_pair(shape, case, precision=g.FP64):
    e, o, psi = make_pair(shape, case, precision=precision)
    e.set_weizsacker(WZ[case])
    o.set_weizsacker(WZ[case])
    return e, o, psi


@pytest.mark.parametrize("case", list(WZ))
@pytest.mark.parametrize("shape", SHAPES[:3])
def test_weizsacker_fp64_per_step_parity(cuda_device, gpe_lib, case, shape):
    """Weizsaecker term (new form, oracle-pinned): <= 1e-12 per step against the oracle."""
    e, o, _ = make_wz_pair(shape, case)
    beta = CASES[case][2]
    for step in range(3):
        mu_e = e.evolve_qf(1)
        mu_o = o.evolve_qf(1)
        _, po = o.get_psi()
        assert rel(e.get_psi()[1], po) <= TOL_FP64_STEP, (step, rel(e.get_psi()[1], po))
        if beta != 0.0:
            assert abs(mu_e - mu_o) <= 1e-10 * max(1.0, abs(mu_o))
        e.set_psi(0.0, po)
        o.set_psi(0.0, po)


@pytest.mark.parametrize("case", ["ufg_rte_qf", "ufg_ite_qf", "ufg_rte"])
def test_weizsacker_multi_step_fp64_fp32(cuda_device, gpe_lib, case):
    """30 steps through the replayed step (sums of the z axis carried from the previous step's
    last pass); the FP32 form within 2e-5 per step; the term changes the evolution."""
    shape = (32, 16, 16)
    e, o, psi = make_wz_pair(shape, case)
    for _ in range(3):
        e.evolve_qf(10)
        o.evolve_qf(10)
    po = o.get_psi()[1]
    assert rel(e.get_psi()[1], po) <= 3e-11
    plain, _, _ = make_pair(shape, case)
    plain.evolve_qf(30)
    assert rel(plain.get_psi()[1], po) > 1e-6
    e32, o32, _ = make_wz_pair(shape, case, precision=g.FP32)
    e32.evolve_qf(1)
    o32.evolve_qf(1)
    assert rel(e32.get_psi()[1], o32.get_psi()[1]) <= TOL_FP32_STEP
    e32.evolve_qf(20)
    o32.evolve_qf(20)
    assert rel(e32.get_psi()[1], o32.get_psi()[1]) <= 20 * TOL_FP32_STEP


def test_weizsacker_off_restores_plain_step(cuda_device, gpe_lib):
    shape = (16, 16, 16)
    e, o, psi = make_pair(shape, "ufg_rte_qf")
    e.set_weizsacker(0.25)
    e.evolve_qf(2)
    e.set_weizsacker(0.0)
    e.set_psi(0.0, psi)
    e.evolve_qf(3)
    o.evolve_qf(3)
    assert rel(e.get_psi()[1], o.get_psi()[1]) <= 3e-12


def test_weizsacker_substeps_keep_the_step_length(cuda_device, gpe_lib):
    """A step beyond the stability bound (dt |lambda| 3 pi^2 > 0.4) runs as sub-steps; evolve(nt)
    still advances nt dt and matches the oracle, which sub-steps the same way."""
    shape = (16, 16, 16)
    e, o, _ = make_pair(shape, "ufg_rte_qf", dt=0.125)
    e.set_weizsacker(0.25)
    o.set_weizsacker(0.25)
    e.evolve_qf(4)
    o.evolve_qf(4)
    assert e.get_psi()[0] == pytest.approx(0.5)
    assert rel(e.get_psi()[1], o.get_psi()[1]) <= 1e-11


DIP_PARAMS = [0.0625, 0.0625, 0.05, 2.0, 1.5]  # OMEGA_X..Z, A_CON, A_DIP


def make_dip_pair(shape, alpha, beta, precision=g.FP64, seed=31):
    psi = configs.random_state(shape, seed=seed, npart=1.0, gamma=1.0)
    e = g.Engine(shape, -2, alpha, beta, 0.05, 1.0, precision=precision)
    e.set_user_params(DIP_PARAMS)
    e.set_psi(0.0, psi)
    o = oracle.Oracle(shape, -2, alpha, beta, 0.05, 1.0, threads=4)
    o.set_user_params(DIP_PARAMS)
    o.set_psi(0.0, psi)
    return e, o


@pytest.mark.parametrize("ab", [(1.0, 0.0), (0.0, 1.0)], ids=["rte", "ite"])
@pytest.mark.parametrize("shape", [(16, 16, 16), (32, 16, 8), (8, 32, 64)])
def test_dipolar_fp64_per_step_parity(cuda_device, gpe_lib, shape, ab):
    """gpe_evolve_dipolar: density transform as axis passes, kernel multiply in the x pass, potential
    step fused into the last inverse pass; <= 1e-12 per step against the oracle, mu, E_dip."""
    e, o = make_dip_pair(shape, *ab)
    for step in range(3):
        mu_e = e.evolve_dipolar(1)
        mu_o = o.evolve_dipolar(1)
        t, po = o.get_psi()
        assert rel(e.get_psi()[1], po) <= TOL_FP64_STEP, (step, rel(e.get_psi()[1], po))
        if ab[1] != 0.0:
            assert abs(mu_e - mu_o) <= 1e-10 * max(1.0, abs(mu_o))
        e.set_psi(t, po)
        o.set_psi(t, po)
    assert e.energy_dipolar()[1] == pytest.approx(o.energy_dipolar(), rel=1e-12)
    e.evolve_dipolar(10)
    o.evolve_dipolar(10)
    assert rel(e.get_psi()[1], o.get_psi()[1]) <= 2e-11
    assert e.get_psi()[0] == pytest.approx(o.get_psi()[0])


def test_dipolar_fp32_against_fp64_oracle(cuda_device, gpe_lib):
    e, o = make_dip_pair((32, 16, 16), 1.0, 0.0, precision=g.FP32)
    e.evolve_dipolar(1)
    o.evolve_dipolar(1)
    assert rel(e.get_psi()[1], o.get_psi()[1]) <= TOL_FP32_STEP
    e.evolve_dipolar(20)
    o.evolve_dipolar(20)
    assert rel(e.get_psi()[1], o.get_psi()[1]) <= 20 * TOL_FP32_STEP
    assert e.energy_dipolar()[1] == pytest.approx(o.energy_dipolar(), rel=1e-5)


@pytest.mark.parametrize("precision", [g.FP32, g.FP64])
def test_autotune_restores_state_and_keeps_results(cuda_device, gpe_lib, precision):
    """The autotuner runs the engine's own state under each configuration, puts it back, and every
    configuration it may pick computes the same bits."""
    shape = (32, 16, 64)
    e, _, psi = make_pair(shape, "ufg_rte_qf", precision=precision)
    ref, _, _ = make_pair(shape, "ufg_rte_qf", precision=precision)
    e.evolve_qf(3)
    ref.evolve_qf(3)
    before = e.get_psi()
    choice = e.autotune(8)
    assert choice["graph_steps"] in (8, 16, 32) and choice["ms_per_step"] > 0
    assert choice["direct"] in ((0, 1) if precision == g.FP32 else (-1,))
    assert choice["fft_plan"] in ((0, 1, 2) if precision == g.FP32 else (0,))
    assert e.get_fft_plan() == choice["fft_plan"]
    after = e.get_psi()
    assert after[0] == before[0] and np.array_equal(after[1], before[1])
    if choice["fft_plan"] < 2:
        ref.set_fft_plan(choice["fft_plan"])  # operand mode and graph length leave the bits unchanged
    e.evolve_qf(20)
    ref.evolve_qf(20)
    if choice["fft_plan"] == 2:  # a plan per fused pass: FP32 rounding of the other factorisations
        assert rel(e.get_psi()[1], ref.get_psi()[1]) <= 20 * TOL_FP32_STEP
    else:
        assert np.array_equal(e.get_psi()[1], ref.get_psi()[1])
    e.set_fft_plan(0)
    assert e.get_fft_plan() == 0


@pytest.mark.parametrize("precision", [g.FP64, g.FP32])
def test_weizsacker_energy_matches_oracle(cuda_device, gpe_lib, precision):
    """energy() includes E_W = (lambda/8) sum |grad rho|^2/(rho + eps) in eint."""
    shape = (32, 16, 16)
    e, o, _ = make_wz_pair(shape, "ufg_ite_qf", precision=precision)
    e.evolve_qf(2)
    o.evolve_qf(2)
    tol = 1e-10 if precision == g.FP64 else 2e-5
    for a, b in zip(e.energy()[1:], o.energy()[1:]):
        assert abs(a - b) <= tol * max(1.0, abs(b)), (a, b)


@pytest.mark.parametrize("shape", [(32, 64, 128), (256, 16, 8), (8, 16, 512), (512, 32, 8)])
def test_fp32_radix_plan_1_against_oracle(cuda_device, gpe_lib, shape):
    """The alternative radix plans of FP32 pencils of 32 to 512 points (8 <-> 16 points per thread)
    against the FP64 oracle, plain and friction schedules, ITE and RTE; plans 0 and 1 agree to FP32
    rounding."""
    for case in ("bec_ite", "ufg_rte_qf", "ufg_ite_qf"):
        e, o, _ = make_pair(shape, case, precision=g.FP32)
        e0, _, _ = make_pair(shape, case, precision=g.FP32)
        e.set_fft_plan(1)
        assert e.get_fft_plan() == 1 and e0.get_fft_plan() == 0
        e.evolve_qf(2)
        o.evolve_qf(2)
        e0.evolve_qf(2)
        p1, p0, po = e.get_psi()[1], e0.get_psi()[1], o.get_psi()[1]
        assert rel(p1, po) <= 2 * TOL_FP32_STEP, (case, rel(p1, po))
        assert rel(p1, p0) <= 2 * TOL_FP32_STEP, (case, rel(p1, p0))
        for a, b in zip(e.energy()[1:], o.energy()[1:]):
            assert abs(a - b) <= 1e-5 * max(1.0, abs(b)), (case, a, b)


@pytest.mark.parametrize("what", ["dipolar", "currents", "weizsacker"])
def test_fp32_radix_plan_1_other_passes(cuda_device, gpe_lib, what):
    """The dipolar convolution passes, the current passes and the Weizsaecker sums under the
    alternative radix plans, against the FP64 oracle with the FP32 tolerances of plan 0."""
    shape = (32, 64, 128)
    if what == "dipolar":
        e, o = make_dip_pair(shape, 1.0, 0.0, precision=g.FP32)
        e.set_fft_plan(1)
        e.evolve_dipolar(1)
        o.evolve_dipolar(1)
        assert rel(e.get_psi()[1], o.get_psi()[1]) <= TOL_FP32_STEP
        e.evolve_dipolar(10)
        o.evolve_dipolar(10)
        assert rel(e.get_psi()[1], o.get_psi()[1]) <= 10 * TOL_FP32_STEP
        assert e.energy_dipolar()[1] == pytest.approx(o.energy_dipolar(), rel=1e-5)
    elif what == "currents":
        e, o, _ = make_pair(shape, "bec_rte", precision=g.FP32)
        e.set_fft_plan(1)
        ref, got = o.get_currents(), e.get_currents()
        for a in range(1, 4):
            assert rel(got[a], ref[a]) <= 5e-5, (a, rel(got[a], ref[a]))
    else:
        e, o, _ = make_wz_pair(shape, "ufg_rte_qf", precision=g.FP32)
        e.set_fft_plan(1)
        e.evolve_qf(1)
        o.evolve_qf(1)
        assert rel(e.get_psi()[1], o.get_psi()[1]) <= TOL_FP32_STEP
        e.evolve_qf(10)
        o.evolve_qf(10)
        assert rel(e.get_psi()[1], o.get_psi()[1]) <= 10 * TOL_FP32_STEP


def test_fp64_rejects_radix_plan_1(cuda_device, gpe_lib):
    e, _, _ = make_pair((16, 16, 32), "bec_ite")
    with pytest.raises(g.GPEError):
        e.set_fft_plan(1)
    e.set_fft_plan(0)
    assert e.get_fft_plan() == 0


@pytest.mark.parametrize("shape", [(16, 256, 16), (512, 16, 8), (8, 8, 512), (256, 256, 16)])
def test_fp32_long_pencils_against_oracle(cuda_device, gpe_lib, shape):
    """FP32 pencils of 256 and 512 points (persistent kinetic passes with prefetch, 256/1024-thread CTAs
    on x) against the FP64 oracle, plain and friction schedules."""
    for case in ("bec_rte", "ufg_rte_qf"):
        e, o, _ = make_pair(shape, case, precision=g.FP32)
        e.evolve_qf(2)
        o.evolve_qf(2)
        assert rel(e.get_psi()[1], o.get_psi()[1]) <= 2 * TOL_FP32_STEP, (case, rel(e.get_psi()[1], o.get_psi()[1]))
