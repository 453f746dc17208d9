"""Batched solver: independent condensates of uneven lattice sizes stepped by
one launch per fused pass.  Each condensate must evolve exactly as it does
alone (same pass body, same CTA shape), with its own parameters, norm and mu."""
import numpy as np
import pytest

import oracle
import libcugpe_gb300 as g
from libcugpe_gb300 import configs

pytestmark = pytest.mark.gpu

SHAPES = [(32, 32, 32), (64, 32, 32), (32, 64, 64), (64, 64, 64), (128, 32, 32)]


def params_for(i):
    rng = np.random.default_rng(100 + i)
    w = 0.05 * rng.uniform(0.8, 1.25)
    return [0.05, 0.05, w, rng.uniform(5.0, 20.0)]


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_batch_matches_single_engines_exactly(cuda_device, gpe_lib):
    b = g.Batch(SHAPES, interactions=-1, alpha=0.0, beta=1.0, dt=0.05, npart=[1.0] * len(SHAPES))
    singles, psis = [], []
    for i, s in enumerate(SHAPES):
        psi = configs.random_state(s, seed=30 + i)
        psis.append(psi)
        b.engines[i].set_user_params(params_for(i))
        b.engines[i].set_psi(0.0, psi)
        e = g.Engine(s, -1, 0.0, 1.0, 0.05, 1.0, precision=g.FP32)
        e.set_user_params(params_for(i))
        e.set_psi(0.0, psi)
        singles.append(e)
    b.evolve(37)
    mu_b, _ = b.chemical_potentials()
    for i, e in enumerate(singles):
        mu = e.evolve_qf(37)
        assert np.array_equal(b.engines[i].get_psi()[1], e.get_psi()[1]), i
        assert mu_b[i] == mu
        assert b.engines[i].get_psi()[0] == pytest.approx(37 * 0.05)
    assert b.kernel_launches() >= 37 * 6


def test_batch_against_fp64_oracle_and_inactive(cuda_device, gpe_lib):
    shapes = SHAPES[:3]
    b = g.Batch(shapes, interactions=-1, alpha=0.0, beta=1.0, dt=0.05)
    psis = []
    for i, s in enumerate(shapes):
        psis.append(configs.random_state(s, seed=40 + i))
        b.engines[i].set_user_params(params_for(i))
        b.engines[i].set_psi(0.0, psis[i])
    b.set_active(1, False)
    b.evolve(10)
    assert np.array_equal(b.engines[1].get_psi()[1], psis[1].astype(np.complex64).astype(np.complex128))
    for i in (0, 2):
        o = oracle.Oracle(shapes[i], -1, 0.0, 1.0, 0.05, 1.0, threads=4)
        o.set_user_params(params_for(i))
        o.set_psi(0.0, psis[i])
        o.evolve_qf(10)
        assert rel(b.engines[i].get_psi()[1], o.get_psi()[1]) <= 2e-5 * 10


def test_batch_radix_plan_1_against_fp64_oracle(cuda_device, gpe_lib):
    """The batched launches under the alternative radix plan (every condensate's pencils at the other
    point count per thread) against the FP64 oracle."""
    shapes = [(32, 32, 32), (64, 32, 32), (128, 32, 32), (32, 256, 32)]
    b = g.Batch(shapes, interactions=-1, alpha=0.0, beta=1.0, dt=0.05)
    b.set_fft_plan(1)
    psis = []
    for i, s in enumerate(shapes):
        psis.append(configs.random_state(s, seed=60 + i))
        b.engines[i].set_user_params(params_for(i))
        b.engines[i].set_psi(0.0, psis[i])
    b.evolve(10)
    for i, s in enumerate(shapes):
        o = oracle.Oracle(s, -1, 0.0, 1.0, 0.05, 1.0, threads=4)
        o.set_user_params(params_for(i))
        o.set_psi(0.0, psis[i])
        o.evolve_qf(10)
        assert rel(b.engines[i].get_psi()[1], o.get_psi()[1]) <= 2e-5 * 10, i


def test_batch_rejects_unsupported(cuda_device, gpe_lib):
    with pytest.raises(g.GPEError):
        g.Batch([(16, 16, 16)], precision=g.FP32)
    with pytest.raises(g.GPEError):
        g.Batch([(32, 32, 32)], precision=g.FP64)


def test_batch_autotune_keeps_results(cuda_device, gpe_lib):
    """Item order and graph length change neither the state (restored) nor the bits of later steps."""
    def make():
        b = g.Batch(SHAPES, interactions=-1, alpha=0.0, beta=1.0, dt=0.05, npart=[1.0] * len(SHAPES))
        for i, s in enumerate(SHAPES):
            b.engines[i].set_user_params(params_for(i))
            b.engines[i].set_psi(0.0, configs.random_state(s, seed=50 + i))
        return b
    b1, b2 = make(), make()
    choice = b1.autotune(8)
    assert choice["order"] in (0, 1) and choice["graph_steps"] in (8, 16, 32) and choice["fft_plan"] in (0, 1)
    b2.set_fft_plan(choice["fft_plan"])  # item order and graph length leave the bits unchanged
    b1.evolve(21)
    b2.evolve(21)
    for i in range(len(SHAPES)):
        assert np.array_equal(b1.engines[i].get_psi()[1], b2.engines[i].get_psi()[1]), i


def host_side_solve(e, max_steps, check, tol):
    """The convergence rule of gpe_gb_batch_solve evaluated on the host for one engine: every `check`
    steps the mean of mu over the interval is compared with the previous interval's mean."""
    steps, prev = 0, None
    start = e.chemical_potential()[1]
    while steps < max_steps:
        e.evolve_qf(check)
        steps += check
        s = e.chemical_potential()[1]
        mean = (s - start) / check
        if prev is not None and abs(mean - prev) < tol * check:
            return steps, mean
        prev, start = mean, s
    return -1, None


def test_batch_solve_retires_on_device_like_the_host_rule(cuda_device, gpe_lib):
    """gpe_gb_batch_solve: each condensate stops at the step the host-side rule gives, with the same
    interval mean, and ends in the same state as the same solve on its own engine."""
    shapes = [(32, 32, 32), (64, 32, 32), (32, 64, 64), (32, 32, 64)]
    tol, check, max_steps = [3e-7, 1e-7, 2e-7, 1e-7], 25, 3000
    b = g.Batch(shapes, interactions=-1, alpha=0.0, beta=1.0, dt=0.05)
    singles = []
    for i, s in enumerate(shapes):
        psi = configs.random_state(s, seed=70 + i)
        b.engines[i].set_user_params(params_for(i))
        b.engines[i].set_psi(0.0, psi)
        e = g.Engine(s, -1, 0.0, 1.0, 0.05, 1.0, precision=g.FP32)
        e.set_user_params(params_for(i))
        e.set_psi(0.0, psi)
        singles.append(e)
    steps, mu = b.solve(max_steps, check, tol)
    for i, e in enumerate(singles):
        st, mean = host_side_solve(e, max_steps, check, tol[i])
        assert st > 0 and steps[i] == st, (i, steps[i], st)
        assert mu[i] == pytest.approx(mean, rel=1e-12, abs=1e-15)
        assert np.array_equal(b.engines[i].get_psi()[1], e.get_psi()[1]), i
        assert b.engines[i].get_psi()[0] == pytest.approx(st * 0.05)
    assert len(set(steps.tolist())) > 1  # condensates retire at different steps
    # the test is cleared afterwards: the batch evolves every condensate again
    before = [b.engines[i].get_psi()[1] for i in range(len(shapes))]
    b.evolve(3)
    for i in range(len(shapes)):
        assert not np.array_equal(b.engines[i].get_psi()[1], before[i]), i


def test_batch_solve_reports_unconverged(cuda_device, gpe_lib):
    b = g.Batch([(32, 32, 32)], interactions=-1, alpha=0.0, beta=1.0, dt=0.05)
    b.engines[0].set_user_params(params_for(0))
    b.engines[0].set_psi(0.0, configs.random_state((32, 32, 32), seed=80))
    steps, mu = b.solve(40, 10, 0.0)
    assert steps[0] == -1 and np.isfinite(mu[0])
    assert b.engines[0].get_psi()[0] == pytest.approx(40 * 0.05)


def test_batch_with_quantum_friction(cuda_device, gpe_lib):
    """Imaginary time with quantum friction in a batch (the first step runs per condensate, forming the
    friction Laplacian): against each condensate on its own and against the FP64 oracle."""
    shapes = [(32, 32, 32), (64, 32, 32), (32, 32, 64)]
    qf = 0.2
    b = g.Batch(shapes, interactions=-1, alpha=0.0, beta=1.0, dt=0.05)
    for i, s in enumerate(shapes):
        psi = configs.random_state(s, seed=90 + i)
        b.engines[i].set_user_params(params_for(i))
        b.engines[i].set_quantum_friction_coeff(qf)
        b.engines[i].set_psi(0.0, psi)
    b.evolve(12)
    b.evolve(7)
    for i, s in enumerate(shapes):
        psi = configs.random_state(s, seed=90 + i)
        e = g.Engine(s, -1, 0.0, 1.0, 0.05, 1.0, precision=g.FP32)
        e.set_user_params(params_for(i))
        e.set_quantum_friction_coeff(qf)
        e.set_psi(0.0, psi)
        e.evolve_qf(12)
        e.evolve_qf(7)
        assert rel(b.engines[i].get_psi()[1], e.get_psi()[1]) <= 2e-6, i
        o = oracle.Oracle(s, -1, 0.0, 1.0, 0.05, 1.0, threads=4)
        o.set_user_params(params_for(i))
        o.set_quantum_friction_coeff(qf)
        o.set_psi(0.0, psi)
        o.evolve_qf(19)
        assert rel(b.engines[i].get_psi()[1], o.get_psi()[1]) <= 2e-5 * 19, i
        e.close()


def test_batch_refuses_mixed_steps(cuda_device, gpe_lib):
    b = g.Batch([(32, 32, 32), (32, 32, 32)], interactions=-1, alpha=0.0, beta=1.0, dt=0.05)
    for i in range(2):
        b.engines[i].set_user_params(params_for(i))
        b.engines[i].set_psi(0.0, configs.random_state((32, 32, 32), seed=95 + i))
    b.engines[1].set_quantum_friction_coeff(0.1)
    with pytest.raises(g.GPEError):
        b.evolve(2)
