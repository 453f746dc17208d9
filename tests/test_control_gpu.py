"""Adjoint gradients of the optimal-control loss against a taped FP64
restatement (autograd on CPU) and against central finite differences."""
import numpy as np
import pytest

import libcugpe_gb300 as g
from libcugpe_gb300 import configs
from libcugpe_gb300.control import ControlProblem

pytestmark = pytest.mark.gpu


def gaussians(shape, centres, sigma):
    X, Y, Z = configs.grid(shape)
    return np.stack([np.exp(-((X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2) / (2 * sigma * sigma))
                     for c in centres])


def small_problem(seed=0):
    rng = np.random.default_rng(seed)
    shape = (16, 16, 16)
    params = [0.1, 0.1, 0.12, 2.0]
    dt, nsteps, sps, ck = 0.1, 40, 10, 10
    basis = gaussians(shape, rng.uniform(-3, 3, (3, 3)), 2.0)
    psi0 = configs.random_state(shape, seed=seed)
    target = configs.random_state(shape, seed=seed + 1, phase=False)
    controls = 0.02 * rng.standard_normal((nsteps // sps, basis.shape[0]))
    return shape, params, dt, nsteps, sps, ck, basis, psi0, target, controls


def make(shape, params, dt, nsteps, sps, ck, basis, target):
    e = g.Engine(shape, -1, 1.0, 0.0, dt, 1.0, precision=g.FP64)
    e.set_user_params(params)
    return e, ControlProblem(e, basis, nsteps // sps, sps, nsteps, target, checkpoint_every=ck)


def test_adjoint_matches_taped_restatement(cuda_device, gpe_lib):
    import torch
    from oracle.taped_control import loss_taped
    shape, params, dt, nsteps, sps, ck, basis, psi0, target, controls = small_problem()
    e, cp = make(shape, params, dt, nsteps, sps, ck, basis, target)
    loss, grad = cp.loss_and_grad(controls, psi0)
    c = torch.tensor(controls, dtype=torch.float64, requires_grad=True)
    ref = loss_taped(c, basis, psi0, target, params, dt, nsteps, sps)
    ref.backward()
    assert loss == pytest.approx(ref.item(), rel=1e-10, abs=1e-12)
    gref = c.grad.numpy()
    assert np.linalg.norm(grad - gref) <= 1e-8 * np.linalg.norm(gref)


def test_adjoint_matches_central_differences(cuda_device, gpe_lib):
    shape, params, dt, nsteps, sps, ck, basis, psi0, target, controls = small_problem(seed=3)
    e, cp = make(shape, params, dt, nsteps, sps, ck, basis, target)
    _, grad = cp.loss_and_grad(controls, psi0)
    h = 1e-4
    rng = np.random.default_rng(9)
    for _ in range(5):
        s, k = rng.integers(controls.shape[0]), rng.integers(controls.shape[1])
        cp_, cm_ = controls.copy(), controls.copy()
        cp_[s, k] += h
        cm_[s, k] -= h
        fd = (cp.loss(cp_, psi0) - cp.loss(cm_, psi0)) / (2 * h)
        assert abs(fd - grad[s, k]) <= 1e-5 * max(abs(grad[s, k]), 1e-3 * np.abs(grad).max()), (s, k, fd, grad[s, k])


def test_torch_autograd_function(cuda_device, gpe_lib):
    import torch
    from libcugpe_gb300.control import ControlLoss
    shape, params, dt, nsteps, sps, ck, basis, psi0, target, controls = small_problem(seed=5)
    e, cp = make(shape, params, dt, nsteps, sps, ck, basis, target)
    c = torch.tensor(controls, dtype=torch.float64, requires_grad=True)
    loss = ControlLoss.apply(c, cp, psi0)
    (2.0 * loss).backward()
    _, grad = cp.loss_and_grad(controls, psi0)
    assert np.allclose(c.grad.numpy(), 2.0 * grad, rtol=1e-12, atol=0)
