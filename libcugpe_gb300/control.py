"""Optimal control of a real-time condensate through the GPU adjoint.

``ControlProblem`` wraps the C ABI's gpe_gb_control_*: the loss
L(c) = 1 - |<psi_target|psi(T)>|^2 of the discrete real-time evolution
under a time-sliced potential trap + sum_k c[s, k] basis_k(x), and its exact
gradient from the hand-written adjoint of the split step (FP64).
``ControlLoss`` exposes it to PyTorch as an autograd Function.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import Engine, _check, _dp, _lib


class ControlProblem:
    def __init__(self, engine: Engine, basis, nslices, steps_per_slice, nsteps, psi_target, checkpoint_every=100):
        self.engine = engine
        self.basis = np.ascontiguousarray(basis, dtype=np.float64)
        self.nbasis = self.basis.shape[0]
        self.nslices = int(nslices)
        tgt = np.ascontiguousarray(psi_target, dtype=np.complex128)
        h = ctypes.c_void_p()
        _check(_lib().gpe_gb_control_create(ctypes.byref(h), engine.handle, self.nbasis, _dp(self.basis),
                                            self.nslices, int(steps_per_slice), int(nsteps), int(checkpoint_every),
                                            _dp(tgt.view(np.float64))), "gpe_gb_control_create")
        self._h = h

    def _prep(self, controls, psi0):
        c = np.ascontiguousarray(controls, dtype=np.float64).reshape(self.nslices, self.nbasis)
        p = np.ascontiguousarray(psi0, dtype=np.complex128)
        return c, p

    def loss(self, controls, psi0) -> float:
        c, p = self._prep(controls, psi0)
        out = ctypes.c_double()
        _check(_lib().gpe_gb_control_loss(self._h, _dp(c), _dp(p.view(np.float64)), ctypes.byref(out)), "control_loss")
        return out.value

    def loss_and_grad(self, controls, psi0):
        c, p = self._prep(controls, psi0)
        out = ctypes.c_double()
        g = np.zeros_like(c)
        _check(_lib().gpe_gb_control_loss_grad(self._h, _dp(c), _dp(p.view(np.float64)), ctypes.byref(out), _dp(g)),
               "control_loss_grad")
        return out.value, g

    def close(self):
        if getattr(self, "_h", None):
            _lib().gpe_gb_control_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _function():
    import torch

    class ControlLoss(torch.autograd.Function):
        """loss = ControlLoss.apply(controls, problem, psi0); backward runs the GPU adjoint."""

        @staticmethod
        def forward(ctx, controls, problem, psi0):
            loss, grad = problem.loss_and_grad(controls.detach().cpu().numpy(), psi0)
            ctx.save_for_backward(torch.from_numpy(grad).to(controls.device, controls.dtype))
            return torch.tensor(loss, dtype=controls.dtype, device=controls.device)

        @staticmethod
        def backward(ctx, gout):
            (grad,) = ctx.saved_tensors
            return gout * grad, None, None

    return ControlLoss


def __getattr__(name):
    if name == "ControlLoss":
        return _function()
    raise AttributeError(name)
