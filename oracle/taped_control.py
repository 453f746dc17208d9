"""Taped FP64 restatement of the controlled real-time step (small grids).

TEST INFRASTRUCTURE ONLY: the reference for the GPU adjoint.  The forward
step follows dev/gpe_engine.cu:719-742 (Vstep1), 876-891 (kinetic), 770-797
(Vstep2), 866-874 (Vstep3) for a contact BEC in real time (c3 = -i dt/2),
with the time-sliced potential trap + sum_k c[s, k] basis_k; PyTorch's
autograd tapes it and gives the exact gradient of the discrete map.
"""
from __future__ import annotations

import numpy as np
import torch


def kgrid(n):
    i = np.arange(n)
    return 2.0 * np.pi / n * np.where(i < n // 2, i, i - n).astype(np.float64)


def trap(shape, w):
    idx = [(np.arange(s) - s // 2).astype(np.float64) for s in shape]
    X, Y, Z = np.meshgrid(*idx, indexing="ij")
    return 0.5 * X * X * w[0] * w[0] + 0.5 * Y * Y * w[1] * w[1] + 0.5 * Z * Z * w[2] * w[2]


def loss_taped(controls, basis, psi0, target, params, dt, nsteps, steps_per_slice):
    """controls: torch (nslices, nbasis) requires_grad; returns the loss tensor."""
    shape = psi0.shape
    c3y = -0.5 * dt
    g = 4 * np.pi * params[3]
    kx, ky, kz = (kgrid(s) for s in shape)
    k2 = kx[:, None, None] ** 2 + ky[None, :, None] ** 2 + kz[None, None, :] ** 2
    kin = torch.from_numpy(np.exp(1j * c3y * k2))
    vt = torch.from_numpy(trap(shape, params[:3]))
    B = torch.from_numpy(np.ascontiguousarray(basis))
    nslices = controls.shape[0]
    fields = torch.einsum("sk,kxyz->sxyz", controls, B)

    def vext(it):
        return vt + fields[min(it // steps_per_slice, nslices - 1)]

    def K(a):
        return torch.fft.ifftn(torch.fft.fftn(a) * kin)

    psi = torch.from_numpy(np.ascontiguousarray(psi0, dtype=np.complex128))
    for it in range(nsteps):
        V = vext(it) + g * psi.abs() ** 2
        E = torch.exp(1j * c3y * V)
        P = E * K(E * psi)
        W = 0.5 * (V + vext(it + 1) + g * P.abs() ** 2)
        F = torch.exp(1j * c3y * W)
        psi = F * K(F * psi)
    o = torch.sum(torch.conj(torch.from_numpy(target)) * psi)
    return 1.0 - o.abs() ** 2
