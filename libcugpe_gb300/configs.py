"""Workloads of the split-step evolution, restated in the reference's lattice units.

The reference engine works in lattice units with dx = 1: k_i = 2 pi i / n
(dev/gpe_engine.cu:147-175) and the trap uses the index offset i - n/2 with
no dx (dev/gpe_user_defined.h:500-510).  A problem posed in oscillator units
with spacing dx maps to lattice units as
    x' = x/dx,  t' = t/dx^2,  omega' = omega dx^2,  psi'_i = phi(x_i) dx^{3/2},
    4 pi a' = g N / dx  (contact BEC with npart = 1, sum |psi'|^2 = 1),
and the unitary-Fermi-gas functional is scale invariant.  Initial states are
seeded with numpy's PCG64 (default_rng(seed)).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class Workload:
    name: str
    shape: tuple
    interactions: int
    alpha: float
    beta: float
    dt: float           # lattice units
    npart: float
    params: list        # [omega_x', omega_y', omega_z', a_scat']
    qf: float = 0.0
    steps: int = 100
    psi0: np.ndarray | None = field(default=None, repr=False)

    @property
    def gamma(self) -> float:
        return 1.0 if self.interactions < 0 else 2.0  # particles (-1, -2) or dimers (0, 1)


def grid(shape, dx=1.0):
    """Coordinates (x, y, z) of the lattice points, centred as the reference trap (i - n/2)."""
    axes = [(np.arange(n) - n // 2) * dx for n in shape]
    return np.meshgrid(*axes, indexing="ij")


def normalise(psi, npart, gamma):
    s = gamma * np.sum(np.abs(psi) ** 2)
    return psi * np.sqrt(npart / s)


def bec_ground_state_ite(n=64, dx=0.25, omega=1.0, gN=100.0, dt=1e-3, steps=2000, seed=0, width=1.0) -> Workload:
    """3D BEC imaginary-time ground state: Gaussian of width `width` times (1 + 0.01 u), u ~ U[-1, 1]."""
    rng = np.random.default_rng(seed)
    shape = (n, n, n)
    X, Y, Z = grid(shape, dx)
    psi = np.exp(-(X * X + Y * Y + Z * Z) / (2.0 * width * width)) * (1.0 + 0.01 * rng.uniform(-1.0, 1.0, shape))
    psi = normalise(psi.astype(np.complex128), 1.0, 1.0)
    w = omega * dx * dx
    a = gN / dx / (4.0 * np.pi)
    return Workload("bec_ite_%d" % n, shape, -1, 0.0, 1.0, dt / (dx * dx), 1.0, [w, w, w, a], 0.0, steps, psi)


def ufg_vortex_rte_qf(n=128, dx=0.2, omega=(1.0, 1.0, 1.5), xi_qf=0.1, dt=5e-3, steps=10000, npart=1000.0,
                      seed=0) -> Workload:
    """Unitary Fermi gas (dimers) real-time evolution with quantum friction.

    Initial state: Thomas-Fermi profile of the reference functional
    (0.37 (3 pi^2 rho)^{2/3}/2 + V = mu) times the vortex phase atan2(y, x)
    and a 1e-3 seeded perturbation; the caller may relax it with a short ITE.
    """
    rng = np.random.default_rng(seed)
    shape = (n, n, n)
    w = [o * dx * dx for o in omega]
    idx = [(np.arange(s) - s // 2).astype(np.float64) for s in shape]
    X, Y, Z = np.meshgrid(*idx, indexing="ij")
    V = 0.5 * (X * X * w[0] ** 2 + Y * Y * w[1] ** 2 + Z * Z * w[2] ** 2)

    def tf_density(mu):
        return np.maximum(mu - V, 0.0) ** 1.5 / (0.185 ** 1.5 * 3.0 * np.pi ** 2)

    lo, hi = 0.0, float(V.max())
    for _ in range(100):  # mu such that sum rho = npart
        mid = 0.5 * (lo + hi)
        if tf_density(mid).sum() > npart:
            hi = mid
        else:
            lo = mid
    rho = tf_density(0.5 * (lo + hi))
    amp = np.sqrt(rho / 2.0) * (1.0 + 1e-3 * rng.uniform(-1.0, 1.0, shape))
    psi = (amp * np.exp(1j * np.arctan2(Y + 0.5, X + 0.5))).astype(np.complex128)
    psi = normalise(psi, npart, 2.0)
    return Workload("ufg_rte_qf_%d" % n, shape, 0, 1.0, 0.0, dt / (dx * dx), npart, [w[0], w[1], w[2], 0.0],
                    xi_qf, steps, psi)


def ufg_vortex_lines(n=512, dx=0.1, omega=1.0, xi_qf=0.2, dt=2e-3, steps=5000, npart=5.0e4, lines=8,
                     radius=4.0, seed=0) -> Workload:
    """Large cooling run: unitary Fermi gas (dimers) with quantum friction, isotropic trap, Thomas-Fermi
    profile of the reference functional times `lines` straight vortex lines along z, of charge +1 at
    seeded positions uniform in the disk of `radius` (oscillator units) of the x-y plane.  npart is not
    fixed by the problem statement; 5e4 gives a Thomas-Fermi radius of about 8 oscillator lengths."""
    rng = np.random.default_rng(seed)
    shape = (n, n, n)
    w = omega * dx * dx
    ii = np.arange(n, dtype=np.int64) - n // 2
    idx = ii.astype(np.float64)
    X, Y = idx[:, None], idx[None, :]
    # the trap depends on the integer r^2 only: bisect mu on the histogram of r^2
    r2 = (ii[:, None, None] ** 2 + ii[None, :, None] ** 2).astype(np.int32) + (ii[None, None, :] ** 2).astype(np.int32)
    count = np.bincount(r2.ravel())
    v = 0.5 * w * w * np.arange(count.size, dtype=np.float64)

    def tf_density(mu):
        return np.maximum(mu - v, 0.0) ** 1.5 / (0.185 ** 1.5 * 3.0 * np.pi ** 2)

    lo, hi = 0.0, float(v.max())
    for _ in range(80):
        mid = 0.5 * (lo + hi)
        if (count * tf_density(mid)).sum() > npart:
            hi = mid
        else:
            lo = mid
    amp = np.sqrt(tf_density(0.5 * (lo + hi)) / 2.0)[r2]
    del r2
    rr = radius / dx * np.sqrt(rng.uniform(0.0, 1.0, lines))
    th = rng.uniform(0.0, 2.0 * np.pi, lines)
    phase = np.zeros((n, n))
    for r, t in zip(rr, th):
        phase += np.arctan2(Y - r * np.sin(t) + 0.5, X - r * np.cos(t) + 0.5)
    psi = (amp * np.exp(1j * phase)[:, :, None]).astype(np.complex128)
    del amp
    psi = normalise(psi, npart, 2.0)
    return Workload("ufg_cool_%d" % n, shape, 0, 1.0, 0.0, dt / (dx * dx), npart, [w, w, w, 0.0], xi_qf, steps,
                    psi)


def random_state(shape, seed=0, npart=1.0, gamma=1.0, width=None, phase=True):
    """Seeded smooth complex test state for parity checks."""
    rng = np.random.default_rng(seed)
    X, Y, Z = grid(shape)
    wdt = width or (max(shape) / 4.0)
    amp = np.exp(-(X * X + Y * Y + Z * Z) / (2.0 * wdt * wdt)) * (1.0 + 0.05 * rng.uniform(-1.0, 1.0, shape))
    ph = 0.3 * rng.standard_normal(3)
    psi = amp * (np.exp(1j * (ph[0] * X + ph[1] * Y + ph[2] * Z) / wdt) if phase else 1.0)
    return normalise(psi.astype(np.complex128), npart, gamma)
