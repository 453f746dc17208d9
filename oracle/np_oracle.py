"""Second restatement of libcugpe's step sequence, with numpy's FFT.

TEST INFRASTRUCTURE ONLY (small lattices).  It exists to cross-check the C
restatement (gpe_oracle.c) with an independent FFT.  Same citations:
dev/gpe_engine.cu:126-220 (tables), 716-933 (kernels), 1030-1109 (loop),
1669-1705 (energy); dev/gpe_user_defined.h:118-135, 305-322, 488-513.
"""
from __future__ import annotations

import numpy as np


def kgrid(n: int) -> np.ndarray:
    i = np.arange(n)
    return 2.0 * np.pi / n * np.where(i < n // 2, i, i - n).astype(np.float64)


class NpOracle:
    def __init__(self, shape, interactions, alpha, beta, dt, npart, params, qf=0.0):
        self.shape = tuple(shape)
        self.inter = interactions
        self.gamma = 1.0 if interactions == -1 else 2.0
        self.alpha, self.beta, self.dt, self.npart = alpha, beta, dt, npart
        self.p = np.zeros(32)
        self.p[: len(params)] = params
        n = int(np.prod(shape))
        self.n = n
        self.qf = qf / (self.gamma * n) if qf != 0.0 else 0.0
        self.c3 = (self.gamma * 0.5 * dt) / complex(-beta, alpha)
        kx, ky, kz = (kgrid(s) for s in shape)
        self.k2 = kx[:, None, None] ** 2 + ky[None, :, None] ** 2 + kz[None, None, :] ** 2
        g2 = self.gamma ** 2
        ex, ey, ez = (np.exp(self.c3 * k * k / g2) for k in (kx, ky, kz))
        self.expT = ex[:, None, None] * ey[None, :, None] * (ez / n)[None, None, :]
        idx = [np.arange(s) - (s // 2) for s in shape]
        X, Y, Z = np.meshgrid(*idx, indexing="ij")
        wx, wy, wz = self.p[:3]
        self.vext = 0.5 * X * X * wx * wx + 0.5 * Y * Y * wy * wy + 0.5 * Z * Z * wz * wz
        self.it = 0
        self.psi = np.zeros(shape, dtype=np.complex128)

    def dEDFdn(self, rho):
        if self.inter == -1:
            return 4 * np.pi * self.p[3] * rho
        if self.inter == 0:
            return 0.37 * np.power(3.0 * np.pi * np.pi * rho, 2.0 / 3.0) / 2.0
        raise NotImplementedError

    def EDF(self, rho):
        if self.inter == -1:
            return 2 * np.pi * self.p[3] * rho * rho
        if self.inter == 0:
            return 0.37 * 0.6 * rho * np.power(3.0 * np.pi * np.pi * rho, 2.0 / 3.0) / 2.0
        raise NotImplementedError

    def density(self, psi):
        return self.gamma * (psi.real ** 2 + psi.imag ** 2)

    def normalize(self, psi):
        s = self.density(psi).sum()
        psi *= np.sqrt(self.npart / s)
        return s

    def kinetic(self, psi):
        return np.fft.ifftn(np.fft.fftn(psi) * self.expT) * self.n

    def qf_potential(self, psi):
        w = np.fft.ifftn(np.fft.fftn(psi) * (self.qf * self.k2)) * self.n
        a = np.conj(psi)
        return (a.real * w.imag + a.imag * w.real) / (self.density(psi) + 1e-12)

    def evolve_qf(self, nt):
        mu = 0.0
        for _ in range(nt):
            qf = self.qf != 0.0
            V = self.vext + self.dEDFdn(self.density(self.psi))
            if qf:
                V = V + self.qf_potential(self.psi)
            psi2 = self.kinetic(self.psi * np.exp(self.c3 * V))
            if self.beta == 0.0 and not qf:
                pp = psi2 * np.exp(self.c3 * V)
                Vn = 0.5 * (V + self.vext + self.dEDFdn(self.density(pp)))
            else:
                psi2 = psi2 * np.exp(self.c3 * V)
                if self.beta != 0.0:
                    self.normalize(psi2)
                Vn = V + self.vext + self.dEDFdn(self.density(psi2))
                if qf:
                    Vn = Vn + self.qf_potential(self.psi)
                Vn = 0.5 * Vn
            wrkC = np.exp(self.c3 * Vn)
            self.psi = self.kinetic(self.psi * wrkC) * wrkC
            if self.beta != 0.0:
                norm = self.normalize(self.psi)
                mu = -0.5 * np.log(norm / self.npart) / self.dt
            self.it += 1
        return mu

    def energy(self):
        if self.beta == 0.0:
            self.normalize(self.psi)
        rho = self.density(self.psi)
        eext = float((rho * self.vext).sum())
        eint = float(self.EDF(rho).sum())
        w = np.fft.ifftn(np.fft.fftn(self.psi) * self.k2 / (2.0 * self.gamma * self.n)) * self.n
        ekin = float((self.psi.real * w.real + self.psi.imag * w.imag).sum())
        return ekin, eint, eext
