"""Workload builders (libcugpe_gb300/configs.py): oscillator units restated in the reference's lattice
units, normalisation, the vortex phases.  CPU only."""
import numpy as np
import pytest

from libcugpe_gb300 import configs


def winding(phase2d, cx, cy, r):
    """Phase winding (in turns) around a square loop of half-side r centred on (cx, cy)."""
    pts = [(cx - r + i, cy - r) for i in range(2 * r)] + [(cx + r, cy - r + i) for i in range(2 * r)] + \
          [(cx + r - i, cy + r) for i in range(2 * r)] + [(cx - r, cy + r - i) for i in range(2 * r)]
    w = 0.0
    for (a, b), (c, d) in zip(pts, pts[1:] + pts[:1]):
        w += (phase2d[c, d] - phase2d[a, b] + np.pi) % (2 * np.pi) - np.pi
    return w / (2 * np.pi)


def test_bec_ground_state_units():
    """64^3, dx = 0.25, omega = 1, gN = 100, dt = 1e-3: omega' = omega dx^2, dt' = dt/dx^2,
    4 pi a' = gN/dx, sum |psi|^2 = 1."""
    w = configs.bec_ground_state_ite(n=64)
    assert w.shape == (64, 64, 64) and (w.interactions, w.alpha, w.beta, w.npart) == (-1, 0.0, 1.0, 1.0)
    assert w.params[:3] == [0.0625] * 3
    assert w.params[3] == pytest.approx(400.0 / (4.0 * np.pi))
    assert w.dt == pytest.approx(0.016)
    assert np.sum(np.abs(w.psi0) ** 2) == pytest.approx(1.0, rel=1e-12)
    assert w.gamma == 1.0
    again = configs.bec_ground_state_ite(n=64)
    assert np.array_equal(w.psi0, again.psi0)


def test_ufg_vortex_workload_units_and_phase():
    """The 128^3 workload's physics on a 32^3 lattice: omega' = omega dx^2, dt' = dt/dx^2, dimers
    (Gamma = 2) normalised to npart, one vortex of charge +1 on the z axis."""
    w = configs.ufg_vortex_rte_qf(n=32)
    assert (w.interactions, w.alpha, w.beta, w.qf, w.gamma) == (0, 1.0, 0.0, 0.1, 2.0)
    assert w.params == pytest.approx([0.04, 0.04, 0.06, 0.0])
    assert w.dt == pytest.approx(0.125)
    assert 2.0 * np.sum(np.abs(w.psi0) ** 2) == pytest.approx(1000.0, rel=1e-12)
    ph = np.angle(w.psi0[:, :, 16])
    assert winding(ph, 16, 16, 4) == pytest.approx(1.0, abs=1e-9)
    assert winding(ph, 6, 6, 3) == pytest.approx(0.0, abs=1e-9)


def test_cooling_workload_vortex_lines():
    """Straight lines along z at seeded positions inside the disk: total winding around a loop that
    encloses the disk equals the number of lines."""
    n, lines = 64, 8
    w = configs.ufg_vortex_lines(n=n, dx=0.4, lines=lines, radius=4.0)
    assert w.params[:3] == pytest.approx([0.16] * 3) and w.dt == pytest.approx(2e-3 / 0.16)
    assert 2.0 * np.sum(np.abs(w.psi0) ** 2) == pytest.approx(5.0e4, rel=1e-12)
    ph = np.angle(w.psi0[:, :, n // 2])
    assert winding(ph, n // 2, n // 2, 14) == pytest.approx(lines, abs=1e-9)
    other = w.psi0[:, :, n // 2 + 5]  # the lines are straight: the same phase in another plane
    mask = np.abs(other) > 0
    assert mask.sum() > 100 and np.allclose(np.angle(other)[mask], ph[mask])


def test_random_state_is_seeded_and_normalised():
    a = configs.random_state((16, 8, 32), seed=5, npart=10.0, gamma=2.0)
    b = configs.random_state((16, 8, 32), seed=5, npart=10.0, gamma=2.0)
    c = configs.random_state((16, 8, 32), seed=6, npart=10.0, gamma=2.0)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert 2.0 * np.sum(np.abs(a) ** 2) == pytest.approx(10.0, rel=1e-12)
