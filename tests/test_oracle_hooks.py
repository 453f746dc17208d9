"""The oracle's user hooks (CPU): a hook header compiled for the host (oracle/hooks_host.cpp) stands in
for the oracle's built-in trap, functional and psi modifier.

* The default header (include/gpe_user_defined.h) reproduces the built-in harmonic trap and unitary-gas
  functional of the oracle (the mean field written as 0.185 cbrt(3 pi^2 rho)^2 instead of
  0.37 (3 pi^2 rho)^{2/3} / 2: equal to rounding).
* The hooks of tests/hooks/moving_trap_kick.h evaluate to their closed forms, with the run-time values
  (user parameters, lattice sides, d_dt, d_t0) that the oracle hands them.
* Its Woods-Saxon tube (VEXT 1) against the formula of dev/gpe_user_defined.h:520-558.
"""
import math
import os
import shutil

import numpy as np
import pytest

import oracle
from libcugpe_gb300 import configs

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
DEFAULT = os.path.join(ROOT, "include", "gpe_user_defined.h")
KICK = os.path.join(HERE, "hooks", "moving_trap_kick.h")

pytestmark = pytest.mark.skipif(shutil.which("g++") is None or not os.path.isdir("/usr/local/cuda/include"),
                                reason="needs g++ and the CUDA headers")


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("case", [(1.0, 0.0, 0.1), (0.0, 1.0, 0.0), (1.0, 0.0, 0.0)])
def test_default_header_hooks_reproduce_builtin_oracle(case):
    alpha, beta, qf = case
    shape = (8, 16, 16)
    params = [0.04, 0.05, 0.06, 0.0]
    hooks = oracle.Hooks(oracle.build_hooks(DEFAULT, "cpu_default", ["INTERACTIONS=0", "VEXT=0"]))
    psi = configs.random_state(shape, seed=5, npart=100.0, gamma=2.0)
    a = oracle.Oracle(shape, 0, alpha, beta, 0.05, 100.0, threads=2)
    b = oracle.Oracle(shape, 0, alpha, beta, 0.05, 100.0, threads=2)
    b.set_hooks(hooks)
    for o in (a, b):
        o.set_user_params(params)
        o.set_quantum_friction_coeff(qf)
        o.set_psi(0.0, psi)
        o.evolve_qf(3)
    assert rel(b.get_psi()[1], a.get_psi()[1]) <= 1e-14
    for x, y in zip(b.energy(), a.energy()):
        assert abs(x - y) <= 1e-13 * max(1.0, abs(y))


def test_kick_header_hooks_evaluate_their_closed_forms():
    lib = oracle.Hooks(oracle.build_hooks(KICK, "cpu_kick", ["INTERACTIONS=-1"])).L
    import ctypes
    lib.hooks_vext.restype = ctypes.c_double
    lib.hooks_vext.argtypes = [ctypes.c_uint] * 4
    lib.hooks_dedf.restype = ctypes.c_double
    lib.hooks_dedf.argtypes = [ctypes.c_double, ctypes.c_uint]
    lib.hooks_edf.restype = ctypes.c_double
    lib.hooks_edf.argtypes = [ctypes.c_double, ctypes.c_uint]
    lib.hooks_modify.argtypes = [ctypes.c_uint] * 4 + [ctypes.POINTER(ctypes.c_double)] * 2
    p = [0.06, 0.05, 0.07, 8.0, 1.5, 0.9, 0.3, 0.05]
    arr = (ctypes.c_double * len(p))(*p)
    nx, ny, nz, dt, t0 = 16, 32, 8, 0.05, 0.3
    lib.hooks_set(arr, len(p), nx, ny, nz, dt, t0, 1.0)
    for ix, iy, iz, it in ((3, 7, 2, 0), (15, 0, 7, 11), (8, 16, 4, 5)):
        t = t0 + it * dt
        x0 = p[4] * math.sin(p[5] * t)
        x, y, z = ix - nx // 2 - x0, iy - ny // 2, iz - nz // 2
        v = 0.5 * (p[0] ** 2 * x * x + p[1] ** 2 * y * y + p[2] ** 2 * z * z)
        assert lib.hooks_vext(ix, iy, iz, it) == pytest.approx(v, rel=1e-14)
        a = p[3] * (1.0 + p[6] * math.cos(p[5] * t))
        assert lib.hooks_dedf(0.7, it) == pytest.approx(4 * math.pi * a * 0.7, rel=1e-14)
        assert lib.hooks_edf(0.7, it) == pytest.approx(2 * math.pi * a * 0.49, rel=1e-14)
        re, im = ctypes.c_double(0.3), ctypes.c_double(-0.4)
        lib.hooks_modify(ix, iy, iz, it, ctypes.byref(re), ctypes.byref(im))
        k = p[7] * math.sin(2 * math.pi * it / 16.0) * (ix - nx // 2)
        w = complex(0.3, -0.4) * complex(math.cos(k), math.sin(k))
        assert re.value == pytest.approx(w.real, abs=1e-15) and im.value == pytest.approx(w.imag, abs=1e-15)


def test_woods_saxon_tube_hook():
    import ctypes
    lib = oracle.Hooks(oracle.build_hooks(DEFAULT, "cpu_tube", ["INTERACTIONS=0", "VEXT=1"])).L
    lib.hooks_vext.restype = ctypes.c_double
    lib.hooks_vext.argtypes = [ctypes.c_uint] * 4
    p = [2.0, 1.5, 6.0, 0.0]
    arr = (ctypes.c_double * 4)(*p)
    lib.hooks_set(arr, 4, 32, 32, 16, 0.05, 0.0, 100.0)
    for ix, iy, iz in ((16, 16, 3), (0, 5, 9), (31, 20, 0), (22, 16, 15)):
        r = math.hypot(ix - 16, iy - 16)
        v = p[0] * (1.0 - 1.0 / (1.0 + math.exp((r - p[2]) / p[1])))
        assert lib.hooks_vext(ix, iy, iz, 7) == pytest.approx(v, rel=1e-14, abs=1e-15)
