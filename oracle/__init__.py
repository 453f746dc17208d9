"""CPU FP64 oracle for libcugpe's split-step evolution.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` may import this package, and only as the
checker or the timed CPU baseline.  The product (``libcugpe_gb300``) never
imports it and has no CPU fallback.

``gpe_oracle.c`` restates the reference algorithm (citations in its header);
``np_oracle.py`` restates it again with numpy's FFT so the C restatement's own
FFT can be cross-checked; ``build_ref.py`` builds the reference engine itself
(on a machine with a GPU) for golden vectors and reference timings.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libgpe_oracle.so")

INTER_GAMMA = {-2: 1.0, -1: 1.0, 0: 2.0, 1: 2.0}


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "gpe_oracle.c")
    if not force and os.path.isfile(LIB) and os.path.getmtime(LIB) > os.path.getmtime(src):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    # -ffp-contract=off keeps results identical on x86-64 and aarch64 hosts
    cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=gnu99",
           src, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        L = ctypes.CDLL(path)
        vp, d, i = ctypes.c_void_p, ctypes.c_double, ctypes.c_int
        dp = ctypes.POINTER(ctypes.c_double)
        L.oracle_create.restype = vp
        L.oracle_create.argtypes = [i, i, i, i, d, d, d, d, d]
        L.oracle_destroy.argtypes = [vp]
        L.oracle_set_threads.argtypes = [vp, i]
        L.oracle_max_threads.restype = i
        L.oracle_set_user_params.argtypes = [vp, i, dp]
        L.oracle_set_user_params.restype = i
        L.oracle_change_alpha_beta.argtypes = [vp, d, d]
        L.oracle_set_time.argtypes = [vp, d]
        L.oracle_set_qf.argtypes = [vp, d]
        L.oracle_set_vextra.argtypes = [vp, dp, i, i]
        L.oracle_set_psi.argtypes = [vp, d, dp]
        L.oracle_get_psi.argtypes = [vp, dp, dp]
        L.oracle_get_density.argtypes = [vp, dp, dp]
        L.oracle_get_norm.argtypes = [vp]
        L.oracle_get_norm.restype = d
        L.oracle_normalize.argtypes = [vp]
        L.oracle_evolve_qf.argtypes = [vp, i, dp]
        L.oracle_evolve_qf.restype = i
        L.oracle_energy.argtypes = [vp, dp, dp, dp, dp]
        L.oracle_energy.restype = i
        L.oracle_get_currents.argtypes = [vp, dp, dp, dp, dp]
        L.oracle_set_wz.argtypes = [vp, d, d]
        L.oracle_evolve_dipolar.argtypes = [vp, i, dp]
        L.oracle_evolve_dipolar.restype = i
        L.oracle_energy_dipolar.argtypes = [vp]
        L.oracle_energy_dipolar.restype = d
        L.oracle_wz_potential.argtypes = [vp, dp]
        L.oracle_get_currents.restype = i
        L.oracle_fft3d.argtypes = [i, i, i, dp, i, i]
        L.oracle_set_vortex.argtypes = [vp, d, d, i]
        L.oracle_get_phase.argtypes = [vp, dp]
        L.oracle_set_phase.argtypes = [vp, dp]
        L.oracle_evolve_enforced.argtypes = [vp, i, dp, i]
        L.oracle_evolve_enforced.restype = i
        L.oracle_set_hooks.argtypes = [vp, vp, vp, vp, vp]
        _lib = L
    return _lib


def build_hooks(header: str, name: str, defines=()) -> str:
    """Compiles a user hook header for the host (oracle/hooks_host.cpp) into
    oracle/_build/libhooks_<name>.so, so that the oracle evaluates the same hooks as a hook build of
    the engine.  `defines`: preprocessor definitions ("VEXT=1", "INTERACTIONS=-1", ...)."""
    os.makedirs(BUILD, exist_ok=True)
    header = os.path.abspath(header)
    out = os.path.join(BUILD, f"libhooks_{name}.so")
    src = os.path.join(HERE, "hooks_host.cpp")
    tmp = out + f".tmp{os.getpid()}"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-I", "/usr/local/cuda/include",
           f'-DGPE_USER_HOOKS="{header}"', *[f"-D{d}" for d in defines], src, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, out)
    return out


class Hooks:
    """A host build of a user hook header (build_hooks), handed to Oracle.set_hooks."""

    def __init__(self, path: str):
        self.path = path
        self.L = ctypes.CDLL(path)
        self.L.hooks_set.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_uint, ctypes.c_uint,
                                     ctypes.c_uint, ctypes.c_double, ctypes.c_double, ctypes.c_double]
        self.L.hooks_interactions.restype = ctypes.c_int

    def address(self, name: str) -> int:
        return ctypes.cast(getattr(self.L, name), ctypes.c_void_p).value

    @property
    def interactions(self) -> int:
        return self.L.hooks_interactions()


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Oracle:
    """Mirror of the reference engine API (dev/gpe_engine.h:299-552) on the CPU."""

    def __init__(self, shape, interactions, alpha, beta, dt, npart, gamma=None, threads=1):
        self.shape = tuple(int(s) for s in shape)
        self.gamma = INTER_GAMMA[interactions] if gamma is None else gamma
        L = lib()
        self._h = L.oracle_create(*self.shape, int(interactions), float(self.gamma),
                                  float(alpha), float(beta), float(dt), float(npart))
        if not self._h:
            raise ValueError(f"unsupported lattice {shape}")
        L.oracle_set_threads(self._h, int(threads))
        self._vextra = None
        self._hooks = None
        self._params = np.zeros(0)
        self._t0 = 0.0
        self._dt, self._npart = float(dt), float(npart)

    def set_hooks(self, hooks: "Hooks"):
        """Evaluate the user hooks of `hooks` instead of the built-in trap and functional (the hook
        library holds one set of run-time values: one oracle per hook library at a time)."""
        self._hooks = hooks
        lib().oracle_set_hooks(self._h, hooks.address("hooks_vext"), hooks.address("hooks_dedf"),
                               hooks.address("hooks_edf"), hooks.address("hooks_modify"))
        self._push_hook_values()

    def _push_hook_values(self):
        if self._hooks is not None:
            p = np.ascontiguousarray(self._params, dtype=np.float64)
            self._hooks.L.hooks_set(_dp(p), len(p), *[ctypes.c_uint(s) for s in self.shape], self._dt, self._t0,
                                    self._npart)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().oracle_destroy(h)
            self._h = None

    def set_threads(self, t):
        lib().oracle_set_threads(self._h, int(t))

    def set_user_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float64)
        self._params = p.copy()
        self._push_hook_values()
        return lib().oracle_set_user_params(self._h, len(p), _dp(p))

    def change_alpha_beta(self, alpha, beta):
        lib().oracle_change_alpha_beta(self._h, float(alpha), float(beta))

    def set_time(self, t0):
        self._t0 = float(t0)
        self._push_hook_values()
        lib().oracle_set_time(self._h, float(t0))

    def set_quantum_friction_coeff(self, q):
        lib().oracle_set_qf(self._h, float(q))

    def set_vextra(self, fields, steps_per_slice):
        self._vextra = np.ascontiguousarray(fields, dtype=np.float64)
        lib().oracle_set_vextra(self._h, _dp(self._vextra), self._vextra.shape[0], int(steps_per_slice))

    def set_psi(self, t, psi):
        self._t0 = float(t)
        self._push_hook_values()
        p = np.ascontiguousarray(psi, dtype=np.complex128).reshape(self.shape)
        lib().oracle_set_psi(self._h, float(t), _dp(p.view(np.float64)))

    def get_psi(self):
        out = np.empty(self.shape, dtype=np.complex128)
        t = ctypes.c_double()
        lib().oracle_get_psi(self._h, ctypes.byref(t), _dp(out.view(np.float64)))
        return t.value, out

    def get_density(self):
        out = np.empty(self.shape, dtype=np.float64)
        t = ctypes.c_double()
        lib().oracle_get_density(self._h, ctypes.byref(t), _dp(out))
        return t.value, out

    def evolve_dipolar(self, nt):
        mu = ctypes.c_double(0.0)
        lib().oracle_evolve_dipolar(self._h, int(nt), ctypes.byref(mu))
        return mu.value

    def energy_dipolar(self):
        return lib().oracle_energy_dipolar(self._h)

    def set_weizsacker(self, lam, eps=0.0):
        lib().oracle_set_wz(self._h, float(lam), float(eps))

    def wz_potential(self):
        """V_W = (lambda/8)(|grad rho|^2/rho^2 - 2 lap rho/rho) of the current psi."""
        out = np.empty(self.shape, dtype=np.float64)
        lib().oracle_wz_potential(self._h, _dp(out))
        return out

    def get_currents(self):
        """(t, jx, jy, jz) as gpe_get_currents (dev/gpe_engine.cu:1856-1904)."""
        j = [np.empty(self.shape, dtype=np.float64) for _ in range(3)]
        t = ctypes.c_double()
        lib().oracle_get_currents(self._h, ctypes.byref(t), _dp(j[0]), _dp(j[1]), _dp(j[2]))
        return t.value, j[0], j[1], j[2]

    def get_norm(self):
        return lib().oracle_get_norm(self._h)

    def normalize_psi(self):
        lib().oracle_normalize(self._h)

    def evolve_qf(self, nt):
        mu = ctypes.c_double(0.0)
        lib().oracle_evolve_qf(self._h, int(nt), ctypes.byref(mu))
        return mu.value

    def set_vortex(self, x0, y0, q=1):
        lib().oracle_set_vortex(self._h, float(x0), float(y0), int(q))

    def get_phase(self):
        out = np.empty(self.shape, dtype=np.float64)
        lib().oracle_get_phase(self._h, _dp(out))
        return out

    def set_phase(self, phase):
        p = np.ascontiguousarray(phase, dtype=np.float64).reshape(self.shape)
        lib().oracle_set_phase(self._h, _dp(p))

    def evolve_vortex(self, nt, method=1):
        mu = ctypes.c_double(0.0)
        lib().oracle_evolve_enforced(self._h, int(nt), ctypes.byref(mu), int(method))
        return mu.value

    def evolve_enforced_phase(self, nt):
        mu = ctypes.c_double(0.0)
        lib().oracle_evolve_enforced(self._h, int(nt), ctypes.byref(mu), 4)
        return mu.value

    def energy(self):
        t, a, b, c = (ctypes.c_double() for _ in range(4))
        lib().oracle_energy(self._h, ctypes.byref(t), ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return t.value, a.value, b.value, c.value


def fft3d(a: np.ndarray, sign: int, threads: int = 1) -> np.ndarray:
    out = np.ascontiguousarray(a, dtype=np.complex128).copy()
    lib().oracle_fft3d(*out.shape, _dp(out.view(np.float64)), int(sign), int(threads))
    return out
