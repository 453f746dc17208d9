"""GB300-native split-step GPE engine (libcugpe's gpe_evolve_qf path).

Python binding of the C ABI in ``include/gpe_gb300.h`` (``libgpe_gb300.so``,
built in-tree by ``libcugpe_gb300.build``).  The engine runs only on the GPU:
if the shared library is missing or no CUDA device is present, every call
fails with an exception; there is no CPU path.

``Engine`` mirrors the reference engine API (KKobuszewski/libcugpe
dev/gpe_engine.h:299-552) with the lattice and functional given at run time:

    e = Engine((64, 64, 64), interactions=-1, alpha=0.0, beta=1.0, dt=0.016, npart=1.0)
    e.set_user_params([wx, wy, wz, a_scat])
    e.set_psi(0.0, psi)          # complex128 [nx, ny, nz]
    mu = e.evolve_qf(2000)
    t, ekin, eint, eext = e.energy()
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libgpe_gb300.so")

FP64 = 0
FP32 = 1

ERR_TOO_MANY_PARAMS = -9
ERR_LATTICE = -10
ERR_NO_ENGINE = -11
ERR_ARGUMENT = -12
ERR_FUNCTIONAL = -13
ERR_NOALLOC_SIZE = -14
ERR_IO = -15
ERR_NOT_IMPLEMENTED = -98

# entry points declared in include/gpe_gb300.h
C_ABI_SYMBOLS = [
    "gpe_gb_create", "gpe_gb_destroy", "gpe_gb_get_lattice", "gpe_gb_change_alpha_beta", "gpe_gb_set_time",
    "gpe_gb_set_user_params", "gpe_gb_set_quantum_friction_coeff", "gpe_gb_set_psi", "gpe_gb_get_psi",
    "gpe_gb_get_density", "gpe_gb_get_currents", "gpe_gb_get_norm", "gpe_gb_normalize_psi", "gpe_gb_evolve_qf", "gpe_gb_energy",
    "gpe_gb_set_psi_device", "gpe_gb_get_psi_device", "gpe_gb_synchronize", "gpe_gb_kernel_launches",
    "gpe_gb_use_graphs", "gpe_gb_set_potential_slices", "gpe_gb_error_string", "gpe_gb_get_stream",
    "gpe_gb_profile_passes", "gpe_gb_norm_noalloc", "gpe_gb_set_vortex", "gpe_gb_get_phase", "gpe_gb_set_phase",
    "gpe_gb_evolve_vortex", "gpe_gb_evolve_enforced_phase", "gpe_gb_batch_create", "gpe_gb_batch_destroy",
    "gpe_gb_batch_engine", "gpe_gb_batch_set_active", "gpe_gb_batch_evolve", "gpe_gb_batch_chemical_potentials",
    "gpe_gb_batch_kernel_launches", "gpe_gb_chemical_potential", "gpe_gb_control_create", "gpe_gb_control_loss",
    "gpe_gb_control_loss_grad", "gpe_gb_control_destroy", "gpe_gb_snapshots_open", "gpe_gb_snapshots_push",
    "gpe_gb_snapshots_close", "gpe_gb_dftc_write_info", "gpe_gb_dftc_read_info", "gpe_gb_set_weizsacker",
    "gpe_gb_evolve_dipolar", "gpe_gb_energy_dipolar", "gpe_gb_autotune", "gpe_gb_batch_autotune",
    "gpe_gb_set_fft_plan", "gpe_gb_get_fft_plan", "gpe_gb_batch_set_fft_plan", "gpe_gb_fp64_fma_rate",
    "gpe_gb_user_hooks", "gpe_gb_set_plane_passes", "gpe_gb_batch_solve",
]


class GPEError(RuntimeError):
    def __init__(self, code: int, where: str, lib=None):
        self.code = code
        L = lib if lib is not None else _LIBS.get(LIB_PATH)
        msg = L.gpe_gb_error_string(code).decode() if L is not None else str(code)
        super().__init__(f"{where} failed with code {code}: {msg}")


_LIBS = {}


def _lib(path: str | None = None):
    """The C-ABI library at `path` (default: the in-tree libgpe_gb300.so), loaded once."""
    path = os.path.abspath(path) if path else LIB_PATH
    L = _LIBS.get(path)
    if L is None:
        if not os.path.isfile(path):
            raise ImportError(f"{os.path.basename(path)} not built ({path}); run libcugpe_gb300.build.build()")
        L = ctypes.CDLL(path)
        vp, d, i = ctypes.c_void_p, ctypes.c_double, ctypes.c_int
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        sig = {
            "gpe_gb_create": (i, [ctypes.POINTER(vp), i, i, i, i, i, d, d, d, d]),
            "gpe_gb_destroy": (i, [vp]),
            "gpe_gb_get_lattice": (i, [vp, ip, ip, ip]),
            "gpe_gb_change_alpha_beta": (i, [vp, d, d]),
            "gpe_gb_set_time": (i, [vp, d]),
            "gpe_gb_set_user_params": (i, [vp, i, dp]),
            "gpe_gb_set_quantum_friction_coeff": (i, [vp, d]),
            "gpe_gb_set_weizsacker": (i, [vp, d, d]),
            "gpe_gb_evolve_dipolar": (i, [vp, i, dp]),
            "gpe_gb_autotune": (i, [vp, i, ip, ip, ip, dp]),
            "gpe_gb_batch_autotune": (i, [vp, i, ip, ip, ip, dp]),
            "gpe_gb_set_fft_plan": (i, [vp, i]),
            "gpe_gb_get_fft_plan": (i, [vp, ip]),
            "gpe_gb_batch_set_fft_plan": (i, [vp, i]),
            "gpe_gb_energy_dipolar": (i, [vp, dp, dp]),
            "gpe_gb_set_psi": (i, [vp, d, dp]),
            "gpe_gb_get_psi": (i, [vp, dp, dp]),
            "gpe_gb_get_density": (i, [vp, dp, dp]),
            "gpe_gb_get_norm": (i, [vp, dp]),
            "gpe_gb_get_currents": (i, [vp, dp, dp, dp, dp]),
            "gpe_gb_normalize_psi": (i, [vp]),
            "gpe_gb_evolve_qf": (i, [vp, i, dp]),
            "gpe_gb_energy": (i, [vp, dp, dp, dp, dp]),
            "gpe_gb_set_psi_device": (i, [vp, d, vp]),
            "gpe_gb_get_psi_device": (i, [vp, dp, vp]),
            "gpe_gb_synchronize": (i, [vp]),
            "gpe_gb_kernel_launches": (ctypes.c_longlong, [vp]),
            "gpe_gb_use_graphs": (i, [vp, i]),
            "gpe_gb_set_potential_slices": (i, [vp, dp, i, i]),
            "gpe_gb_error_string": (ctypes.c_char_p, [i]),
            "gpe_gb_get_stream": (vp, [vp]),
            "gpe_gb_norm_noalloc": (i, [vp, i, ctypes.c_longlong, d, vp, vp]),
            "gpe_gb_fp64_fma_rate": (i, [dp]),
            "gpe_gb_user_hooks": (i, [ip, ip]),
            "gpe_gb_set_plane_passes": (i, [vp, i]),
            "gpe_gb_batch_solve": (i, [vp, i, i, dp, ip, dp]),
            "gpe_gb_set_vortex": (i, [vp, d, d, i]),
            "gpe_gb_get_phase": (i, [vp, dp]),
            "gpe_gb_set_phase": (i, [vp, dp]),
            "gpe_gb_evolve_vortex": (i, [vp, i, dp, i]),
            "gpe_gb_evolve_enforced_phase": (i, [vp, i, dp]),
            "gpe_gb_batch_create": (i, [ctypes.POINTER(vp), i, ip, i, i, d, d, dp, dp]),
            "gpe_gb_batch_destroy": (i, [vp]),
            "gpe_gb_batch_engine": (vp, [vp, i]),
            "gpe_gb_batch_set_active": (i, [vp, i, i]),
            "gpe_gb_batch_evolve": (i, [vp, i]),
            "gpe_gb_batch_chemical_potentials": (i, [vp, dp, dp]),
            "gpe_gb_batch_kernel_launches": (ctypes.c_longlong, [vp]),
            "gpe_gb_chemical_potential": (i, [vp, dp, dp]),
            "gpe_gb_control_create": (i, [ctypes.POINTER(vp), vp, i, dp, i, i, i, i, dp]),
            "gpe_gb_control_loss": (i, [vp, dp, dp, dp]),
            "gpe_gb_control_loss_grad": (i, [vp, dp, dp, dp, dp]),
            "gpe_gb_control_destroy": (i, [vp]),
            "gpe_gb_profile_passes": (i, [vp, i, ctypes.POINTER(ctypes.c_float), dp, ip, ip, i, ip]),
            "gpe_gb_snapshots_open": (i, [ctypes.POINTER(vp), vp, ctypes.c_char_p, i]),
            "gpe_gb_snapshots_push": (i, [vp, dp]),
            "gpe_gb_snapshots_close": (i, [vp, ctypes.POINTER(ctypes.c_longlong)]),
            "gpe_gb_dftc_write_info": (i, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, i, i, i, d, i, d, d,
                                           d, d, d, d]),
            "gpe_gb_dftc_read_info": (i, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, i, ip, ip, ip, dp, ip,
                                          dp, dp, dp, dp, dp, dp]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _LIBS[path] = L
    return L


def lib_path() -> str:
    return LIB_PATH


def fp64_fma_rate() -> float:
    """Measured FP64 FMA throughput of the current device, TFLOP/s."""
    r = ctypes.c_double()
    _check(_lib().gpe_gb_fp64_fma_rate(ctypes.byref(r)), "fp64_fma_rate")
    return r.value


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _check(rc: int, where: str, lib=None):
    if rc != 0:
        raise GPEError(rc, where, lib)


def user_hooks(library: str | None = None):
    """(True, interactions) for a library built with a user hook header, else (False, 0)."""
    en, inter = ctypes.c_int(), ctypes.c_int()
    _check(_lib(library).gpe_gb_user_hooks(ctypes.byref(en), ctypes.byref(inter)), "user_hooks")
    return bool(en.value), inter.value


class Engine:
    """One condensate on the GPU; the methods follow the reference API."""

    def __init__(self, shape, interactions=-1, alpha=0.0, beta=1.0, dt=1e-3, npart=1.0, precision=FP64,
                 library=None, _handle=None):
        """`library`: path of a C-ABI library built with user hooks (libcugpe_gb300.build), default the
        in-tree libgpe_gb300.so."""
        self._L = _lib(library)
        self.shape = tuple(int(s) for s in shape)
        self.precision = precision
        self.alpha, self.beta, self.dt, self.npart = alpha, beta, dt, npart
        self._owned = _handle is None
        if _handle is not None:  # a condensate owned by a Batch
            self._h = ctypes.c_void_p(_handle)
            return
        L = self._L
        h = ctypes.c_void_p()
        _check(L.gpe_gb_create(ctypes.byref(h), *self.shape, int(interactions), int(precision),
                               float(alpha), float(beta), float(dt), float(npart)), "gpe_gb_create", L)
        self._h = h

    def close(self):
        if getattr(self, "_h", None) and self._owned:
            self._L.gpe_gb_destroy(self._h)
        self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def set_user_params(self, params):
        p = np.ascontiguousarray(params, dtype=np.float64)
        _check(self._L.gpe_gb_set_user_params(self._h, len(p), _dp(p)), "set_user_params", self._L)

    def change_alpha_beta(self, alpha, beta):
        self.alpha, self.beta = alpha, beta
        _check(self._L.gpe_gb_change_alpha_beta(self._h, float(alpha), float(beta)), "change_alpha_beta", self._L)

    def set_rte_evolution(self):
        self.change_alpha_beta(1.0, 0.0)

    def set_ite_evolution(self):
        self.change_alpha_beta(0.0, 1.0)

    def set_time(self, t0):
        _check(self._L.gpe_gb_set_time(self._h, float(t0)), "set_time", self._L)

    def set_quantum_friction_coeff(self, q):
        _check(self._L.gpe_gb_set_quantum_friction_coeff(self._h, float(q)), "set_quantum_friction_coeff", self._L)

    def set_weizsacker(self, lam, eps=0.0):
        """Weizsaecker gradient term (lambda/8) |grad rho|^2/(rho + eps) in the functional; lam = 0 turns
        it off, eps <= 0 selects 1e-2 npart / n.  Steps longer than the term's stability bound
        (dt |lam| 3 pi^2 <= 0.4) run as equal sub-steps."""
        _check(self._L.gpe_gb_set_weizsacker(self._h, float(lam), float(eps)), "set_weizsacker", self._L)

    def set_psi(self, t, psi):
        p = np.ascontiguousarray(psi, dtype=np.complex128).reshape(self.shape)
        _check(self._L.gpe_gb_set_psi(self._h, float(t), _dp(p.view(np.float64))), "set_psi", self._L)

    def get_psi(self, out=None):
        out = np.empty(self.shape, dtype=np.complex128) if out is None else out
        t = ctypes.c_double()
        _check(self._L.gpe_gb_get_psi(self._h, ctypes.byref(t), _dp(out.view(np.float64))), "get_psi", self._L)
        return t.value, out

    def set_psi_device(self, t, ptr: int):
        _check(self._L.gpe_gb_set_psi_device(self._h, float(t), ctypes.c_void_p(ptr)), "set_psi_device", self._L)

    def get_psi_device(self, ptr: int):
        t = ctypes.c_double()
        _check(self._L.gpe_gb_get_psi_device(self._h, ctypes.byref(t), ctypes.c_void_p(ptr)), "get_psi_device", self._L)
        return t.value

    def get_density(self):
        out = np.empty(self.shape, dtype=np.float64)
        t = ctypes.c_double()
        _check(self._L.gpe_gb_get_density(self._h, ctypes.byref(t), _dp(out)), "get_density", self._L)
        return t.value, out

    def get_currents(self):
        """(t, jx, jy, jz): probability currents Re(conj(psi) IFFT(k_a/(Gamma n) FFT psi))."""
        j = [np.empty(self.shape, dtype=np.float64) for _ in range(3)]
        t = ctypes.c_double()
        _check(self._L.gpe_gb_get_currents(self._h, ctypes.byref(t), _dp(j[0]), _dp(j[1]), _dp(j[2])),
               "get_currents")
        return t.value, j[0], j[1], j[2]

    def get_norm(self):
        n = ctypes.c_double()
        _check(self._L.gpe_gb_get_norm(self._h, ctypes.byref(n)), "get_norm", self._L)
        return n.value

    def normalize_psi(self):
        _check(self._L.gpe_gb_normalize_psi(self._h), "normalize_psi", self._L)

    def evolve_qf(self, nt):
        mu = ctypes.c_double(0.0)
        _check(self._L.gpe_gb_evolve_qf(self._h, int(nt), ctypes.byref(mu)), "evolve_qf", self._L)
        return mu.value

    def autotune(self, nsteps=32):
        """Times each launch configuration on this engine's state and keeps the fastest; psi, time
        and step counter are restored.  Returns {"direct", "graph_steps", "fft_plan", "ms_per_step"};
        fft_plan 2 means a radix plan chosen per fused pass."""
        d, c, p, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        _check(self._L.gpe_gb_autotune(self._h, int(nsteps), ctypes.byref(d), ctypes.byref(c), ctypes.byref(p),
                                      ctypes.byref(ms)), "autotune")
        return {"direct": d.value, "graph_steps": c.value, "fft_plan": p.value, "ms_per_step": ms.value}

    def set_plane_passes(self, enable: bool):
        """Real-time FP32 steps on 128 x 128 yz-planes as yz-plane passes (default) or pencil passes only."""
        _check(self._L.gpe_gb_set_plane_passes(self._h, 1 if enable else 0), "set_plane_passes", self._L)

    def set_fft_plan(self, plan):
        """Radix plan of the pencil FFTs: 0 default, 1 the alternative (FP32, pencils of 32-512 points)."""
        _check(self._L.gpe_gb_set_fft_plan(self._h, int(plan)), "set_fft_plan", self._L)

    def get_fft_plan(self):
        p = ctypes.c_int()
        _check(self._L.gpe_gb_get_fft_plan(self._h, ctypes.byref(p)), "get_fft_plan", self._L)
        return p.value

    def evolve_dipolar(self, nt):
        """gpe_evolve_dipolar: nt steps of the dipolar BEC (interactions -2); mu in ITE."""
        mu = ctypes.c_double(0.0)
        _check(self._L.gpe_gb_evolve_dipolar(self._h, int(nt), ctypes.byref(mu)), "evolve_dipolar", self._L)
        return mu.value

    def energy_dipolar(self):
        """(t, E_dip) with E_dip = 1/2 sum rho vdip."""
        t, ed = ctypes.c_double(), ctypes.c_double()
        _check(self._L.gpe_gb_energy_dipolar(self._h, ctypes.byref(t), ctypes.byref(ed)), "energy_dipolar", self._L)
        return t.value, ed.value

    def set_vortex(self, x0, y0, q=1):
        _check(self._L.gpe_gb_set_vortex(self._h, float(x0), float(y0), int(q)), "set_vortex", self._L)

    def get_phase(self):
        out = np.empty(self.shape, dtype=np.float64)
        _check(self._L.gpe_gb_get_phase(self._h, _dp(out)), "get_phase", self._L)
        return out

    def set_phase(self, phase):
        p = np.ascontiguousarray(phase, dtype=np.float64).reshape(self.shape)
        _check(self._L.gpe_gb_set_phase(self._h, _dp(p)), "set_phase", self._L)

    def evolve_vortex(self, nt, method=1):
        mu = ctypes.c_double(0.0)
        _check(self._L.gpe_gb_evolve_vortex(self._h, int(nt), ctypes.byref(mu), int(method)), "evolve_vortex", self._L)
        return mu.value

    def evolve_enforced_phase(self, nt):
        mu = ctypes.c_double(0.0)
        _check(self._L.gpe_gb_evolve_enforced_phase(self._h, int(nt), ctypes.byref(mu)), "evolve_enforced_phase", self._L)
        return mu.value

    def chemical_potential(self):
        """(mu of the last ITE step, running sum of mu over all ITE steps)."""
        mu, ms = ctypes.c_double(), ctypes.c_double()
        _check(self._L.gpe_gb_chemical_potential(self._h, ctypes.byref(mu), ctypes.byref(ms)), "chemical_potential", self._L)
        return mu.value, ms.value

    def energy(self):
        t, a, b, c = (ctypes.c_double() for _ in range(4))
        _check(self._L.gpe_gb_energy(self._h, ctypes.byref(t), ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
               "energy")
        return t.value, a.value, b.value, c.value

    def synchronize(self):
        _check(self._L.gpe_gb_synchronize(self._h), "synchronize", self._L)

    def stream_handle(self) -> int:
        return int(self._L.gpe_gb_get_stream(self._h) or 0)

    def kernel_launches(self) -> int:
        return int(self._L.gpe_gb_kernel_launches(self._h))

    def profile_passes(self, nsteps: int):
        """Per-pass mean duration (ms), algorithmic bytes, axis and kernel class over nsteps steps."""
        cap = 16
        ms = (ctypes.c_float * cap)()
        by = (ctypes.c_double * cap)()
        ax = (ctypes.c_int * cap)()
        kd = (ctypes.c_int * cap)()
        npass = ctypes.c_int()
        _check(self._L.gpe_gb_profile_passes(self._h, int(nsteps), ms, by, ax, kd, cap, ctypes.byref(npass)),
               "profile_passes")
        kinds = {0: "kin", 1: "epi", 2: "lap", 3: "energy", 4: "dipolar", 8: "plane"}
        return [{"ms": ms[p], "bytes": by[p], "axis": ("x", "y", "z", "yz")[ax[p]], "kind": kinds.get(kd[p], str(kd[p]))}
                for p in range(min(npass.value, cap))]

    def use_graphs(self, enable: bool):
        _check(self._L.gpe_gb_use_graphs(self._h, 1 if enable else 0), "use_graphs", self._L)

    def set_potential_slices(self, fields, steps_per_slice):
        if fields is None:
            _check(self._L.gpe_gb_set_potential_slices(self._h, None, 0, 0), "set_potential_slices", self._L)
            return
        f = np.ascontiguousarray(fields, dtype=np.float64)
        self._slices = f
        _check(self._L.gpe_gb_set_potential_slices(self._h, _dp(f), f.shape[0], int(steps_per_slice)),
               "set_potential_slices")


class Batch:
    """Independent condensates stepped together (FP32-mixed): one launch per
    fused pass covers every active condensate, whatever its lattice size."""

    def __init__(self, shapes, interactions=-1, alpha=0.0, beta=1.0, dt=1e-3, npart=None, precision=FP32,
                 library=None):
        L = self._L = _lib(library)
        shapes = [tuple(int(x) for x in s) for s in shapes]
        n = len(shapes)
        npart = [1.0] * n if npart is None else list(npart)
        dts = [float(dt)] * n if np.isscalar(dt) else [float(x) for x in dt]
        sides = (ctypes.c_int * (3 * n))(*[x for s in shapes for x in s])
        nps = (ctypes.c_double * n)(*[float(x) for x in npart])
        dtp = (ctypes.c_double * n)(*dts)
        h = ctypes.c_void_p()
        _check(L.gpe_gb_batch_create(ctypes.byref(h), n, sides, int(interactions), int(precision), float(alpha),
                                     float(beta), dtp, nps), "gpe_gb_batch_create")
        self._h = h
        self.engines = [Engine(shapes[i], interactions, alpha, beta, dts[i], npart[i], precision, library,
                               _handle=L.gpe_gb_batch_engine(h, i)) for i in range(n)]

    def __len__(self):
        return len(self.engines)

    def evolve(self, nt):
        _check(self._L.gpe_gb_batch_evolve(self._h, int(nt)), "batch_evolve", self._L)

    def set_active(self, i, active):
        _check(self._L.gpe_gb_batch_set_active(self._h, int(i), 1 if active else 0), "batch_set_active", self._L)

    def autotune(self, nsteps=32):
        """Item order and graph length of the batched passes, timed on the batch's state (restored)."""
        o, c, p, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        _check(self._L.gpe_gb_batch_autotune(self._h, int(nsteps), ctypes.byref(o), ctypes.byref(c),
                                            ctypes.byref(p), ctypes.byref(ms)), "batch_autotune")
        return {"order": o.value, "graph_steps": c.value, "fft_plan": p.value, "ms_per_step": ms.value}

    def set_fft_plan(self, plan):
        """Radix plan of every condensate's pencil FFTs (0 default, 1 alternative)."""
        _check(self._L.gpe_gb_batch_set_fft_plan(self._h, int(plan)), "batch_set_fft_plan", self._L)

    def solve(self, max_steps, check, tol):
        """Imaginary-time solve with the convergence test on the device: each active condensate stops
        once the mean of mu over `check` steps changes by less than tol (per step, lattice units; a
        scalar or one value per condensate) between intervals.  Returns (steps, mu): steps to
        convergence (-1 if not converged within max_steps) and the converged interval mean of mu."""
        n = len(self.engines)
        t = np.ascontiguousarray(np.broadcast_to(np.asarray(tol, dtype=np.float64), (n,)))
        steps = np.zeros(n, dtype=np.int32)
        mu = np.zeros(n)
        _check(self._L.gpe_gb_batch_solve(self._h, int(max_steps), int(check), _dp(t),
                                          steps.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _dp(mu)),
               "batch_solve", self._L)
        return steps, mu

    def chemical_potentials(self):
        """Per condensate: (mu of the last ITE step, running sum of mu)."""
        n = len(self.engines)
        mu = np.zeros(n)
        ms = np.zeros(n)
        _check(self._L.gpe_gb_batch_chemical_potentials(self._h, _dp(mu), _dp(ms)), "batch_chemical_potentials", self._L)
        return mu, ms

    def kernel_launches(self) -> int:
        return int(self._L.gpe_gb_batch_kernel_launches(self._h))

    def close(self):
        if getattr(self, "_h", None):
            for e in self.engines:
                e._h = None
            self._L.gpe_gb_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
