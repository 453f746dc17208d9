"""Wavefunction snapshots in libcugpe's .dftc format.

A ``.dftc`` file holds ``nom`` frames of ``nx*ny*nz`` complex128 values in C
order, one after the other; ``<file>.dftc.info`` is the text header written
by the reference's ``gpe_save_info`` (dev/gpe_io.h:45-104) and read by its
``gpe_get_info`` (dev/gpe_io.h:130-166) and ``read_dftc_info``
(python/read_dftc_info.py:4-50).  The writing pipeline is native
(``csrc/gpe_snapshots.cpp``): frames go to the host on a side stream and to
the file from a writer thread while the engine keeps evolving.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _check, _lib

INFO_FIELDS = ("system", "mode", "nx", "ny", "nz", "dt", "nom", "a_scattering", "aspect_ratio", "omega_x", "r0",
               "npart", "total_time")


@dataclass
class Info:
    system: str = "bosons"
    mode: str = "contact"
    nx: int = 0
    ny: int = 0
    nz: int = 0
    dt: float = 0.0
    nom: int = 0
    a_scattering: float = 0.0
    aspect_ratio: float = 1.0
    omega_x: float = 1.0
    r0: float = 0.0
    npart: float = 1.0
    total_time: float = 0.0


def system_mode(interactions: int) -> tuple[str, str]:
    """The info file's system and mode lines for a functional code (dev/gpe_io.h:66-83)."""
    if interactions == -1:
        return "bosons", "contact"
    return "fermions", ("unitary" if interactions == 0 else "bec")


def write_info(dftc_path: str, info: Info) -> None:
    _check(_lib().gpe_gb_dftc_write_info(dftc_path.encode(), info.system.encode(), info.mode.encode(), info.nx,
                                         info.ny, info.nz, info.dt, info.nom, info.a_scattering, info.aspect_ratio,
                                         info.omega_x, info.r0, info.npart, info.total_time), "dftc_write_info")


def read_info(dftc_path: str) -> Info:
    sysb, modeb = ctypes.create_string_buffer(64), ctypes.create_string_buffer(64)
    ints = [ctypes.c_int() for _ in range(4)]
    dbl = [ctypes.c_double() for _ in range(7)]
    _check(_lib().gpe_gb_dftc_read_info(dftc_path.encode(), sysb, modeb, 64, ctypes.byref(ints[0]),
                                        ctypes.byref(ints[1]), ctypes.byref(ints[2]), ctypes.byref(dbl[0]),
                                        ctypes.byref(ints[3]), ctypes.byref(dbl[1]), ctypes.byref(dbl[2]),
                                        ctypes.byref(dbl[3]), ctypes.byref(dbl[4]), ctypes.byref(dbl[5]),
                                        ctypes.byref(dbl[6])), "dftc_read_info")
    return Info(sysb.value.decode(), modeb.value.decode(), ints[0].value, ints[1].value, ints[2].value, dbl[0].value,
                ints[3].value, dbl[1].value, dbl[2].value, dbl[3].value, dbl[4].value, dbl[5].value, dbl[6].value)


def read_frames(dftc_path: str, shape=None) -> np.ndarray:
    """All frames as an array [nom, nx, ny, nz] (memory-mapped), shape from the info file if not given."""
    if shape is None:
        i = read_info(dftc_path)
        shape = (i.nx, i.ny, i.nz)
    data = np.memmap(dftc_path, dtype=np.complex128, mode="r")
    n = int(np.prod(shape))
    return data.reshape((data.size // n,) + tuple(shape))


class Snapshots:
    """Frames of one engine appended to a .dftc file while it evolves.

    ``push()`` queues the engine's current psi (waiting only when ``nbuf``
    frames are still in flight) and returns its time; ``close()`` waits for
    the writes and, when ``info`` is given, writes the info file with ``nom``
    set to the frames written.
    """

    def __init__(self, engine, dftc_path: str, nbuf: int = 3, info: Info | None = None):
        self._h = ctypes.c_void_p()
        self.path = dftc_path
        self.info = info
        self.times: list[float] = []
        _check(_lib().gpe_gb_snapshots_open(ctypes.byref(self._h), engine._h, dftc_path.encode(), int(nbuf)),
               "snapshots_open")

    def push(self) -> float:
        t = ctypes.c_double()
        _check(_lib().gpe_gb_snapshots_push(self._h, ctypes.byref(t)), "snapshots_push")
        self.times.append(t.value)
        return t.value

    def close(self) -> int:
        if not self._h:
            return 0
        frames = ctypes.c_longlong()
        h, self._h = self._h, ctypes.c_void_p()
        _check(_lib().gpe_gb_snapshots_close(h, ctypes.byref(frames)), "snapshots_close")
        if self.info is not None:
            self.info.nom = int(frames.value)
            if self.times:
                self.info.total_time = self.times[-1]
            write_info(self.path, self.info)
        return int(frames.value)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
