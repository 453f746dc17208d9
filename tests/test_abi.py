"""The C-ABI library: it loads, exports every entry point the headers
declare, and a reference-style driver links against it.  No GPU needed."""
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def declared_c_abi():
    text = open(os.path.join(INCLUDE, "gpe_gb300.h")).read()
    return sorted(set(re.findall(r"\b(gpe_gb_\w+)\s*\(", text)))


def test_library_loads_and_exports_c_abi(gpe_lib):
    import ctypes
    import libcugpe_gb300 as g
    lib = ctypes.CDLL(gpe_lib)
    names = declared_c_abi()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
    assert sorted(g.C_ABI_SYMBOLS) == names


def test_error_strings_without_gpu(gpe_lib):
    import libcugpe_gb300 as g
    L = g._lib()
    assert L.gpe_gb_error_string(-9) == b"too many user parameters"
    assert L.gpe_gb_error_string(g.ERR_LATTICE).startswith(b"unsupported lattice")
    assert L.gpe_gb_error_string(-98).startswith(b"entry point not implemented")


def test_argument_checks_without_gpu(gpe_lib):
    import ctypes
    import libcugpe_gb300 as g
    L = g._lib()
    h = ctypes.c_void_p()
    # lattice and functional are checked before any CUDA call
    assert L.gpe_gb_create(ctypes.byref(h), 12, 16, 16, -1, 0, 0.0, 1.0, 0.1, 1.0) == g.ERR_LATTICE
    assert L.gpe_gb_create(ctypes.byref(h), 16, 16, 1024, -1, 0, 0.0, 1.0, 0.1, 1.0) == g.ERR_LATTICE
    assert L.gpe_gb_create(ctypes.byref(h), 16, 16, 16, 5, 0, 0.0, 1.0, 0.1, 1.0) == g.ERR_FUNCTIONAL
    assert L.gpe_gb_create(None, 16, 16, 16, -1, 0, 0.0, 1.0, 0.1, 1.0) == g.ERR_ARGUMENT
    assert L.gpe_gb_evolve_qf(None, 1, None) == g.ERR_NO_ENGINE
    assert L.gpe_gb_set_user_params(None, 3, None) == g.ERR_NO_ENGINE
    # radix plans and autotuners check their handle first
    p = ctypes.c_int()
    assert L.gpe_gb_set_fft_plan(None, 1) == g.ERR_NO_ENGINE
    assert L.gpe_gb_get_fft_plan(None, ctypes.byref(p)) == g.ERR_NO_ENGINE
    assert L.gpe_gb_batch_set_fft_plan(None, 1) == g.ERR_ARGUMENT
    assert L.gpe_gb_autotune(None, 8, None, None, None, None) == g.ERR_NO_ENGINE
    assert L.gpe_gb_batch_autotune(None, 8, None, None, None, None) == g.ERR_ARGUMENT


DRIVER = r"""
#include "gpe_engine.h"
// every entry point of the reference API (dev/gpe_engine.h:299-558)
int main() {
    int nx, ny, nz, ierr = 0;
    double t, a, b, c, mu, p[4] = {0.1, 0.1, 0.1, 0.0};
    cuCplx* psi = 0;
    gpe_get_lattice(&nx, &ny, &nz);
    gpe_exec(gpe_create_engine(0.0, 1.0, 0.1, 1.0), ierr);
    gpe_change_alpha_beta(0.0, 1.0); gpe_set_rte_evolution(); gpe_set_ite_evolution();
    gpe_set_time(0.0); gpe_set_user_params(4, p); gpe_set_quantum_friction_coeff(0.0);
    gpe_set_vortex(0.5, 0.5); gpe_get_phase(); gpe_set_phase(0);
    gpe_set_psi(0.0, psi); gpe_get_psi(&t, psi); gpe_get_density(&t, 0); gpe_get_currents(&t, 0, 0, 0);
    gpe_normalize_psi(); gpe_get_norm(&a); gpe_evolve(1); gpe_evolve_qf(1, &mu); gpe_evolve_qf(1);
    gpe_evolve_vortex(1); gpe_evolve_vortex2(1); gpe_evolve_vortex3(1); gpe_evolve_enforced_phase(1);
    gpe_evolve_dipolar(1); gpe_evolve_dipolar(1, &mu); gpe_energy_dipolar(&t, &a); gpe_energy_dipolar2(&t, &a);
    gpe_energy(&t, &a, &b, &c); gpe_print_potential_type(); gpe_destroy_engine();
    return 0;
}
"""


def test_reference_style_driver_links(gpe_lib, tmp_path):
    src = tmp_path / "driver.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "driver"
    cmd = ["g++", "-DNX=16", "-DNY=16", "-DNZ=16", "-I", INCLUDE, "-I", "/usr/local/cuda/include", str(src),
           "-L", os.path.dirname(gpe_lib), "-lgpe_gb300", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # the mangled names match the reference library's (C++ linkage, same signatures)
    nm = subprocess.run(["nm", "-D", "--defined-only", gpe_lib], capture_output=True, text=True).stdout
    for sym in ["_Z17gpe_create_engineddddi", "_Z13gpe_evolve_qfiPd", "_Z11gpe_set_psidP7double2",
                "_Z10gpe_energyPdS_S_S_", "_Z19gpe_set_user_paramsiPd", "_Z14gpe_set_vortexdda"]:
        assert sym in nm, sym
