"""Snapshots in the .dftc format: the info file in the line layout of the
reference's gpe_save_info / gpe_get_info (dev/gpe_io.h:45-166), and frames
written by the native pipeline while the engine evolves, compared bit for bit
with get_psi at the same moments."""
import os

import numpy as np
import pytest

import libcugpe_gb300 as g
from libcugpe_gb300 import configs, dftc


def test_info_round_trip_and_layout(tmp_path, gpe_lib):
    path = str(tmp_path / "psi.dftc")
    info = dftc.Info("fermions", "unitary", 128, 64, 32, 0.125, 7, float("inf"), 1.5, 0.04, 3.25, 1000.0, 12.5)
    dftc.write_info(path, info)
    lines = open(path + ".info").read().splitlines()
    assert len(lines) == 13
    assert lines[0] == "fermions   # system type" and lines[1] == "unitary   # mode"
    assert lines[2] == "128   # nx" and lines[6] == "7   # nom"
    assert lines[5] == "%.15e   # dt" % 0.125
    # the reference's python reader skips two lines and takes the first number of each
    assert [float(x.split()[0]) for x in lines[2:]][:5] == [128, 64, 32, 0.125, 7]
    back = dftc.read_info(path)
    assert back == info


def test_info_reads_a_reference_style_file(tmp_path, gpe_lib):
    path = str(tmp_path / "gs.dftc")
    text = ("bosons   # system type\ncontact   # mode\n32   # nx\n32   # ny\n16   # nz\n"
            "1.000000000000000e-03   # dt\n1   # nom\n2.500000000000000e+00   # a_scattering\n"
            "1.000000000000000e+00   # aspect_ratio\n1.000000000000000e+00   # omega_x\n"
            "0.000000000000000e+00   # r0\n1.000000000000000e+00   # npart\n")
    open(path + ".info", "w").write(text)
    i = dftc.read_info(path)
    assert (i.system, i.mode, i.nx, i.ny, i.nz, i.nom) == ("bosons", "contact", 32, 32, 16, 1)
    assert i.dt == 1e-3 and i.a_scattering == 2.5 and i.total_time == 0.0
    with pytest.raises(g.GPEError):
        dftc.read_info(str(tmp_path / "missing.dftc"))


def test_read_frames_layout(tmp_path, gpe_lib):
    """Frames are consecutive complex128 lattices in C order; the shape comes from the info file."""
    path = str(tmp_path / "f.dftc")
    rng = np.random.default_rng(3)
    frames = rng.standard_normal((3, 8, 4, 16)) + 1j * rng.standard_normal((3, 8, 4, 16))
    frames.astype(np.complex128).tofile(path)
    dftc.write_info(path, dftc.Info("bosons", "contact", 8, 4, 16, 0.1, 3, 1.0, 1.0, 0.1, 0.0, 1.0, 0.3))
    got = dftc.read_frames(path)
    assert got.shape == (3, 8, 4, 16) and np.array_equal(got, frames)
    assert np.array_equal(dftc.read_frames(path, shape=(16, 4, 8))[2], frames[2].reshape(16, 4, 8))


IO_DRIVER = r"""
#include <cstdio>
#include <cstring>
#include "gpe_engine.h"
#include "gpe_io.h"
// the driver-side headers of the reference (timers, .dftc.info), as test_vortex/ite_vortex.c and
// rte_vortex.c use them
int main(int argc, char** argv) {
    b_t();
    char name[256];
    snprintf(name, sizeof name, "%s/run.dftc", argv[1]);
    gpe_save_info(name, 64, 32, 16, 0.125, 3, 2.5, 1.5, 0.04, 0.0, 1000.0, 12.5);
    int nx, ny, nz, nom;
    double dt, a, ar, w, r0, np, tt = -1.0;
    gpe_get_info(name, &nx, &ny, &nz, &dt, &nom, &a, &ar, &w, &r0, &np, &tt);
    printf("NEW %d %d %d %.17g %d %.17g %.17g %.17g %.17g %.17g %.17g\n", nx, ny, nz, dt, nom, a, ar, w, r0, np, tt);
    snprintf(name, sizeof name, "%s/old.dftc", argv[1]);
    save_info(name, 8, 16, 32, 0.5, 2, 1.25, 2.0, 0.1, 3.0, 10.0);
    snprintf(name, sizeof name, "%s/old.dftc.info", argv[1]);
    get_info(name, &nx, &ny, &nz, &dt, &nom, &a, &ar, &w, &r0, &np);
    printf("OLD %d %d %d %.17g %d %.17g %.17g %.17g %.17g %.17g\n", nx, ny, nz, dt, nom, a, ar, w, r0, np);
    const double s = e_t(0);
    printf("TIME %d %d\n", s >= 0.0 && s < 60.0, e_t(1) == s);
    return 0;
}
"""


def test_reference_driver_headers_timing_and_info(tmp_path, gpe_lib):
    """gpe_timing.h and gpe_io.h: a driver using b_t/e_t, gpe_save_info/gpe_get_info and the older
    save_info/get_info compiles against include/ and runs without a GPU; the new-style header is the
    one dftc.read_info parses, for the functional given by -DINTERACTIONS."""
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src, exe = tmp_path / "io.cpp", tmp_path / "io"
    src.write_text(IO_DRIVER)
    cmd = ["g++", "-O1", "-DNX=64", "-DNY=32", "-DNZ=16", "-DINTERACTIONS=0", "-I", os.path.join(root, "include"),
           "-I", "/usr/local/cuda/include", str(src), "-L", os.path.dirname(gpe_lib), "-lgpe_gb300",
           "-Wl,-rpath," + os.path.dirname(gpe_lib), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    out = {l.split()[0]: l.split()[1:] for l in r.stdout.splitlines() if l.strip()}
    assert [float(x) for x in out["NEW"]] == [64, 32, 16, 0.125, 3, 2.5, 1.5, 0.04, 0.0, 1000.0, 12.5]
    assert [float(x) for x in out["OLD"]] == [8, 16, 32, 0.5, 2, 1.25, 2.0, 0.1, 3.0, 10.0]
    assert out["TIME"] == ["1", "1"]
    info = dftc.read_info(str(tmp_path / "run.dftc"))
    assert (info.system, info.mode, info.nx, info.total_time) == ("fermions", "unitary", 64, 12.5)
    old = open(tmp_path / "old.dftc.info").read().splitlines()
    assert len(old) == 10 and old[0] == "8   # nx" and old[3] == "0.500000   # dt"


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [g.FP64, g.FP32])
def test_snapshots_match_get_psi(tmp_path, cuda_device, gpe_lib, precision):
    shape = (32, 16, 64)
    e = g.Engine(shape, 0, 1.0, 0.0, 0.05, 1000.0, precision=precision)
    e.set_user_params([0.04, 0.04, 0.06, 0.0])
    e.set_quantum_friction_coeff(0.1)
    e.set_psi(0.0, configs.random_state(shape, seed=3, npart=1000.0, gamma=2.0))
    path = str(tmp_path / "frames.dftc")
    sm = dftc.system_mode(0)
    info = dftc.Info(sm[0], sm[1], *shape, 0.05, 0, 0.0, 1.5, 0.04, 0.0, 1000.0)
    expect = []
    with dftc.Snapshots(e, path, nbuf=2, info=info) as snaps:
        for k in range(5):
            e.evolve_qf(3)
            t = snaps.push()
            expect.append(e.get_psi())
            assert t == pytest.approx(expect[-1][0])
    frames = dftc.read_frames(path)
    assert frames.shape == (5,) + shape
    for k in range(5):
        assert np.array_equal(frames[k], expect[k][1]), k
    back = dftc.read_info(path)
    assert back.nom == 5 and back.total_time == pytest.approx(expect[-1][0])
    assert os.path.getsize(path) == 5 * 16 * np.prod(shape)
