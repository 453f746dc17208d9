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
