"""User hooks (include/gpe_user_defined.h) compiled into the pass kernels.

The reference's plugin surface is a header of compile-time __device__ hooks
(dev/gpe_user_defined.h): gpe_external_potential, gpe_dEDFdn, gpe_EDF and
gpe_modify_psi, evaluated inside its pointwise kernels at `it` and `it + 1`
(dev/gpe_engine.cu:733-735, 758-760, 789, 794, 829-834, 855-861).  Here a
library is built from a hook header (libcugpe_gb300.build, small lattices
only) and checked three ways:

* the header's Woods-Saxon tube (VEXT 1) against the reference engine built
  with -DVEXT=1: <= 1e-12 relative L2 per step, energies after 20 steps;
* a user header whose potential, functional and gpe_modify_psi all depend on
  the step (tests/hooks/moving_trap_kick.h) against the CPU oracle evaluating
  the same header compiled for the host;
* the default header against the library without hooks: the same FP64 arithmetic (to the last few
  units of rounding, which fused multiply-adds the compiler chose apart).
"""
import os

import numpy as np
import pytest

import libcugpe_gb300 as g
from libcugpe_gb300 import build, configs
import oracle
from oracle import build_ref, ref_run

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
DEFAULT_HEADER = os.path.join(ROOT, "include", "gpe_user_defined.h")
KICK_HEADER = os.path.join(HERE, "hooks", "moving_trap_kick.h")


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def hook_library(name, header, defines, precisions=("f64",)):
    return build.build(hooks=header, name=name, defines=tuple(defines), lengths=[16, 32],
                       precisions=list(precisions), batch=False)


@pytest.fixture(scope="module")
def tube_lib(cuda_device, gpe_lib):
    return hook_library("test_tube", DEFAULT_HEADER, ["INTERACTIONS=0", "VEXT=1"])


@pytest.fixture(scope="module")
def kick_lib(cuda_device, gpe_lib):
    return hook_library("test_kick", KICK_HEADER, ["INTERACTIONS=-1"], precisions=("f64", "f32"))


@pytest.fixture(scope="module")
def default_lib(cuda_device, gpe_lib):
    return hook_library("test_default", DEFAULT_HEADER, ["INTERACTIONS=0", "VEXT=0"], precisions=("f64", "f32"))


def test_hook_library_reports_its_functional(tube_lib, kick_lib):
    assert g.user_hooks(tube_lib) == (True, 0)
    assert g.user_hooks(kick_lib) == (True, -1)
    assert g.user_hooks(None) == (False, 0)
    with pytest.raises(g.GPEError) as ex:  # compiled for INTERACTIONS -1 only
        g.Engine((16, 16, 16), 0, 1.0, 0.0, 0.05, 10.0, library=kick_lib)
    assert ex.value.code == g.ERR_FUNCTIONAL


# Woods-Saxon tube: d_user_param[V_0, A, R] = depth, width, radius; the UFG functional
TUBE = [2.0, 1.5, 6.0, 0.0]
TUBE_CASES = [
    # shape, alpha, beta, dt, qf
    ((32, 32, 16), 1.0, 0.0, 0.05, 0.1),
    ((16, 32, 32), 0.0, 1.0, 0.05, 0.0),
]


@pytest.mark.parametrize("case", TUBE_CASES, ids=lambda c: f"{c[0]}_b{c[2]}_qf{c[4]}")
def test_woods_saxon_tube_matches_reference(tube_lib, case):
    if not ref_run.available():
        pytest.skip("reference sources not available on this machine")
    shape, alpha, beta, dt, qf = case
    npart = 100.0
    psi = configs.random_state(shape, seed=31, npart=npart, gamma=2.0)
    build_ref.build_one(*shape, 0, vext=1)
    out = ref_run.run(shape, 0, alpha, beta, dt, npart, TUBE, psi, ["S1", "D", "S1", "D", "S1", "D"], qf=qf, vext=1)
    prev = psi
    for k, ref in enumerate(out["psi"]):
        e = g.Engine(shape, 0, alpha, beta, dt, npart, library=tube_lib)
        e.set_user_params(TUBE)
        if qf:
            e.set_quantum_friction_coeff(qf)
        e.set_psi(0.0, prev)
        e.evolve_qf(1)
        _, ours = e.get_psi()
        e.close()
        assert rel(ours, ref) <= 1e-12, (k, rel(ours, ref))
        prev = ref
    out = ref_run.run(shape, 0, alpha, beta, dt, npart, TUBE, psi, ["E", "S20", "E", "D"], qf=qf, vext=1)
    e = g.Engine(shape, 0, alpha, beta, dt, npart, library=tube_lib)
    e.set_user_params(TUBE)
    if qf:
        e.set_quantum_friction_coeff(qf)
    e.set_psi(0.0, psi)
    e0 = e.energy()
    e.evolve_qf(20)
    e1 = e.energy()
    _, ours = e.get_psi()
    e.close()
    assert rel(ours, out["psi"][0]) <= 1e-11
    for ours_e, ref_e in ((e0, out["energy"][0]), (e1, out["energy"][1])):
        for a, b in zip(ours_e[1:], ref_e[1:]):
            assert abs(a - b) <= 1e-10 * max(1.0, abs(b)), (a, b)


# moving trap, modulated scattering length, phase kicks: [wx, wy, wz, a, shift, drive, a_mod, kick]
KICK = [0.06, 0.05, 0.07, 8.0, 1.5, 0.9, 0.3, 0.05]
KICK_CASES = [
    # shape, alpha, beta, dt, qf, t0
    ((16, 16, 32), 1.0, 0.0, 0.05, 0.0, 0.3),
    ((32, 16, 16), 1.0, 0.0, 0.05, 0.1, 0.0),
    ((16, 32, 16), 0.0, 1.0, 0.05, 0.0, 1.1),
]


@pytest.mark.parametrize("case", KICK_CASES, ids=lambda c: f"{c[0]}_b{c[2]}_qf{c[4]}")
def test_time_dependent_user_hooks_match_oracle(kick_lib, case):
    shape, alpha, beta, dt, qf, t0 = case
    hooks = oracle.Hooks(oracle.build_hooks(KICK_HEADER, "test_kick", ["INTERACTIONS=-1"]))
    assert hooks.interactions == -1
    psi = configs.random_state(shape, seed=32, npart=1.0, gamma=1.0)
    o = oracle.Oracle(shape, -1, alpha, beta, dt, 1.0, threads=4)
    o.set_hooks(hooks)
    o.set_user_params(KICK)
    o.set_quantum_friction_coeff(qf)
    o.set_psi(t0, psi)
    e = g.Engine(shape, -1, alpha, beta, dt, 1.0, library=kick_lib)
    e.set_user_params(KICK)
    if qf:
        e.set_quantum_friction_coeff(qf)
    e.set_psi(t0, psi)
    done = 0
    for steps, tol in ((1, 1e-12), (4, 3e-12), (15, 1e-11)):
        mo = o.evolve_qf(steps)
        me = e.evolve_qf(steps)
        done += steps
        _, ref = o.get_psi()
        _, ours = e.get_psi()
        assert rel(ours, ref) <= tol, (done, rel(ours, ref))
        if beta != 0.0:
            assert abs(me - mo) <= 1e-10 * max(1.0, abs(mo)), (me, mo)
    eo, ee = o.energy(), e.energy()
    assert ee[0] == pytest.approx(eo[0], abs=1e-12)
    for a, b in zip(ee[1:], eo[1:]):
        assert abs(a - b) <= 1e-10 * max(1.0, abs(b)), (a, b)
    # the hooks must act: the same run with the built-in physics ends elsewhere
    plain = g.Engine(shape, -1, alpha, beta, dt, 1.0)
    plain.set_user_params(KICK[:4])
    if qf:
        plain.set_quantum_friction_coeff(qf)
    plain.set_psi(t0, psi)
    plain.evolve_qf(done)
    assert rel(plain.get_psi()[1], ref) > 1e-3
    # FP32-mixed form of the same hook library
    f = g.Engine(shape, -1, alpha, beta, dt, 1.0, precision=g.FP32, library=kick_lib)
    f.set_user_params(KICK)
    if qf:
        f.set_quantum_friction_coeff(qf)
    f.set_psi(t0, psi)
    f.evolve_qf(done)
    assert rel(f.get_psi()[1], ref) <= 1e-4
    for x in (e, plain, f):
        x.close()


@pytest.mark.parametrize("qf", [0.0, 0.1])
def test_user_hooks_inside_the_plane_passes(kick_lib, qf):
    """FP32 real time on 128 x 128 yz-planes runs the hooks inside the plane kernel (Vstep1 and the
    corrector with the potential and functional at it and it + 1, gpe_modify_psi on psi_n): against the
    oracle evaluating the same header, FP32 tolerances."""
    shape, dt, t0 = (16, 128, 128), 0.05, 0.4
    hooks = oracle.Hooks(oracle.build_hooks(KICK_HEADER, "test_kick", ["INTERACTIONS=-1"]))
    psi = configs.random_state(shape, seed=34, npart=1.0, gamma=1.0)
    o = oracle.Oracle(shape, -1, 1.0, 0.0, dt, 1.0, threads=8)
    o.set_hooks(hooks)
    o.set_user_params(KICK)
    o.set_quantum_friction_coeff(qf)
    o.set_psi(t0, psi)
    e = g.Engine(shape, -1, 1.0, 0.0, dt, 1.0, precision=g.FP32, library=kick_lib)
    e.set_user_params(KICK)
    if qf:
        e.set_quantum_friction_coeff(qf)
    e.set_psi(t0, psi)
    for steps, tol in ((1, 2e-5), (9, 1e-4)):
        o.evolve_qf(steps)
        e.evolve_qf(steps)
        assert rel(e.get_psi()[1], o.get_psi()[1]) <= tol, (steps, rel(e.get_psi()[1], o.get_psi()[1]))
    # (the library holds 16- and 32-point pencils only: the plane passes carry every y and z transform)
    kinds = [p["kind"] for p in e.profile_passes(1)]
    assert kinds.count("plane") == 2 and len(kinds) == 4, kinds
    e.close()


DEFAULT_CASES = [
    # shape, alpha, beta, dt, qf
    ((16, 32, 32), 1.0, 0.0, 0.05, 0.1),
    ((32, 16, 16), 0.0, 1.0, 0.05, 0.1),
    ((32, 32, 16), 1.0, 0.0, 0.05, 0.0),
]


@pytest.mark.parametrize("case", DEFAULT_CASES, ids=lambda c: f"{c[0]}_b{c[2]}_qf{c[4]}")
def test_default_header_reproduces_builtin_physics(default_lib, case):
    """FP64: the same arithmetic as the library without hooks; the two libraries are separately
    compiled, and the compiler's choice of which products to fuse into multiply-adds may differ between
    them, so agreement is to a few units of the last place (3.7e-16 relative L2 measured), not bit for
    bit.  FP32: the hooks compute in FP64 before rounding, so only to FP32 accuracy."""
    shape, alpha, beta, dt, qf = case
    params = [0.04, 0.05, 0.06, 0.0]
    psi = configs.random_state(shape, seed=33, npart=100.0, gamma=2.0)
    for prec, exact in ((g.FP64, True), (g.FP32, False)):
        a = g.Engine(shape, 0, alpha, beta, dt, 100.0, precision=prec, library=default_lib)
        b = g.Engine(shape, 0, alpha, beta, dt, 100.0, precision=prec)
        for x in (a, b):
            x.set_user_params(params)
            if qf:
                x.set_quantum_friction_coeff(qf)
            x.set_psi(0.0, psi)
        for _ in range(3):
            ma, mb = a.evolve_qf(2), b.evolve_qf(2)
            pa, pb = a.get_psi()[1], b.get_psi()[1]
            if exact:
                assert rel(pa, pb) <= 2e-15, rel(pa, pb)
                assert abs(ma - mb) <= 1e-14 * max(1.0, abs(mb))
            else:
                assert rel(pa, pb) <= 1e-5
        ea, eb = a.energy(), b.energy()
        if exact:
            assert all(abs(x - y) <= 1e-14 * max(1.0, abs(y)) for x, y in zip(ea, eb))
        else:
            assert all(abs(x - y) <= 1e-5 * max(1.0, abs(y)) for x, y in zip(ea, eb))
        a.close()
        b.close()
