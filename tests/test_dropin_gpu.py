"""A driver written against the reference API (include/gpe_engine.h, C++ linkage, lattice and
functional fixed with -DNX -DNY -DNZ -DINTERACTIONS as the reference's drivers are built) runs end to
end on the GPU through libgpe_gb300.so; its psi, mu and energies match the CPU oracle."""
import os
import subprocess

import numpy as np
import pytest

import oracle
from libcugpe_gb300 import configs

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

DRIVER = r"""
#include <cstdio>
#include <vector>
#include "gpe_engine.h"
// ITE with normalisation, then RTE with quantum friction, as test_compare/gpe_imag.c and gpe_real.c do
int main(int argc, char** argv) {
    int nx, ny, nz;
    gpe_get_lattice(&nx, &ny, &nz);
    const size_t n = (size_t)nx * ny * nz;
    std::vector<cuCplx> psi(n);
    FILE* f = fopen(argv[1], "rb");
    if (!f || fread(psi.data(), sizeof(cuCplx), n, f) != n) return 3;
    fclose(f);
    double p[4] = {0.04, 0.04, 0.06, 0.0}, mu = 0.0, t, ek, ei, ee;
    int ierr = 0;
    gpe_exec(gpe_create_engine(0.0, 1.0, 0.05, 1000.0), ierr);
    gpe_exec(gpe_set_user_params(4, p), ierr);
    gpe_exec(gpe_set_psi(0.0, psi.data()), ierr);
    gpe_exec(gpe_normalize_psi(), ierr);
    gpe_exec(gpe_evolve_qf(20, &mu), ierr);
    gpe_exec(gpe_energy(&t, &ek, &ei, &ee), ierr);
    printf("ITE %.17g %.17g %.17g %.17g %.17g\n", mu, t, ek, ei, ee);
    gpe_exec(gpe_set_rte_evolution(), ierr);
    gpe_exec(gpe_set_quantum_friction_coeff(0.1), ierr);
    gpe_exec(gpe_evolve_qf(15), ierr);
    gpe_exec(gpe_get_psi(&t, psi.data()), ierr);
    FILE* g = fopen(argv[2], "wb");
    fwrite(psi.data(), sizeof(cuCplx), n, g);
    fclose(g);
    gpe_exec(gpe_energy(&t, &ek, &ei, &ee), ierr);
    printf("RTE %.17g %.17g %.17g %.17g\n", t, ek, ei, ee);
    gpe_exec(gpe_destroy_engine(), ierr);
    return ierr;
}
"""


def test_reference_style_driver_runs_on_gpu(cuda_device, gpe_lib, tmp_path):
    shape = (16, 32, 16)
    src, exe = tmp_path / "driver.cpp", tmp_path / "driver"
    src.write_text(DRIVER)
    cmd = ["g++", "-O2", "-DNX=16", "-DNY=32", "-DNZ=16", "-DINTERACTIONS=0", "-I", os.path.join(ROOT, "include"),
           "-I", "/usr/local/cuda/include", str(src), "-L", os.path.dirname(gpe_lib), "-lgpe_gb300",
           "-Wl,-rpath," + os.path.dirname(gpe_lib), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    psi0 = configs.random_state(shape, seed=41, npart=1000.0, gamma=2.0)
    inp, outp = tmp_path / "psi0.bin", tmp_path / "psi1.bin"
    psi0.astype(np.complex128).tofile(inp)
    r = subprocess.run([str(exe), str(inp), str(outp)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = {l.split()[0]: [float(x) for x in l.split()[1:]] for l in r.stdout.splitlines() if l.strip()}
    o = oracle.Oracle(shape, 0, 0.0, 1.0, 0.05, 1000.0, threads=4)
    o.set_user_params([0.04, 0.04, 0.06, 0.0])
    o.set_psi(0.0, psi0)
    o.normalize_psi()
    mu = o.evolve_qf(20)
    t, ek, ei, ee = o.energy()
    assert lines["ITE"][0] == pytest.approx(mu, rel=1e-10)
    for a, b in zip(lines["ITE"][2:], (ek, ei, ee)):
        assert a == pytest.approx(b, rel=1e-10)
    o.change_alpha_beta(1.0, 0.0)
    o.set_quantum_friction_coeff(0.1)
    o.evolve_qf(15)
    _, po = o.get_psi()
    ours = np.fromfile(outp, dtype=np.complex128).reshape(shape)
    assert float(np.linalg.norm(ours - po) / np.linalg.norm(po)) <= 1e-11
    t, ek, ei, ee = o.energy()
    for a, b in zip(lines["RTE"][1:], (ek, ei, ee)):
        assert a == pytest.approx(b, rel=1e-10)


QUEUE_DRIVER = r"""
#include <cstdio>
#include <vector>
#include "gpe_queue.h"
// the frame-queue pattern of test_vortex/rte_vortex.c: one thread evolves and queues frames of psi,
// a second one writes them to a file
gpe_queue wf_queue;
int main(int argc, char** argv) {
    int nx, ny, nz;
    gpe_get_lattice(&nx, &ny, &nz);
    const size_t n = (size_t)nx * ny * nz;
    std::vector<cuCplx> psi0(n);
    FILE* f = fopen(argv[1], "rb");
    if (!f || fread(psi0.data(), sizeof(cuCplx), n, f) != n) return 3;
    fclose(f);
    double p[4] = {0.04, 0.04, 0.06, 0.0}, t;
    int ierr = 0;
    gpe_exec(gpe_create_engine(1.0, 0.0, 0.05, 1000.0), ierr);
    gpe_exec(gpe_set_user_params(4, p), ierr);
    gpe_exec(gpe_set_quantum_friction_coeff(0.1), ierr);
    gpe_exec(gpe_set_psi(0.0, psi0.data()), ierr);
    create_gpe_queue(n, 5);
    FILE* frames = fopen(argv[2], "wb");
    int written = 0;
#pragma omp parallel num_threads(2)
    {
#pragma omp sections
        {
#pragma omp section
            {
                for (int k = 0; k < 10; k++) {
                    cplx* psi = get_gpe_queue_buffer();
                    gpe_exec(gpe_evolve_qf(5), ierr);
                    gpe_exec(gpe_get_psi(&t, (cuCplx*)psi), ierr);
                    add_to_gpe_queue(psi);
                }
                flag_stop = 1;
            }
#pragma omp section
            {
                while (1) {
                    if (wf_queue.q.empty()) {
                        if (wf_queue.q.empty() && flag_stop) break;
                    } else {
                        cplx* buf = take_off_gpe_queue();
                        fwrite(buf, sizeof(cplx) * n, 1, frames);
                        written++;
                    }
                }
            }
        }
    }
    fclose(frames);
    destroy_gpe_queue();
    gpe_exec(gpe_destroy_engine(), ierr);
    printf("FRAMES %d\n", written);
    return ierr;
}
"""


def test_reference_frame_queue_driver(cuda_device, gpe_lib, tmp_path):
    """include/gpe_queue.h: a driver using the reference's queue API (two OpenMP sections, as
    test_vortex/rte_vortex.c) writes 10 frames; each equals the psi the engine gives after the same
    number of steps."""
    import libcugpe_gb300 as g
    shape = (16, 16, 32)
    src, exe = tmp_path / "qdriver.cpp", tmp_path / "qdriver"
    src.write_text(QUEUE_DRIVER)
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-DNX=16", "-DNY=16", "-DNZ=32", "-DINTERACTIONS=0",
           "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include", str(src),
           "-L", os.path.dirname(gpe_lib), "-lgpe_gb300", "-L", "/usr/local/cuda/lib64", "-lcudart",
           "-Wl,-rpath," + os.path.dirname(gpe_lib), "-Wl,-rpath,/usr/local/cuda/lib64", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    psi0 = configs.random_state(shape, seed=42, npart=1000.0, gamma=2.0)
    inp, outp = tmp_path / "psi0.bin", tmp_path / "frames.bin"
    psi0.astype(np.complex128).tofile(inp)
    r = subprocess.run([str(exe), str(inp), str(outp)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "FRAMES 10" in r.stdout
    frames = np.fromfile(outp, dtype=np.complex128).reshape((10,) + shape)
    e = g.Engine(shape, 0, 1.0, 0.0, 0.05, 1000.0)
    e.set_user_params([0.04, 0.04, 0.06, 0.0])
    e.set_quantum_friction_coeff(0.1)
    e.set_psi(0.0, psi0)
    for k in range(10):
        e.evolve_qf(5)
        assert np.array_equal(frames[k], e.get_psi()[1]), k
    e.close()
