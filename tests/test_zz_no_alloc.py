"""gpe_gb_norm_noalloc: the norm for callers that cannot allocate device memory.

Callers inside stream capture, applications whose own pool owns all device
memory, or plugins in hosts that forbid allocation after start-up cannot let
the library call cudaMalloc.  This entry point computes sum gamma |psi|^2 of
a wavefunction the caller already holds on the device, into a device double
the caller provides, using only a fixed scratch array inside the library.
Here it is called twice in a row through the C ABI and compared with the
engine's own gpe_gb_get_norm on the same wavefunction.  The file is named to
be collected last.
"""
import ctypes

import numpy as np
import pytest

import libcugpe_gb300 as g
from libcugpe_gb300 import configs

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", [(32, 16, 64), (64, 64, 64)], ids=["32k", "256k"])
@pytest.mark.parametrize("precision", [g.FP64, g.FP32])
def test_norm_noalloc_matches_get_norm_twice(cuda_device, gpe_lib, precision, shape):
    """Both lattices: one smaller than the kernel's fixed grid (most CTAs sum nothing), one larger (the
    grid-stride loop runs twice)."""
    import torch
    gamma = 2.0
    psi = 3.0 * configs.random_state(shape, seed=17, npart=10.0, gamma=gamma)
    e = g.Engine(shape, 0, 1.0, 0.0, 0.05, 10.0, precision=precision)
    e.set_psi(0.0, psi)
    ref = e.get_norm()  # the existing entry point
    ctype = torch.complex128 if precision == g.FP64 else torch.complex64
    dpsi = torch.from_numpy(psi.astype(np.complex128)).to(ctype).to(cuda_device)
    out = torch.full((1,), -1.0, dtype=torch.float64, device=cuda_device)
    torch.cuda.synchronize()
    lib = g._lib()
    for call in range(2):
        out.fill_(-1.0)
        torch.cuda.synchronize()
        rc = lib.gpe_gb_norm_noalloc(ctypes.c_void_p(dpsi.data_ptr()), precision, dpsi.numel(), gamma,
                                     ctypes.c_void_p(out.data_ptr()), None)
        assert rc == 0, lib.gpe_gb_error_string(rc)
        torch.cuda.synchronize()
        assert abs(out.item() - ref) <= 1e-12 * abs(ref), (call, out.item(), ref)
    e.close()


@pytest.mark.parametrize("precision", [g.FP64, g.FP32])
def test_norm_noalloc_ragged_count(cuda_device, gpe_lib, precision):
    """A point count that is no multiple of the fixed grid (64*64*37 points of a larger buffer), twice in
    a row, against an FP64 sum of the same values on the host."""
    import torch
    shape = (64, 64, 64)
    n = 64 * 64 * 37
    gamma = 1.0
    psi = configs.random_state(shape, seed=23, npart=5.0, gamma=gamma).reshape(-1)
    ctype = torch.complex128 if precision == g.FP64 else torch.complex64
    dpsi = torch.from_numpy(psi.astype(np.complex128)).to(ctype).to(cuda_device)
    host = dpsi[:n].cpu().numpy().astype(np.complex128)
    ref = float(gamma * np.sum(host.real * host.real + host.imag * host.imag))
    out = torch.full((1,), -1.0, dtype=torch.float64, device=cuda_device)
    lib = g._lib()
    for call in range(2):
        out.fill_(-1.0)
        torch.cuda.synchronize()
        rc = lib.gpe_gb_norm_noalloc(ctypes.c_void_p(dpsi.data_ptr()), precision, n, gamma,
                                     ctypes.c_void_p(out.data_ptr()), None)
        assert rc == 0, lib.gpe_gb_error_string(rc)
        torch.cuda.synchronize()
        assert abs(out.item() - ref) <= 1e-12 * abs(ref), (call, out.item(), ref)


def test_norm_noalloc_rejects_oversize_and_bad_arguments(cuda_device, gpe_lib):
    import torch
    lib = g._lib()
    buf = torch.zeros(2, dtype=torch.float64, device=cuda_device)
    p = ctypes.c_void_p(buf.data_ptr())
    assert lib.gpe_gb_norm_noalloc(p, g.FP64, (1 << 27) + 1, 1.0, p, None) == g.ERR_NOALLOC_SIZE
    assert lib.gpe_gb_norm_noalloc(p, g.FP64, 0, 1.0, p, None) == g.ERR_NOALLOC_SIZE
    assert lib.gpe_gb_norm_noalloc(None, g.FP64, 1, 1.0, p, None) == g.ERR_ARGUMENT
    assert lib.gpe_gb_norm_noalloc(p, 7, 1, 1.0, p, None) == g.ERR_ARGUMENT
