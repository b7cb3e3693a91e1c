"""GPU: the transform kernels through the C-ABI against the reference's transform conventions
(python/conatus/reference/transforms.py, restated in oracle/ivp.py): 1e-13 relative, the bar of
the reference's own transform tests (tests/core/test_core_transforms.py:25-38)."""
from __future__ import annotations

import numpy as np
import pytest

from oracle import ivp as oi

pytestmark = pytest.mark.gpu
TOL = 1e-13


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("N,M", [(16, 24), (17, 30), (64, 96), (129, 200), (128, 192)])
def test_chebyshev_round_trip_and_values(N, M, rng, cuda_lib):
    import torch
    from conatus_gb300._lib import call
    cols = 37
    c = rng.standard_normal((cols, N)) + 1j * rng.standard_normal((cols, N))
    f_ref = oi.cheb_backward(c.T, M).T
    cin = torch.as_tensor(c, device="cuda")
    f = torch.zeros((cols, M), dtype=torch.complex128, device="cuda")
    call("cng_cheb_transform", 0, cin.data_ptr(), f.data_ptr(), cols, N, M, None)
    back = torch.zeros((cols, N), dtype=torch.complex128, device="cuda")
    call("cng_cheb_transform", 1, f.data_ptr(), back.data_ptr(), cols, N, M, None)
    torch.cuda.synchronize()
    assert _rel(f.cpu().numpy(), f_ref) < TOL
    assert _rel(back.cpu().numpy(), c) < TOL
    g = rng.standard_normal((cols, M)) + 1j * rng.standard_normal((cols, M))
    gi = torch.as_tensor(g, device="cuda")
    call("cng_cheb_transform", 1, gi.data_ptr(), back.data_ptr(), cols, N, M, None)
    torch.cuda.synchronize()
    assert _rel(back.cpu().numpy(), oi.cheb_forward(g.T, N).T) < TOL


@pytest.mark.parametrize("Nc,L,inner", [(8, 12, 5), (192, 288, 24), (64, 96, 3)])
def test_complex_fft_axis(Nc, L, inner, rng, cuda_lib):
    import torch
    from conatus_gb300._lib import call
    outer = 3
    K = Nc // 2
    spec = rng.standard_normal((outer, Nc, inner)) + 1j * rng.standard_normal((outer, Nc, inner))
    spec[:, K] = 0
    full = np.zeros((outer, L, inner), complex)
    full[:, :K] = spec[:, :K]
    full[:, L - K + 1:] = spec[:, K + 1:]
    ref = np.fft.ifft(full, axis=1) * L
    si = torch.as_tensor(spec, device="cuda")
    g = torch.zeros((outer, L, inner), dtype=torch.complex128, device="cuda")
    call("cng_fft_axis", 0, si.data_ptr(), g.data_ptr(), outer, inner, Nc, L, None)
    back = torch.zeros_like(si)
    call("cng_fft_axis", 1, g.data_ptr(), back.data_ptr(), outer, inner, Nc, L, None)
    torch.cuda.synchronize()
    assert _rel(g.cpu().numpy(), ref) < TOL
    assert _rel(back.cpu().numpy(), spec) < TOL


@pytest.mark.parametrize("K,L,inner", [(4, 12, 6), (96, 288, 40), (128, 384, 8)])
def test_real_fft_axis(K, L, inner, rng, cuda_lib):
    import torch
    from conatus_gb300._lib import call
    outer = 2
    spec = rng.standard_normal((outer, K, inner)) + 1j * rng.standard_normal((outer, K, inner))
    spec[:, 0] = spec[:, 0].real
    F = np.zeros((outer, L // 2 + 1, inner), complex)
    F[:, :K] = spec
    ref = np.fft.irfft(F, n=L, axis=1) * L
    si = torch.as_tensor(spec, device="cuda")
    g = torch.zeros((outer, L, inner), dtype=torch.float64, device="cuda")
    call("cng_rfft_axis", 0, si.data_ptr(), g.data_ptr(), outer, inner, K, L, None)
    back = torch.zeros_like(si)
    call("cng_rfft_axis", 1, g.data_ptr(), back.data_ptr(), outer, inner, K, L, None)
    torch.cuda.synchronize()
    assert _rel(g.cpu().numpy(), ref) < TOL
    assert _rel(back.cpu().numpy(), spec) < TOL
