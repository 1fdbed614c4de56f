"""GPU edge cases beyond the reference's sweeps: real transforms on the
three-level schedule, zero-padded multi-pass real inputs, padded batch
distances on multi-pass plans, very unbalanced 2D shapes and large batches
of tiny transforms.  FP64 (numpy) is the reference; the bar is the plain
path's accuracy (relative L2 within a few 1e-7, well under 1e-5)."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import rel_l2
from mufft_gb300 import capi as K
from mufft_gb300 import signals

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import mufft_gb300
    return mufft_gb300.load()


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available()
    return t


@pytest.mark.parametrize("lg", [23, 25])
def test_real_transforms_on_three_level_schedule(gpu, lg):
    """N real points -> N/2 complex on the three-level path, with the r2c
    fix-up in place afterwards, and back."""
    N = 1 << lg
    x = signals.uniform(70000 + lg, N)
    X = gpu.fft_r2c(x)
    ref = np.fft.rfft(x.astype(np.float64))
    assert rel_l2(X, ref) < 2e-6
    back = gpu.fft_c2r(X, N)
    assert rel_l2(back / N, x) < 4e-6


@pytest.mark.parametrize("lg", [17, 21])
def test_zero_padded_real_multipass(gpu, lg):
    N = 1 << lg
    xh = signals.uniform(71000 + lg, N // 2)
    X = gpu.fft_r2c(xh, K.FLAG_ZERO_PAD_UPPER_HALF, N)
    ref = np.fft.rfft(np.concatenate([xh, np.zeros(N // 2)]).astype(np.float64))
    assert rel_l2(X, ref) < 2e-6


@pytest.mark.parametrize("N,B,pad", [(1 << 17, 3, 64), (1 << 22, 2, 256), (4096, 5, 8)])
def test_padded_batch_distances(gpu, torch, N, B, pad):
    dist = N + pad
    x = np.zeros((B, dist), np.complex64)
    x[:, :N] = signals.complex_uniform(72000 + N, B * N).reshape(B, N)
    dx = torch.from_numpy(x).cuda()
    dy = torch.zeros_like(dx)
    plan = gpu.gb_create_plan_1d_c2c_batched(N, K.FORWARD, 0, B, dist, dist)
    assert plan, gpu.gb_last_error_string()
    assert gpu.gb_execute_plan_1d_async(plan, dy.data_ptr(), dx.data_ptr(), torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    gpu.free_plan_1d(plan)
    y = dy.cpu().numpy()
    ref = np.fft.fft(x[:, :N].astype(np.complex128), axis=1)
    assert rel_l2(y[:, :N], ref) < 2e-6
    assert np.all(y[:, N:] == 0)  # the padding is never written


@pytest.mark.parametrize("Nx,Ny", [(16384, 16), (16, 16384), (8192, 64), (2, 8192)])
def test_unbalanced_2d(gpu, Nx, Ny):
    x = signals.complex_uniform(73000 + Nx + Ny, Nx * Ny).reshape(Ny, Nx)
    got = gpu.fft2_c2c(x, K.FORWARD)
    assert rel_l2(got, np.fft.fft2(x.astype(np.complex128))) < 2e-6
    if Nx >= 4:
        xr = signals.uniform(73100 + Nx + Ny, Nx * Ny).reshape(Ny, Nx)
        X = gpu.fft2_r2c(xr)
        assert rel_l2(X[:, : Nx // 2 + 1], np.fft.rfft2(xr.astype(np.float64))) < 2e-6
        back = gpu.fft2_c2r(X)
        assert rel_l2(back / (Nx * Ny), xr) < 4e-6


@pytest.mark.parametrize("N,B", [(2, 1 << 20), (16, 1 << 18), (64, 100003)])
def test_large_batches_of_tiny_transforms(gpu, torch, N, B):
    x = signals.complex_uniform(74000 + N, N * B).reshape(B, N)
    dx = torch.from_numpy(x).cuda()
    dy = torch.empty_like(dx)
    plan = gpu.gb_create_plan_1d_c2c_batched(N, K.INVERSE, 0, B, 0, 0)
    assert plan, gpu.gb_last_error_string()
    assert gpu.gb_execute_plan_1d_async(plan, dy.data_ptr(), dx.data_ptr(), torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    gpu.free_plan_1d(plan)
    y = dy.cpu().numpy()
    rows = np.r_[0:4, B // 2:B // 2 + 4, B - 4:B]
    ref = np.fft.ifft(x[rows].astype(np.complex128), axis=1) * N
    assert rel_l2(y[rows], ref) < 2e-6


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("Nx,Ny", [(64, 64), (16, 2048), (4096, 4096), (2048, 8192), (8, 16384)])
def test_2d_column_schedules(gpu, mode, Nx, Ny):
    """2D columns as one pass of whole-column tiles (1) or as the two-pass
    four-step along the columns (2): c2c both directions, r2c and c2r."""
    opts = gpu.options(columns_2d=mode)
    x = signals.complex_uniform(75000 + Nx + Ny, Nx * Ny).reshape(Ny, Nx)
    ref = np.fft.fft2(x.astype(np.complex128))
    got = gpu.fft2_c2c(x, K.FORWARD, opts=opts)
    assert rel_l2(got, ref) < 2e-6
    inv = gpu.fft2_c2c(got, K.INVERSE, opts=opts)
    assert rel_l2(inv / (Nx * Ny), x) < 4e-6
    xr = signals.uniform(75100 + Nx + Ny, Nx * Ny).reshape(Ny, Nx)
    X = gpu.fft2_r2c(xr, opts=opts)
    assert rel_l2(X[:, : Nx // 2 + 1], np.fft.rfft2(xr.astype(np.float64))) < 2e-6
    back = gpu.fft2_c2r(X, opts=opts)
    assert rel_l2(back / (Nx * Ny), xr) < 4e-6
