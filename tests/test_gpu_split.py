"""GPU tests of the split-precision tensor-core transforms
(MUFFT_GB_FLAG_SPLIT_BF16X3 / _BF16X2).  No reference counterpart: the
oracle is the FP64 DFT (numpy), and the plain FP32 path measured on the same
input sets the error the three-limb form has to match."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import max_abs, rel_l2
from mufft_gb300 import capi as K
from mufft_gb300 import signals

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import mufft_gb300
    return mufft_gb300.load()


@pytest.fixture(params=[0, 1], ids=["tcgen05", "mma.sync"])
def engine(request, gpu):
    """Plan options selecting the split-precision engine."""
    return gpu.options(split_engine=request.param)


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available()
    return t


def run(gpu, torch, x, direction, flags, opts=None):
    B, N = x.shape
    dx = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    dy = torch.full_like(dx, complex(float("nan"), 0))
    plan = gpu.gb_create_plan_1d(0, N, direction, flags, B, 0, 0, C.byref(opts) if opts else None)
    assert plan, gpu.gb_last_error_string()
    try:
        rc = gpu.gb_execute_plan_1d_async(plan, dy.data_ptr(), dx.data_ptr(), torch.cuda.current_stream().cuda_stream)
        assert rc == 0, gpu.gb_last_error_string()
        torch.cuda.synchronize()
    finally:
        gpu.free_plan_1d(plan)
    return dy.cpu().numpy()


def ref_f64(x, direction):
    X = np.fft.fft(x.astype(np.complex128), axis=1)
    return X if direction == K.FORWARD else np.conj(np.fft.fft(np.conj(x.astype(np.complex128)), axis=1))


def inputs(kind, seed, B, N):
    if kind == "uniform":
        return signals.complex_uniform(seed, B * N).reshape(B, N)
    return signals.complex_logmag(seed, B * N).reshape(B, N)  # magnitudes 1e-3..1e3


@pytest.mark.parametrize("N,B", [(4096, 1), (4096, 37), (4096, 1000), (256, 1), (256, 100), (256, 4096)])
@pytest.mark.parametrize("direction", [K.FORWARD, K.INVERSE])
@pytest.mark.parametrize("kind", ["uniform", "logmag"])
def test_split_bf16x3_matches_fp32_error(gpu, torch, engine, N, B, direction, kind):
    x = inputs(kind, 40000 + N + B, B, N)
    ref = ref_f64(x, direction)
    split = run(gpu, torch, x, direction, K.FLAG_SPLIT_BF16X3, engine)
    plain = run(gpu, torch, x, direction, 0)
    e_split, e_plain = rel_l2(split, ref), rel_l2(plain, ref)
    assert np.all(np.isfinite(split))
    # FP32-level: within a small factor of the plain FP32 path and under 1e-6
    assert e_split < 1e-6 and e_split < 3 * e_plain, (e_split, e_plain)
    assert max_abs(split, ref) < 20 * max(max_abs(plain, ref), 1e-30) + 1e-6 * np.abs(ref).max()


@pytest.mark.parametrize("N,B", [(4096, 9), (256, 64)])
@pytest.mark.parametrize("kind", ["uniform", "logmag"])
def test_split_bf16x2_error(gpu, torch, engine, N, B, kind):
    x = inputs(kind, 41000 + N + B, B, N)
    for direction in (K.FORWARD, K.INVERSE):
        got = run(gpu, torch, x, direction, K.FLAG_SPLIT_BF16X2, engine)
        e = rel_l2(got, ref_f64(x, direction))
        assert 1e-7 < e < 5e-5, e  # two limbs: ~16 significant bits


@pytest.mark.parametrize("N,dist", [(4096, 4096 + 64), (4096, 4097), (256, 257), (256, 300)])
def test_split_strided_batch(gpu, torch, engine, N, dist):
    """Padded batch distances go through the split path too (odd distances
    take the per-thread loads instead of bulk copies)."""
    B = 5
    x = np.zeros((B, dist), np.complex64)
    x[:, :N] = signals.complex_uniform(42000, B * N).reshape(B, N)
    dx = torch.from_numpy(x).cuda()
    dy = torch.zeros_like(dx)
    plan = gpu.gb_create_plan_1d(0, N, K.FORWARD, K.FLAG_SPLIT_BF16X3, B, dist, dist, C.byref(engine))
    assert plan
    assert gpu.gb_execute_plan_1d_async(plan, dy.data_ptr(), dx.data_ptr(),
                                        torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    gpu.free_plan_1d(plan)
    y = dy.cpu().numpy()
    assert rel_l2(y[:, :N], ref_f64(x[:, :N], K.FORWARD)) < 1e-6
    assert np.all(y[:, N:] == 0)
