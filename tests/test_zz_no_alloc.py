"""mufft_gb_execute_c2c_noalloc: the allocation-free complex FFT for callers
that cannot allocate GPU memory when they transform (a real-time audio
callback, a plugin whose host owns the device memory).  Its output must equal
the plan-based execute's, and two calls in a row must both be right, since
every call reuses the same fixed scratch array.  This file is collected last
so that a run stopping at the first failure has run every other test."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import REL_L2_TOL, rel_l2
from mufft_gb300 import capi as K
from mufft_gb300 import signals

pytestmark = pytest.mark.gpu

MAX_POINTS = 1 << 20


@pytest.fixture(scope="module")
def env():
    import torch

    import mufft_gb300
    assert torch.cuda.is_available()
    return mufft_gb300.load(), torch


def _plan_result(lib, torch, N, direction, dx):
    dy = torch.empty_like(dx)
    plan = lib.create_plan_1d_c2c(N, direction, 0)
    assert plan, lib.gb_last_error_string()
    assert lib.gb_execute_plan_1d_async(plan, dy.data_ptr(), dx.data_ptr(),
                                        torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    lib.free_plan_1d(plan)
    return dy.cpu().numpy()


@pytest.mark.parametrize("N,direction", [(MAX_POINTS, K.FORWARD), (1 << 17, K.INVERSE), (4096, K.FORWARD)])
def test_noalloc_matches_plan_twice(env, N, direction):
    lib, torch = env
    st = torch.cuda.current_stream().cuda_stream
    inputs = [signals.complex_uniform(31000 + N, N), signals.complex_uniform(32000 + N, N)]
    for x in inputs:  # two calls in a row, different data, shared scratch
        dx = torch.from_numpy(x).cuda()
        dy = torch.full_like(dx, float("nan"))
        rc = lib.gb_execute_c2c_noalloc(N, direction, dy.data_ptr(), dx.data_ptr(), st)
        assert rc == 0, rc
        torch.cuda.synchronize()
        got = dy.cpu().numpy()
        want = _plan_result(lib, torch, N, direction, dx)
        assert np.all(np.isfinite(got))
        assert rel_l2(got, want) <= REL_L2_TOL


def test_noalloc_rejects_sizes_beyond_the_scratch(env):
    lib, torch = env
    dx = torch.zeros(2 * MAX_POINTS, dtype=torch.complex64, device="cuda")
    dy = torch.zeros_like(dx)
    assert lib.gb_execute_c2c_noalloc(2 * MAX_POINTS, K.FORWARD, dy.data_ptr(), dx.data_ptr(), None) == -2
    assert lib.gb_execute_c2c_noalloc(3000, K.FORWARD, dy.data_ptr(), dx.data_ptr(), None) == -1
    x = np.zeros(16, np.complex64)
    assert lib.gb_execute_c2c_noalloc(16, K.FORWARD, dy.data_ptr(), x.ctypes.data, None) == -4
