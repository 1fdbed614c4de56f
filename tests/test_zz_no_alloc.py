"""mufft_gb_execute_c2c_noalloc: the allocation-free complex FFT for callers
that cannot allocate GPU memory when they transform (a real-time audio
callback, a plugin whose host owns the device memory).  Its output must match
the oracle at every size the fixed scratch allows and equal the plan-based
execute's, and two calls in a row must both be right, since every call
reuses the same fixed scratch array.  This file is collected last
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
    from oracle.oracle import load_oracle
    assert torch.cuda.is_available()
    return mufft_gb300.load(), torch, load_oracle()


def _plan_result(lib, torch, N, direction, dx):
    dy = torch.empty_like(dx)
    plan = lib.create_plan_1d_c2c(N, direction, 0)
    assert plan, lib.gb_last_error_string()
    assert lib.gb_execute_plan_1d_async(plan, dy.data_ptr(), dx.data_ptr(),
                                        torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    lib.free_plan_1d(plan)
    return dy.cpu().numpy()


# every size the fixed scratch allows: single-pass tiles up to 16384 points,
# the two-pass four-step above; both directions
SIZES = [(1 << lg, d) for lg in range(1, 21) for d in (K.FORWARD, K.INVERSE)]


@pytest.mark.parametrize("N,direction", SIZES, ids=[f"{n}-{'fwd' if d < 0 else 'inv'}" for n, d in SIZES])
def test_noalloc_matches_oracle_twice(env, N, direction):
    """Two calls in a row on different data (the second reuses the scratch the
    first left behind), each against the oracle's c2c of the same input."""
    lib, torch, ora = env
    st = torch.cuda.current_stream().cuda_stream
    for seed in (31000 + N, 32000 + N):
        x = signals.complex_uniform(seed + (direction > 0), N)
        dx = torch.from_numpy(x).cuda()
        dy = torch.full_like(dx, float("nan"))
        rc = lib.gb_execute_c2c_noalloc(N, direction, dy.data_ptr(), dx.data_ptr(), st)
        assert rc == 0, rc
        torch.cuda.synchronize()
        got = dy.cpu().numpy()
        want = ora.c2c_many(x.reshape(1, N), direction, 1)[0]
        assert np.all(np.isfinite(got))
        assert rel_l2(got, want) <= REL_L2_TOL, (N, direction, rel_l2(got, want))


@pytest.mark.parametrize("N,direction", [(MAX_POINTS, K.FORWARD), (1 << 17, K.INVERSE), (4096, K.FORWARD)])
def test_noalloc_matches_plan(env, N, direction):
    """The allocation-free call and the plan-based execute agree."""
    lib, torch, _ = env
    st = torch.cuda.current_stream().cuda_stream
    x = signals.complex_uniform(33000 + N, N)
    dx = torch.from_numpy(x).cuda()
    dy = torch.full_like(dx, float("nan"))
    assert lib.gb_execute_c2c_noalloc(N, direction, dy.data_ptr(), dx.data_ptr(), st) == 0
    torch.cuda.synchronize()
    assert rel_l2(dy.cpu().numpy(), _plan_result(lib, torch, N, direction, dx)) <= REL_L2_TOL


@pytest.mark.parametrize("N,direction", [(8, K.INVERSE), (16384, K.INVERSE), (1 << 18, K.FORWARD),
                                         (MAX_POINTS, K.INVERSE)])
def test_noalloc_in_place(env, N, direction):
    """output == input: the single-pass tile reads everything before it
    stores; the four-step's first pass reads the input into the scratch
    before the second pass writes the output."""
    lib, torch, ora = env
    st = torch.cuda.current_stream().cuda_stream
    x = signals.complex_uniform(34000 + N, N)
    d = torch.from_numpy(x).cuda()
    assert lib.gb_execute_c2c_noalloc(N, direction, d.data_ptr(), d.data_ptr(), st) == 0
    torch.cuda.synchronize()
    want = ora.c2c_many(x.reshape(1, N), direction, 1)[0]
    assert rel_l2(d.cpu().numpy(), want) <= REL_L2_TOL


def test_noalloc_rejects_sizes_beyond_the_scratch(env):
    lib, torch, _ = env
    dx = torch.zeros(2 * MAX_POINTS, dtype=torch.complex64, device="cuda")
    dy = torch.zeros_like(dx)
    assert lib.gb_execute_c2c_noalloc(2 * MAX_POINTS, K.FORWARD, dy.data_ptr(), dx.data_ptr(), None) == -2
    assert lib.gb_execute_c2c_noalloc(3000, K.FORWARD, dy.data_ptr(), dx.data_ptr(), None) == -1
    x = np.zeros(16, np.complex64)
    assert lib.gb_execute_c2c_noalloc(16, K.FORWARD, dy.data_ptr(), x.ctypes.data, None) == -4
