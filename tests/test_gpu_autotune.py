"""GPU tests of the schedule autotuner: tuned plans stay correct, the choice
is remembered and applied, survives a save / clear / load round trip, and
plan creation with MUFFT_GB_FLAG_AUTOTUNE tunes on first use."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import rel_l2
from mufft_gb300 import capi as K
from mufft_gb300 import signals

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import mufft_gb300
    lib = mufft_gb300.load()
    yield lib
    lib.gb_autotune_clear()


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available()
    return t


def describe(gpu, N, kind=0, flags=0, batch=1):
    buf = C.create_string_buffer(4096)
    assert gpu.gb_describe_schedule_1d(N, kind, K.FORWARD if kind != 2 else K.INVERSE, flags, batch, None, buf,
                                       4096) == 0
    return buf.value.decode()


def run_c2c(gpu, torch, N, B, flags=0):
    x = signals.complex_uniform(50000 + N + B, N * B).reshape(B, N)
    dx = torch.from_numpy(x).cuda()
    dy = torch.empty_like(dx)
    plan = gpu.gb_create_plan_1d_c2c_batched(N, K.FORWARD, flags, B, 0, 0)
    assert plan, gpu.gb_last_error_string()
    assert gpu.gb_execute_plan_1d_async(plan, dy.data_ptr(), dx.data_ptr(), torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    gpu.free_plan_1d(plan)
    return rel_l2(dy.cpu().numpy(), np.fft.fft(x.astype(np.complex128), axis=1))


@pytest.mark.parametrize("N,B", [(1 << 20, 1), (8192, 64), (1 << 17, 4)])
def test_autotune_picks_a_correct_schedule(gpu, torch, N, B):
    gpu.gb_autotune_clear()
    default = describe(gpu, N, batch=B)
    rep = C.create_string_buffer(1 << 16)
    assert gpu.gb_autotune_1d(0, N, K.FORWARD, 0, B, rep, 1 << 16) == 0, gpu.gb_last_error_string()
    lines = rep.value.decode().strip().splitlines()
    assert len(lines) >= 3 and lines[-1].startswith("best")
    best_ms = float(lines[-1].split()[1])
    times = [float(l.split()[0]) for l in lines[:-1]]
    assert best_ms <= min(times) * 1.0001 + 1e-9, (best_ms, min(times))
    tuned = describe(gpu, N, batch=B)
    assert run_c2c(gpu, torch, N, B) < 2e-6, (default, tuned)


def test_autotune_cache_round_trip(gpu, torch, tmp_path):
    gpu.gb_autotune_clear()
    N, B = 1 << 21, 1
    assert gpu.gb_autotune_1d(0, N, K.FORWARD, 0, B, None, 0) == 0
    tuned = describe(gpu, N, batch=B)
    path = str(tmp_path / "tune.txt").encode()
    assert gpu.gb_autotune_save(path) == 0
    gpu.gb_autotune_clear()
    assert gpu.gb_autotune_load(path) == 0
    assert describe(gpu, N, batch=B) == tuned
    # a file from another GPU is refused
    text = open(path.decode()).read().splitlines()
    text[1] = "device 7 Some_Other_GPU"
    other = tmp_path / "other.txt"
    other.write_text("\n".join(text) + "\n")
    assert gpu.gb_autotune_load(str(other).encode()) == -1
    gpu.gb_clear_error()


def test_autotune_flag_tunes_on_first_plan(gpu, torch):
    gpu.gb_autotune_clear()
    N, B = 4096, 257
    assert run_c2c(gpu, torch, N, B, flags=K.FLAG_AUTOTUNE) < 2e-6
    # the shape is now remembered: a plain plan of it uses the tuned schedule
    assert run_c2c(gpu, torch, N, B) < 2e-6


@pytest.mark.parametrize("kind,N", [(1, 1 << 20), (2, 1 << 16)])
def test_autotune_real_transforms(gpu, torch, kind, N):
    gpu.gb_autotune_clear()
    assert gpu.gb_autotune_1d(kind, N, K.FORWARD if kind == 1 else K.INVERSE, 0, 1, None, 0) == 0
    x = signals.uniform(51000 + N, N)
    if kind == 1:
        got = gpu.fft_r2c(x)
        ref = np.fft.rfft(x.astype(np.float64))
    else:
        X = np.fft.rfft(x.astype(np.float64)).astype(np.complex64)
        got = gpu.fft_c2r(X, N)
        ref = np.fft.irfft(X.astype(np.complex128), N) * N
    assert rel_l2(got, ref) < 2e-6
