"""GPU tests of the ragged batched transforms (mufft_gb_create_fft_batch):
c2c / r2c / c2r requests of mixed sizes, directions and flags in one
persistent launch, each checked against the oracle's plan of the same kind
(fft.c:476-547, 626-662, 811-850)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import REL_L2_TOL, rel_l2
from mufft_gb300 import capi as K
from mufft_gb300 import signals

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    import mufft_gb300
    return mufft_gb300.load()


@pytest.fixture(scope="module")
def ora():
    from oracle.oracle import load_oracle
    return load_oracle()


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available()
    return t


def out_count(N, kind, flags):
    if kind == 0:
        return N
    if kind == 1:
        return N if flags & K.FLAG_FULL_R2C else N // 2 + 1
    return N


class Batch:
    """Device buffers and the batch handle for (N, kind, direction, flags, input) requests."""

    def __init__(self, gpu, torch, reqs, flags=0, opts=None):
        self.gpu, self.reqs = gpu, reqs
        self.din, self.dout = [], []
        creq = (K.FftRequest * len(reqs))()
        for i, (N, kind, direction, fl, x) in enumerate(reqs):
            din = torch.from_numpy(np.ascontiguousarray(x)).cuda()
            dt = torch.float32 if kind == 2 else torch.complex64
            dout = torch.full((out_count(N, kind, fl),), float("nan"), dtype=dt, device="cuda")
            creq[i] = K.FftRequest(N, kind, direction, fl, din.data_ptr(), dout.data_ptr())
            self.din.append(din)
            self.dout.append(dout)
        self.handle = gpu.gb_create_fft_batch(creq, len(reqs), flags, C.byref(opts) if opts else None)
        assert self.handle, gpu.gb_last_error_string()

    def run(self, torch):
        rc = self.gpu.gb_execute_fft_batch(self.handle, torch.cuda.current_stream().cuda_stream)
        assert rc == 0, self.gpu.gb_last_error_string()
        torch.cuda.synchronize()
        assert self.gpu.gb_fft_batch_status(self.handle) == 0, self.gpu.gb_last_error_string()
        return [d.cpu().numpy() for d in self.dout]

    def describe(self):
        buf = C.create_string_buffer(256)
        assert self.gpu.gb_fft_batch_describe(self.handle, buf, 256) == 0
        return buf.value.decode()

    def free(self):
        self.gpu.gb_free_fft_batch(self.handle)


def oracle_result(ora, N, kind, direction, flags, x):
    if kind == 0:
        return ora.fft_c2c(x, direction, flags, N)
    if kind == 1:
        return ora.fft_r2c(x, flags, N)
    return ora.fft_c2r(x, N, flags)


def check_all(ora, reqs, outs, tol=REL_L2_TOL):
    worst = 0.0
    for i, ((N, kind, direction, flags, x), got) in enumerate(zip(reqs, outs)):
        want = oracle_result(ora, N, kind, direction, flags, x)
        assert np.all(np.isfinite(got)), (i, N, kind)
        err = rel_l2(got, want)
        worst = max(worst, err)
        assert err <= tol, (i, N, kind, direction, flags, err)
    return worst


def test_fft_batch_512_request_mix(gpu, ora, torch):
    """512 requests, N = 2^4..2^16 log-uniform, c2c both directions, r2c
    (half of them FULL_R2C) and c2r, a quarter zero-padded, against the
    oracle at relative L2 <= 1e-5."""
    reqs = signals.ragged_fft_requests(6, 512)
    bt = Batch(gpu, torch, reqs)
    try:
        outs = bt.run(torch)
        again = bt.run(torch)
    finally:
        bt.free()
    worst = check_all(ora, reqs, outs)
    for x, y in zip(outs, again):  # replays give the same bits
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
    print(f"512-request transform mix: worst relative L2 against the oracle {worst:.2e}")


@pytest.mark.parametrize("split", [8192, 32768, 0])
def test_fft_batch_every_size_and_kind(gpu, ora, torch, split):
    """Every length the batch takes -- c2c 2..65536 both directions, r2c
    (both output forms) and c2r 4..131072, zero-padded c2c / r2c -- with the
    long requests as phase tasks from `split` points (0: all whole)."""
    reqs = []
    seed = 36000
    for lg in range(1, 17):
        N = 1 << lg
        for direction in (K.FORWARD, K.INVERSE):
            reqs.append((N, 0, direction, 0, signals.complex_uniform(seed, N)))
            seed += 1
        reqs.append((N, 0, K.FORWARD, K.FLAG_ZERO_PAD_UPPER_HALF, signals.complex_uniform(seed, N // 2 or 1)))
        seed += 1
    for lg in range(2, 18):
        N = 1 << lg
        reqs.append((N, 1, K.FORWARD, 0, signals.uniform(seed, N)))
        reqs.append((N, 1, K.FORWARD, K.FLAG_FULL_R2C, signals.uniform(seed + 1, N)))
        reqs.append((N, 1, K.FORWARD, K.FLAG_ZERO_PAD_UPPER_HALF, signals.uniform(seed + 2, N // 2)))
        reqs.append((N, 2, K.INVERSE, 0, signals.complex_uniform(seed + 3, N // 2 + 1)))
        seed += 4
    bt = Batch(gpu, torch, reqs, opts=gpu.options(fft_split=split))
    try:
        want_split = split if split else 0
        assert f"split={want_split} " in bt.describe(), bt.describe()
        outs = bt.run(torch)
    finally:
        bt.free()
    check_all(ora, reqs, outs)


def test_fft_batch_many_small_requests_in_groups(gpu, ora, torch):
    """Full groups and ragged last groups of several classes interleaved:
    one tile's transforms each take their own request's buffers."""
    reqs = []
    for i in range(300):
        N = (16, 256, 1024)[i % 3]
        kind = i % 4 % 3
        direction = K.INVERSE if i % 4 == 3 else K.FORWARD
        flags = K.FLAG_FULL_R2C if kind == 1 and i % 2 else 0
        x = (signals.complex_uniform(37000 + i, N) if kind == 0 else
             signals.uniform(37000 + i, N) if kind == 1 else signals.complex_uniform(37000 + i, N // 2 + 1))
        reqs.append((N, kind, direction, flags, x))
    bt = Batch(gpu, torch, reqs)
    try:
        outs = bt.run(torch)
    finally:
        bt.free()
    check_all(ora, reqs, outs)


def test_fft_batch_autotuned(gpu, ora, torch):
    """MUFFT_GB_FLAG_AUTOTUNE times split sizes and grids; whatever it keeps,
    the outputs match the oracle."""
    reqs = signals.ragged_fft_requests(7, 96, lo=10, hi=16)
    bt = Batch(gpu, torch, reqs, flags=K.FLAG_AUTOTUNE)
    try:
        outs = bt.run(torch)
    finally:
        bt.free()
    check_all(ora, reqs, outs)


def test_fft_batch_matches_plans(gpu, torch):
    """The batch computes what per-request plans compute: to rounding where
    both run the same single tile (up to 4096 complex points), within the
    parity bar where the plan runs one long tile and the batch a four-step."""
    reqs = [(1024, 0, K.FORWARD, 0, signals.complex_uniform(38000, 1024)),
            (4096, 1, K.FORWARD, K.FLAG_FULL_R2C, signals.uniform(38001, 4096)),
            (512, 2, K.INVERSE, 0, signals.complex_uniform(38002, 257)),
            (16384, 0, K.INVERSE, 0, signals.complex_uniform(38003, 16384)),
            (65536, 1, K.FORWARD, 0, signals.uniform(38004, 65536))]
    bt = Batch(gpu, torch, reqs)
    try:
        outs = bt.run(torch)
    finally:
        bt.free()
    for (N, kind, direction, flags, x), got in zip(reqs, outs):
        if kind == 0:
            want = gpu.fft_c2c(x, direction, flags, N)
        elif kind == 1:
            want = gpu.fft_r2c(x, flags, N)
        else:
            want = gpu.fft_c2r(x, N, flags)
        tol = 1e-6 if (N if kind == 0 else N // 2) <= 4096 else REL_L2_TOL
        assert rel_l2(got, want) <= tol, (N, kind, rel_l2(got, want))
