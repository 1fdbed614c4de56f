"""GPU tests of the ragged batched convolution (mufft_gb_create_conv_batch):
requests of mixed sizes and methods in one persistent launch, each checked
against the oracle's full convolution sequence (fft.c:794-809) and against
the single-request plan path."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import REL_L2_TOL, direct_conv_f64, rel_l2
from mufft_gb300 import capi as K
from mufft_gb300 import signals

pytestmark = pytest.mark.gpu

STEREO = K.CONV_METHOD_FLAG_STEREO_MONO
PAD1 = K.CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_FIRST
PAD2 = K.CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_SECOND


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


def filter_spectrum(gpu, b: np.ndarray, N: int, method: int) -> np.ndarray:
    """Second block transformed by mufft_execute_conv_input(SECOND)."""
    plan = gpu.create_plan_conv(N, 0, method)
    assert plan, gpu.gb_last_error_string()
    try:
        nblk = gpu.conv_get_transformed_block_size(plan) // 8
        out = K.aligned_zeros(nblk, np.complex64)
        src = K.aligned_copy(b, np.float32)
        gpu.execute_conv_input(plan, K.CONV_BLOCK_SECOND, out.ctypes.data, src.ctypes.data)
        gpu.check("conv_input")
    finally:
        gpu.free_plan_conv(plan)
    return out


class Batch:
    """Device buffers and the batch handle for a list of (N, method) requests."""

    def __init__(self, gpu, torch, specs, seed, flags=0, opts=None):
        self.gpu, self.specs = gpu, specs
        self.a, self.b, self.din, self.dh, self.dout = [], [], [], [], []
        reqs = (K.ConvRequest * len(specs))()
        for i, (N, method) in enumerate(specs):
            stereo = (method & 1) == STEREO
            a = (signals.complex_uniform(seed + 2 * i, N) if stereo else signals.uniform(seed + 2 * i, N))
            b = signals.uniform(seed + 2 * i + 1, N)
            H = filter_spectrum(gpu, b, N, method)
            din = torch.from_numpy(np.ascontiguousarray(a)).cuda()
            dh = torch.from_numpy(H).cuda()
            dout = torch.full((N,), float("nan"), dtype=torch.complex64 if stereo else torch.float32, device="cuda")
            reqs[i] = K.ConvRequest(N, method, din.data_ptr(), dh.data_ptr(), dout.data_ptr())
            self.a.append(a), self.b.append(b), self.din.append(din), self.dh.append(dh), self.dout.append(dout)
        self.handle = gpu.gb_create_conv_batch(reqs, len(specs), flags, C.byref(opts) if opts else None)
        assert self.handle, gpu.gb_last_error_string()

    def run(self, torch):
        rc = self.gpu.gb_execute_conv_batch(self.handle, torch.cuda.current_stream().cuda_stream)
        assert rc == 0, self.gpu.gb_last_error_string()
        torch.cuda.synchronize()
        assert self.gpu.gb_conv_batch_status(self.handle) == 0, self.gpu.gb_last_error_string()
        return [d.cpu().numpy() for d in self.dout]

    def free(self):
        self.gpu.gb_free_conv_batch(self.handle)


def _mixed_specs(rng_seed: int, count: int):
    rng = np.random.default_rng(rng_seed)
    specs = []
    for _ in range(count):
        method = int(rng.choice([0, STEREO, PAD1, STEREO | PAD1, PAD2, STEREO | PAD1 | PAD2]))
        stereo = method & 1
        lg = int(rng.integers(4, 17)) + (0 if stereo else 1)  # complex length 2^4 .. 2^16
        specs.append((1 << lg, method))
    return specs


def test_conv_batch_mixed_sizes_vs_oracle(gpu, ora, torch):
    specs = _mixed_specs(7, 48)
    # every kernel branch at least once: complex lengths 16 .. 65536, mono and stereo
    specs += [(1 << (lg + 1), 0) for lg in range(4, 17)] + [(1 << lg, STEREO) for lg in range(4, 17)]
    bt = Batch(gpu, torch, specs, 90000)
    try:
        outs = bt.run(torch)
    finally:
        bt.free()
    for i, ((N, method), got) in enumerate(zip(specs, outs)):
        want = ora.conv(bt.a[i], bt.b[i], N, method)
        assert np.all(np.isfinite(got)), (i, N, method)
        assert rel_l2(got, want) <= REL_L2_TOL, (i, N, method, rel_l2(got, want))


@pytest.mark.parametrize("method", [0, STEREO, PAD1 | PAD2, STEREO | PAD1 | PAD2])
def test_conv_batch_vs_direct_fp64(gpu, torch, method):
    """Zero-padded blocks make the circular convolution a linear one; check
    against the FP64 direct sum."""
    specs = [(N, method) for N in (64, 1024, 8192, 32768, 131072 if not method & 1 else 65536)]
    bt = Batch(gpu, torch, specs, 91000 + method)
    try:
        outs = bt.run(torch)
    finally:
        bt.free()
    for i, (N, m) in enumerate(specs):
        a = bt.a[i].copy()
        b = bt.b[i].copy()
        if m & PAD1:
            a[N // 2:] = 0
        if m & PAD2:
            b[N // 2:] = 0
        ref = direct_conv_f64(a, b, N) if N <= 8192 else np.fft.ifft(
            np.fft.fft(a.astype(np.complex128)) * np.fft.fft(b.astype(np.float64)))
        if not m & 1:
            ref = np.real(ref)
        assert rel_l2(outs[i], ref) < 2e-6, (N, m)


def test_conv_batch_matches_single_plans(gpu, torch):
    """The batch computes what the per-request plan path computes."""
    specs = [(4096, 0), (65536, STEREO), (256, PAD1), (131072, PAD1 | PAD2)]
    bt = Batch(gpu, torch, specs, 92000)
    try:
        outs = bt.run(torch)
    finally:
        bt.free()
    for i, (N, m) in enumerate(specs):
        single = gpu.conv(bt.a[i], bt.b[i], N, m)
        assert rel_l2(outs[i], single) < 1e-6, (N, m)


def test_conv_batch_replay_is_deterministic(gpu, torch):
    specs = _mixed_specs(11, 300)
    bt = Batch(gpu, torch, specs, 93000)
    try:
        first = bt.run(torch)
        for d in bt.dout:
            d.fill_(float("nan"))
        second = bt.run(torch)
    finally:
        bt.free()
    for x, y in zip(first, second):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_conv_batch_rejects_bad_requests(gpu, torch):
    d = torch.zeros(1 << 18, dtype=torch.float32, device="cuda")
    p = d.data_ptr()
    for N, method, ptrs in [(1000, 0, (p, p, p)), (1 << 18, 0, (p, p, p)), (16, 0, (p, p, p)),
                            (1 << 17, STEREO, (p, p, p)), (1024, 0, (p, None, p))]:
        reqs = (K.ConvRequest * 1)(K.ConvRequest(N, method, *ptrs))
        assert not gpu.gb_create_conv_batch(reqs, 1, 0, None)
        assert gpu.gb_last_error() in (-1, -2), (N, method)
        gpu.gb_clear_error()
    assert not gpu.gb_create_conv_batch(None, 0, 0, None)
    gpu.gb_clear_error()


def test_conv_batch_autotuned_split_size(gpu, ora, torch):
    """MUFFT_GB_FLAG_AUTOTUNE times every split size; whatever it keeps, the
    outputs match the oracle (split and whole paths of every large size)."""
    specs = [(1 << 17, 0), (1 << 16, STEREO), (1 << 15, PAD1), (1 << 15, STEREO | PAD1), (1 << 16, 0),
             (1 << 14, STEREO)] + _mixed_specs(13, 40)
    bt = Batch(gpu, torch, specs, 94000, flags=K.FLAG_AUTOTUNE)
    try:
        split = gpu.gb_conv_batch_split_size(bt.handle)
        assert split in (0, 1 << 14, 1 << 15, 1 << 16)
        assert gpu.gb_conv_batch_class_size(bt.handle) in (0, 1 << 14, 1 << 15, 1 << 16)
        outs = bt.run(torch)
    finally:
        bt.free()
    for i, ((N, method), got) in enumerate(zip(specs, outs)):
        want = ora.conv(bt.a[i], bt.b[i], N, method)
        assert rel_l2(got, want) <= REL_L2_TOL, (i, N, method, split)


@pytest.mark.parametrize("split", [0, 1 << 14, 1 << 15])
def test_conv_batch_forced_split_sizes(gpu, ora, torch, split):
    """Every split size gives the oracle's outputs (phase tasks with their
    bounded dependency waits, or whole requests)."""
    specs = [(1 << 17, 0), (1 << 16, STEREO), (1 << 15, PAD1), (1 << 15, STEREO | PAD1), (1 << 16, PAD1 | PAD2),
             (1 << 14, STEREO), (2048, 0), (64, STEREO)]
    bt = Batch(gpu, torch, specs, 95000 + split, opts=gpu.options(conv_split=split, conv_classes=0))
    try:
        assert gpu.gb_conv_batch_split_size(bt.handle) == split
        outs = bt.run(torch)
    finally:
        bt.free()
    for i, ((N, method), got) in enumerate(zip(specs, outs)):
        assert rel_l2(got, ora.conv(bt.a[i], bt.b[i], N, method)) <= REL_L2_TOL, (i, N, method, split)


@pytest.mark.parametrize("classes", [1 << 14, 1 << 15, 1 << 16])
def test_conv_batch_class_pipelines(gpu, ora, torch, classes):
    """Large requests as class pipelines (batched launches per size class on
    parallel graph branches) beside the persistent kernel."""
    specs = [(1 << 17, 0), (1 << 16, STEREO), (1 << 15, PAD1), (1 << 15, STEREO | PAD1), (1 << 16, PAD1 | PAD2),
             (1 << 14, STEREO), (1 << 17, PAD1), (1 << 16, STEREO), (2048, 0), (64, STEREO)]
    bt = Batch(gpu, torch, specs, 96000 + classes, opts=gpu.options(conv_classes=classes))
    try:
        assert gpu.gb_conv_batch_class_size(bt.handle) == classes
        outs = bt.run(torch)
        again = bt.run(torch)
    finally:
        bt.free()
    for i, ((N, method), got) in enumerate(zip(specs, outs)):
        assert rel_l2(got, ora.conv(bt.a[i], bt.b[i], N, method)) <= REL_L2_TOL, (i, N, method, classes)
        assert np.array_equal(got.view(np.uint32), again[i].view(np.uint32))


def test_conv_batch_groups_of_small_requests(gpu, ora, torch):
    """Many requests of one class run in groups (one tile transform per
    request, buffers from tables): full groups and a ragged last group, two
    classes interleaved, against the oracle."""
    specs = []
    for i in range(150):
        specs.append((256, 0 if i % 3 else PAD1))           # mono, two zero-pad classes
        specs.append((512, STEREO if i % 2 else STEREO | PAD1))
    specs += [(32, 0), (16, STEREO), (8192, 0), (4096, STEREO)]
    bt = Batch(gpu, torch, specs, 97000)
    try:
        outs = bt.run(torch)
        again = bt.run(torch)
    finally:
        bt.free()
    for i, ((N, method), got) in enumerate(zip(specs, outs)):
        assert rel_l2(got, ora.conv(bt.a[i], bt.b[i], N, method)) <= REL_L2_TOL, (i, N, method)
        assert np.array_equal(got.view(np.uint32), again[i].view(np.uint32))


def test_conv_batch_ragged_512_request_mix(gpu, ora, torch):
    """The ragged-convolution workload itself: 512 requests, N = 2^8..2^16
    log-uniform, 256 STEREO_MONO, N/2-sample inputs and N/2-tap decaying
    filters with both zero-pad flags (signals.ragged_conv_requests, seed 4),
    as one batch; every output against the oracle's full convolution
    sequence (fft.c:794-809) at relative L2 <= 1e-5."""
    reqs = signals.ragged_conv_requests(4, 512)
    creq = (K.ConvRequest * len(reqs))()
    keep, outs, full = [], [], []
    for i, (N, stereo, x, h) in enumerate(reqs):
        m = PAD1 | PAD2 | (STEREO if stereo else 0)
        hp = np.zeros(N, np.float32)
        hp[: N // 2] = h
        xp = np.zeros(N, np.complex64 if stereo else np.float32)
        xp[: N // 2] = x
        H = filter_spectrum(gpu, hp, N, m)
        din = torch.from_numpy(np.ascontiguousarray(x)).cuda()   # N/2 samples: the upper half is never read
        dh = torch.from_numpy(H).cuda()
        dout = torch.full((N,), float("nan"), dtype=torch.complex64 if stereo else torch.float32, device="cuda")
        creq[i] = K.ConvRequest(N, m, din.data_ptr(), dh.data_ptr(), dout.data_ptr())
        keep += [din, dh]
        outs.append(dout)
        full.append((N, m, xp, hp))
    batch = gpu.gb_create_conv_batch(creq, len(reqs), 0, None)
    assert batch, gpu.gb_last_error_string()
    try:
        assert gpu.gb_execute_conv_batch(batch, torch.cuda.current_stream().cuda_stream) == 0
        torch.cuda.synchronize()
        assert gpu.gb_conv_batch_status(batch) == 0, gpu.gb_last_error_string()
    finally:
        gpu.gb_free_conv_batch(batch)
    worst = 0.0
    for i, ((N, m, xp, hp), dout) in enumerate(zip(full, outs)):
        got = dout.cpu().numpy()
        want = ora.conv(xp, hp, N, m)
        assert np.all(np.isfinite(got)), (i, N, m)
        err = rel_l2(got, want)
        worst = max(worst, err)
        assert err <= REL_L2_TOL, (i, N, m, err)
    print(f"512-request mix: worst relative L2 against the oracle {worst:.2e}")
