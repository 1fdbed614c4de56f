"""GPU tests of the streaming partitioned convolution
(mufft_gb_create_stream_conv): a stream of blocks convolved with filters
shorter and much longer than a block, against the FP64 linear convolution of
the whole stream."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import rel_l2
from mufft_gb300 import capi as K
from mufft_gb300 import signals

pytestmark = pytest.mark.gpu
STEREO = K.CONV_METHOD_FLAG_STEREO_MONO


@pytest.fixture(scope="module")
def gpu():
    import mufft_gb300
    return mufft_gb300.load()


def linear_conv_f64(x, h):
    n = len(x) + len(h) - 1
    L = 1 << (n - 1).bit_length()
    return np.fft.ifft(np.fft.fft(x.astype(np.complex128), L) * np.fft.fft(h.astype(np.float64), L))[: len(x)]


def stream(gpu, block, method, h, x, restart_at=None, fused=1, ranges=0):
    stereo = method & 1
    opts = gpu.options(stream_conv_fused=fused, stream_conv_ranges=ranges)
    conv = gpu.gb_create_stream_conv(block, method, h.ctypes.data, len(h), 0, C.byref(opts))
    assert conv, gpu.gb_last_error_string()
    # one fused launch per block exactly when a 256-thread row tile holds the window
    M = 2 * block if stereo else block
    assert gpu.gb_stream_conv_fused(conv) == (1 if fused and 64 <= M <= 4096 else 0)
    P = (len(h) + block - 1) // block
    if ranges:
        most = max(1, P - 1) if gpu.gb_stream_conv_fused(conv) else P
        used = gpu.gb_stream_conv_ranges(conv)
        # fused launches keep every CTA resident: large requests are capped
        assert used == min(ranges, most) if ranges <= 7 else 1 <= used <= min(ranges, most), (used, ranges, P)
    sample = 8 if stereo else 4
    out = np.zeros(len(x), np.complex64 if stereo else np.float32)
    try:
        inp, outp = gpu.gb_stream_conv_input(conv), gpu.gb_stream_conv_output(conv)
        for k in range(len(x) // block):
            if restart_at is not None and k == restart_at:
                assert gpu.gb_stream_conv_reset(conv, None) == 0
            blk = np.ascontiguousarray(x[k * block:(k + 1) * block])
            assert gpu.gb_memcpy(inp, blk.ctypes.data, block * sample) == 0
            assert gpu.gb_stream_conv_process(conv, None) == 0, gpu.gb_last_error_string()
            assert gpu.gb_memcpy(out[k * block:].ctypes.data, outp, block * sample) == 0
        assert gpu.gb_stream_conv_status(conv) == 0, gpu.gb_last_error_string()
    finally:
        gpu.gb_free_stream_conv(conv)
    return out


@pytest.mark.parametrize("block", [8, 64, 1024])
@pytest.mark.parametrize("taps_of", [lambda b: 1, lambda b: 100, lambda b: b, lambda b: 3 * b + 5, lambda b: 40 * b])
@pytest.mark.parametrize("method", [0, STEREO])
@pytest.mark.parametrize("fused", [1, 0])
def test_stream_conv_matches_linear_convolution(gpu, block, taps_of, method, fused):
    """One fused launch per block (forward row tile, multiply-accumulate and
    inverse in one grid) and the graph of separate launches."""
    taps = taps_of(block)
    blocks = 12
    h = (signals.normal(60000 + taps, taps) * np.exp(-np.arange(taps) / max(1.0, taps / 4))).astype(np.float32)
    n = blocks * block
    x = signals.complex_uniform(61000 + block, n) if method & 1 else signals.uniform(61000 + block, n)
    got = stream(gpu, block, method, h, x, fused=fused)
    ref = linear_conv_f64(x, h)
    if not method & 1:
        ref = ref.real
    assert rel_l2(got, ref) < 1e-5, (block, taps, method)


@pytest.mark.parametrize("ranges", [1, 2, 7, 1000])
@pytest.mark.parametrize("method", [0, STEREO])
def test_stream_conv_partition_ranges(gpu, ranges, method):
    """Any split of the partitions over CTA rows (tickets finish each bin
    group in range order) gives the linear convolution."""
    block, taps = 512, 512 * 37 + 3
    h = (signals.normal(64000, taps) * np.exp(-np.arange(taps) / (taps / 4))).astype(np.float32)
    x = signals.complex_uniform(64001, 10 * block) if method & 1 else signals.uniform(64001, 10 * block)
    ref = linear_conv_f64(x, h)
    if not method & 1:
        ref = ref.real
    for fused in (1, 0):
        got = stream(gpu, block, method, h, x, fused=fused, ranges=ranges)
        assert rel_l2(got, ref) < 1e-5, (ranges, method, fused)


def test_stream_conv_long_filter(gpu):
    """2^20 taps in 256 partitions of 4096."""
    block, taps = 4096, 1 << 20
    h = (signals.normal(62000, taps) * np.exp(-np.arange(taps) / (taps / 8))).astype(np.float32)
    x = signals.uniform(62001, 8 * block)
    got = stream(gpu, block, 0, h, x)
    assert rel_l2(got, linear_conv_f64(x, h).real) < 1e-5


def test_stream_conv_reset_restarts_history(gpu):
    block, taps = 256, 1000
    h = signals.normal(63000, taps).astype(np.float32)
    x = signals.uniform(63001, 6 * block)
    xx = np.concatenate([x, x])
    got = stream(gpu, block, 0, h, xx, restart_at=6)
    assert np.array_equal(got[: 6 * block].view(np.uint32), got[6 * block:].view(np.uint32))


def test_stream_conv_rejects_bad_arguments(gpu):
    h = np.ones(10, np.float32)
    for block, taps in ((1000, 10), (1, 10), (256, 0)):
        assert not gpu.gb_create_stream_conv(block, 0, h.ctypes.data, taps, 0, None)
        assert gpu.gb_last_error() == -1
        gpu.gb_clear_error()


@pytest.mark.parametrize("method", [0, STEREO])
def test_stream_conv_timeout_then_reset(gpu, method):
    """A block whose bounded wait runs out (injected: the awaited flag is
    never published) is reported by the status call; the launches stay
    consistent, so after a reset the stream convolves correctly again --
    every later block, not only the first."""
    block, taps = 512, 512 * 9 + 17
    stereo = method & 1
    sample = 8 if stereo else 4
    h = (signals.normal(65000, taps) * np.exp(-np.arange(taps) / (taps / 4))).astype(np.float32)
    x = signals.complex_uniform(65001, 14 * block) if stereo else signals.uniform(65001, 14 * block)
    conv = gpu.gb_create_stream_conv(block, method, h.ctypes.data, taps, 0, None)
    assert conv, gpu.gb_last_error_string()
    try:
        assert gpu.gb_stream_conv_fused(conv) == 1
        inp, outp = gpu.gb_stream_conv_input(conv), gpu.gb_stream_conv_output(conv)

        def push(blk):
            blk = np.ascontiguousarray(blk)
            assert gpu.gb_memcpy(inp, blk.ctypes.data, block * sample) == 0
            assert gpu.gb_stream_conv_process(conv, None) == 0, gpu.gb_last_error_string()
            out = np.zeros(block, np.complex64 if stereo else np.float32)
            assert gpu.gb_memcpy(out.ctypes.data, outp, block * sample) == 0
            return out

        for k in range(3):
            push(x[k * block:(k + 1) * block])
        assert gpu.gb_stream_conv_status(conv) == 0
        assert gpu.gb_stream_conv_inject_timeout(conv, 1) == 0
        push(x[3 * block:4 * block])
        assert gpu.gb_stream_conv_status(conv) == -2  # the timeout is reported ...
        assert gpu.gb_stream_conv_status(conv) == 0   # ... once
        gpu.gb_clear_error()
        assert gpu.gb_stream_conv_inject_timeout(conv, 0) == 0
        assert gpu.gb_stream_conv_reset(conv, None) == 0
        rest = x[4 * block:]
        got = np.concatenate([push(rest[k * block:(k + 1) * block]) for k in range(len(rest) // block)])
        assert gpu.gb_stream_conv_status(conv) == 0, gpu.gb_last_error_string()
    finally:
        gpu.gb_free_stream_conv(conv)
    ref = linear_conv_f64(rest, h)
    if not stereo:
        ref = ref.real
    assert rel_l2(got, ref) < 1e-5
