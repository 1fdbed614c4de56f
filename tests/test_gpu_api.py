"""GPU tests of the extension API (mufft_gb300.h) and the memory contract:
batched plans, stream execution on device buffers, error reporting, and the
reference's alloc / convolve-func entry points."""
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


def _dev(torch, arr):
    return torch.from_numpy(np.ascontiguousarray(arr)).cuda()


def _stream(torch):
    return torch.cuda.current_stream().cuda_stream


@pytest.mark.parametrize("N,B", [(1024, 4096), (4096, 257), (16, 1000), (2, 3), (16384, 17), (1 << 20, 3)])
@pytest.mark.parametrize("direction", [K.FORWARD, K.INVERSE])
def test_batched_c2c_device(gpu, ora, torch, N, B, direction):
    x = signals.complex_uniform(20000 + N + B, N * B).reshape(B, N)
    dx = _dev(torch, x)
    dy = torch.empty_like(dx)
    plan = gpu.gb_create_plan_1d_c2c_batched(N, direction, 0, B, 0, 0)
    assert plan, gpu.gb_last_error_string()
    try:
        rc = gpu.gb_execute_plan_1d_async(plan, dy.data_ptr(), dx.data_ptr(), _stream(torch))
        assert rc == 0, gpu.gb_last_error_string()
        torch.cuda.synchronize()
    finally:
        gpu.free_plan_1d(plan)
    got = dy.cpu().numpy()
    rows = range(B) if B <= 8 else (0, 1, B // 2, B - 1)
    want = ora.c2c_many(x[list(rows)], direction, 4)
    for i, r in enumerate(rows):
        assert rel_l2(got[r], want[i]) <= REL_L2_TOL, r


def test_batched_strided_r2c_c2r(gpu, ora, torch):
    N, B = 2048, 64
    idist, odist = N + 64, N // 2 + 1 + 7   # padded layouts
    x = np.zeros((B, idist), np.float32)
    x[:, :N] = signals.uniform(21000, N * B).reshape(B, N)
    dx = _dev(torch, x)
    dX = torch.zeros((B, odist), dtype=torch.complex64, device="cuda")
    plan = gpu.gb_create_plan_1d_r2c_batched(N, 0, B, idist, odist)
    assert plan
    assert gpu.gb_execute_plan_1d_async(plan, dX.data_ptr(), dx.data_ptr(), _stream(torch)) == 0
    torch.cuda.synchronize()
    gpu.free_plan_1d(plan)
    X = dX.cpu().numpy()
    for r in (0, 31, 63):
        assert rel_l2(X[r, : N // 2 + 1], ora.fft_r2c(x[r, :N])) <= REL_L2_TOL
    # and back: c2r of the padded spectra into padded real rows
    dy = torch.zeros((B, idist), dtype=torch.float32, device="cuda")
    plan = gpu.gb_create_plan_1d_c2r_batched(N, 0, B, odist, idist)
    assert plan
    assert gpu.gb_execute_plan_1d_async(plan, dy.data_ptr(), dX.data_ptr(), _stream(torch)) == 0
    torch.cuda.synchronize()
    gpu.free_plan_1d(plan)
    y = dy.cpu().numpy()
    assert rel_l2(y[:, :N] / N, x[:, :N]) < 1e-6
    assert np.all(y[:, N:] == 0)  # padding untouched


def test_sync_api_accepts_device_pointers(gpu, ora, torch):
    N = 4096
    x = signals.complex_uniform(22000, N)
    dx = _dev(torch, x)
    dy = torch.empty_like(dx)
    plan = gpu.create_plan_1d_c2c(N, K.FORWARD, 0)
    gpu.execute_plan_1d(plan, dy.data_ptr(), dx.data_ptr())
    gpu.check("execute")
    gpu.free_plan_1d(plan)
    assert rel_l2(dy.cpu().numpy(), ora.fft_c2c(x, K.FORWARD)) <= REL_L2_TOL


def test_async_rejects_host_pointers(gpu):
    N = 256
    x = np.zeros(N, np.complex64)
    y = np.zeros(N, np.complex64)
    plan = gpu.create_plan_1d_c2c(N, K.FORWARD, 0)
    rc = gpu.gb_execute_plan_1d_async(plan, y.ctypes.data, x.ctypes.data, None)
    assert rc == -4  # MUFFT_GB_ERR_HOST_POINTER
    gpu.gb_clear_error()
    gpu.free_plan_1d(plan)


def test_alloc_contract(gpu):
    p = gpu.alloc(1000)
    assert p and p % 64 == 0
    q = gpu.calloc(4096)
    assert q and q % 64 == 0
    assert bytes((C.c_char * 4096).from_address(q)) == b"\0" * 4096
    # mufft_alloc memory works as transform input/output (pinned host memory)
    N = 512
    src = (C.c_float * (2 * N)).from_address(p if 1000 >= 8 * N else q)
    gpu.free(p)
    gpu.free(q)


def test_pinned_buffers_round_trip(gpu, ora):
    N = 8192
    nbytes = N * 8
    pin_in, pin_out = gpu.alloc(nbytes), gpu.alloc(nbytes)
    x = signals.complex_uniform(23000, N)
    C.memmove(pin_in, x.ctypes.data, nbytes)
    plan = gpu.create_plan_1d_c2c(N, K.FORWARD, 0)
    gpu.execute_plan_1d(plan, pin_out, pin_in)
    gpu.check("execute")
    gpu.free_plan_1d(plan)
    y = np.empty(N, np.complex64)
    C.memmove(y.ctypes.data, pin_out, nbytes)
    gpu.free(pin_in)
    gpu.free(pin_out)
    assert rel_l2(y, ora.fft_c2c(x, K.FORWARD)) <= REL_L2_TOL


def test_convolve_func(gpu, ora):
    n = 1000
    a = signals.complex_uniform(24000, n)
    b = signals.complex_uniform(24001, n)
    f = K.CONVOLVE_FUNC(gpu.get_convolve_func(0))
    out = np.zeros(n, np.complex64)
    f(out.ctypes.data, a.ctypes.data, b.ctypes.data, 0.25, n)
    want = np.zeros(n, np.complex64)
    ora.lib.oracle_convolve(want.ctypes.data, a.ctypes.data, b.ctypes.data, 0.25, n)
    assert rel_l2(out, want) < 1e-6


def test_plan_introspection(gpu):
    plan = gpu.create_plan_1d_c2c(1 << 24, K.FORWARD, 0)
    assert gpu.gb_plan_1d_launches(plan) in (2, 3)
    buf = C.create_string_buffer(2048)
    assert gpu.gb_plan_1d_describe(plan, buf, 2048) == 0
    assert b"twiddle" in buf.value
    gpu.free_plan_1d(plan)


@pytest.mark.parametrize("levels,fused,table", [(2, 1, -1), (2, 0, 1), (3, 0, 0), (3, 0, 1), (3, 0, 2), (3, 1, 0), (3, 1, 1)])
@pytest.mark.parametrize("N,B", [(1 << 17, 2), (1 << 20, 3), (1 << 22, 1)])
def test_multipass_variants(gpu, torch, levels, fused, table, N, B):
    """Every multi-pass schedule (four-step, three-level, fused last passes
    with the L2-resident ring, table or sincospif twiddles) against FP64."""
    x = signals.complex_uniform(25000 + N + B, N * B).reshape(B, N)
    dx = _dev(torch, x)
    dy = torch.empty_like(dx)
    opts = gpu.options(multipass_levels=levels, fused_passes=fused, twiddle_table=table)
    for direction in (K.FORWARD, K.INVERSE):
        plan = gpu.gb_create_plan_1d(0, N, direction, 0, B, 0, 0, C.byref(opts))
        assert plan, gpu.gb_last_error_string()
        assert gpu.gb_execute_plan_1d_async(plan, dy.data_ptr(), dx.data_ptr(), _stream(torch)) == 0
        torch.cuda.synchronize()
        gpu.free_plan_1d(plan)
        got = dy.cpu().numpy()
        for r in range(B):
            ref = np.fft.fft(x[r].astype(np.complex128))
            if direction == K.INVERSE:
                ref = np.fft.ifft(x[r].astype(np.complex128)) * N
            assert rel_l2(got[r], ref) < 2e-6, (r, direction)


@pytest.mark.parametrize("mode", [1, 2])
@pytest.mark.parametrize("N,B", [(1 << 17, 3), (1 << 22, 1), (1 << 24, 1)])
def test_tma_staged_column_passes(gpu, torch, mode, N, B):
    """Column tiles staged by TMA tensor copies (double- and single-buffered
    persistent CTAs) against FP64, both directions."""
    x = signals.complex_uniform(26000 + N + B, N * B).reshape(B, N)
    dx = _dev(torch, x)
    dy = torch.empty_like(dx)
    opts = gpu.options(tma=mode)
    for direction in (K.FORWARD, K.INVERSE):
        plan = gpu.gb_create_plan_1d(0, N, direction, 0, B, 0, 0, C.byref(opts))
        assert plan, gpu.gb_last_error_string()
        buf = C.create_string_buffer(4096)
        gpu.gb_plan_1d_describe(plan, buf, 4096)
        assert b"+tma" in buf.value, buf.value
        assert gpu.gb_execute_plan_1d_async(plan, dy.data_ptr(), dx.data_ptr(), _stream(torch)) == 0
        torch.cuda.synchronize()
        gpu.free_plan_1d(plan)
        got = dy.cpu().numpy()
        for r in range(B):
            ref = np.fft.fft(x[r].astype(np.complex128))
            if direction == K.INVERSE:
                ref = np.fft.ifft(x[r].astype(np.complex128)) * N
            assert rel_l2(got[r], ref) < 2e-6, (r, direction)


@pytest.mark.parametrize("N,B", [(256, 1000), (1024, 4096), (2048, 333), (4096, 77)])
def test_streamed_row_tiles(gpu, torch, N, B):
    """Persistent streaming row tiles (next tile's loads in flight) against
    FP64: c2c both directions, r2c and c2r, ragged last tile."""
    x = signals.complex_uniform(27000 + N + B, N * B).reshape(B, N)
    xr = signals.uniform(27500 + N + B, N * B).reshape(B, N)
    st = _stream(torch)
    opts = gpu.options(stream_tiles=1)
    dx = _dev(torch, x)
    dy = torch.empty_like(dx)
    for direction in (K.FORWARD, K.INVERSE):
        plan = gpu.gb_create_plan_1d(0, N, direction, 0, B, 0, 0, C.byref(opts))
        assert plan, gpu.gb_last_error_string()
        buf = C.create_string_buffer(4096)
        gpu.gb_plan_1d_describe(plan, buf, 4096)
        assert b"+stream" in buf.value, buf.value
        assert gpu.gb_execute_plan_1d_async(plan, dy.data_ptr(), dx.data_ptr(), st) == 0
        torch.cuda.synchronize()
        gpu.free_plan_1d(plan)
        got = dy.cpu().numpy()
        ref = np.fft.fft(x.astype(np.complex128), axis=1) if direction == K.FORWARD else \
            np.fft.ifft(x.astype(np.complex128), axis=1) * N
        assert rel_l2(got, ref) < 2e-6, direction
    M = N // 2 + 1
    dxr = _dev(torch, xr)
    dX = torch.empty(B * M, dtype=torch.complex64, device="cuda")
    dyr = torch.empty(B * N, dtype=torch.float32, device="cuda")
    pf = gpu.gb_create_plan_1d(1, N, K.FORWARD, 0, B, 0, 0, C.byref(opts))
    pb = gpu.gb_create_plan_1d(2, N, K.INVERSE, 0, B, 0, 0, C.byref(opts))
    assert pf and pb, gpu.gb_last_error_string()
    assert gpu.gb_execute_plan_1d_async(pf, dX.data_ptr(), dxr.data_ptr(), st) == 0
    assert gpu.gb_execute_plan_1d_async(pb, dyr.data_ptr(), dX.data_ptr(), st) == 0
    torch.cuda.synchronize()
    gpu.free_plan_1d(pf)
    gpu.free_plan_1d(pb)
    ref = np.fft.rfft(xr.astype(np.float64), axis=1)
    assert rel_l2(dX.cpu().numpy().reshape(B, M), ref) < 2e-6
    assert rel_l2(dyr.cpu().numpy().reshape(B, N) / N, xr) < 2e-6


@pytest.mark.parametrize("occ", [1, 3, 8])
def test_tile_occupancy_cap(gpu, torch, occ):
    """Capped resident CTAs per SM (padded shared memory) change nothing in
    the results: a batched single pass, a multi-pass transform and a 2D r2c."""
    st = _stream(torch)
    opts = gpu.options(tile_occupancy=occ)
    for N, B in [(1024, 512), (1 << 20, 1)]:
        x = signals.complex_uniform(28000 + N + occ, N * B).reshape(B, N)
        dx = _dev(torch, x)
        dy = torch.empty_like(dx)
        plan = gpu.gb_create_plan_1d(0, N, K.FORWARD, 0, B, 0, 0, C.byref(opts))
        assert plan, gpu.gb_last_error_string()
        assert gpu.gb_execute_plan_1d_async(plan, dy.data_ptr(), dx.data_ptr(), st) == 0
        torch.cuda.synchronize()
        gpu.free_plan_1d(plan)
        assert rel_l2(dy.cpu().numpy(), np.fft.fft(x.astype(np.complex128), axis=1)) < 2e-6, (N, B)
    Nx, Ny = 512, 256
    xr = signals.uniform(28100 + occ, Nx * Ny).reshape(Ny, Nx)
    plan = gpu.gb_create_plan_2d(1, Nx, Ny, K.FORWARD, 0, C.byref(opts))
    assert plan, gpu.gb_last_error_string()
    dxr = _dev(torch, xr)
    dX = torch.empty(Ny * Nx, dtype=torch.complex64, device="cuda")
    assert gpu.gb_execute_plan_2d_async(plan, dX.data_ptr(), dxr.data_ptr(), st) == 0
    torch.cuda.synchronize()
    gpu.free_plan_2d(plan)
    got = dX.cpu().numpy().reshape(Ny, Nx)[:, : Nx // 2 + 1]
    assert rel_l2(got, np.fft.rfft2(xr.astype(np.float64))) < 2e-6
    bad = gpu.options(tile_occupancy=-1)
    assert not gpu.gb_create_plan_1d(0, 1024, K.FORWARD, 0, 1, 0, 0, C.byref(bad))
    assert gpu.gb_last_error() == -1
    gpu.gb_clear_error()


@pytest.mark.parametrize("kind,N,B", [(0, 1 << 20, 1), (0, 1024, 64), (1, 1 << 16, 3), (2, 4096, 5)])
@pytest.mark.parametrize("count", [1, 2, 5])
def test_host_pipeline_matches_sync_execute(gpu, kind, N, B, count):
    """mufft_gb_execute_plan_1d_host_pipeline on page-locked and pageable host
    buffers gives, bit for bit, what mufft_execute_plan_1d gives per buffer."""
    plan = gpu.gb_create_plan_1d(kind, N, K.FORWARD if kind != 2 else K.INVERSE, 0, B, 0, 0, None)
    assert plan, gpu.gb_last_error_string()
    try:
        if kind == 0:
            xs = [signals.complex_uniform(29600 + i, N * B) for i in range(count)]
            nout, dt = N * B, np.complex64
        elif kind == 1:
            xs = [signals.uniform(29600 + i, N * B) for i in range(count)]
            nout, dt = (N // 2 + 1) * B, np.complex64
        else:
            xs = [signals.complex_uniform(29600 + i, (N // 2 + 1) * B) for i in range(count)]
            nout, dt = N * B, np.float32
        pinned = [gpu.alloc(x.nbytes) for x in xs]
        for h, x in zip(pinned, xs):
            C.memmove(h, x.ctypes.data, x.nbytes)
        outs_p = [gpu.alloc(nout * np.dtype(dt).itemsize) for _ in xs]
        outs_q = [np.full(nout, np.nan, dt) for _ in xs]  # pageable
        for outs in (outs_p, [o.ctypes.data for o in outs_q]):
            ins = (C.c_void_p * count)(*pinned)
            ol = (C.c_void_p * count)(*outs)
            assert gpu.gb_execute_plan_1d_host_pipeline(plan, ol, ins, count) == 0, gpu.gb_last_error_string()
        for i, x in enumerate(xs):
            want = np.full(nout, np.nan, dt)
            gpu.execute_plan_1d(plan, want.ctypes.data, pinned[i])
            gpu.check("execute")
            got_p = np.frombuffer((C.c_char * want.nbytes).from_address(outs_p[i]), dt)
            assert np.array_equal(got_p.view(np.uint32), want.view(np.uint32)), i
            assert np.array_equal(outs_q[i].view(np.uint32), want.view(np.uint32)), i
        for h in pinned + outs_p:
            gpu.free(h)
    finally:
        gpu.free_plan_1d(plan)
