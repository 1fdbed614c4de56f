"""GPU parity: libmufft_gb300 through its C ABI against the oracle (the
reference's scalar path restated) on identical seeded inputs, following the
sweeps of the reference's test.c:490-579.

Bar: relative L2 error <= 1e-5 (REL_L2_TOL) and, as test.c does against FFTW,
a per-element bound |gpu - oracle| < tol * sqrt(N) scaled to the inputs'
range ([-1, 1) here, [-0.5, 0.5) in test.c).
"""
from __future__ import annotations

import numpy as np
import pytest

from helpers import REL_L2_TOL, direct_conv_f64, golden, golden_cases, max_abs, rel_l2
from mufft_gb300 import capi as K
from mufft_gb300.capi import aligned_copy
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


def assert_close(got, want, N, elem_tol=2e-6, what=""):
    assert got.shape == want.shape, what
    assert np.all(np.isfinite(got)), what
    e = rel_l2(got, want)
    assert e <= REL_L2_TOL, f"{what}: rel L2 {e:.3e}"
    m = max_abs(got, want)
    scale = max(1.0, float(np.abs(want).max()) / np.sqrt(N))
    assert m < elem_tol * np.sqrt(N) * scale * 4, f"{what}: max abs {m:.3e}"


SIZES_1D = [2 ** e for e in range(1, 17)]


@pytest.mark.parametrize("N", SIZES_1D)
@pytest.mark.parametrize("direction", [K.FORWARD, K.INVERSE])
def test_c2c(gpu, ora, N, direction):
    x = signals.complex_uniform(1000 + N, N)
    assert_close(gpu.fft_c2c(x, direction), ora.fft_c2c(x, direction), N, what=f"c2c N={N} d={direction}")


@pytest.mark.parametrize("N", SIZES_1D)
@pytest.mark.parametrize("direction", [K.FORWARD, K.INVERSE])
def test_c2c_zero_pad(gpu, ora, N, direction):
    x = signals.complex_uniform(2000 + N, N // 2)
    fl = K.FLAG_ZERO_PAD_UPPER_HALF
    assert_close(gpu.fft_c2c(x, direction, fl, N), ora.fft_c2c(x, direction, fl, N), N, what=f"c2c zp N={N}")


@pytest.mark.parametrize("N", SIZES_1D[1:])
@pytest.mark.parametrize("flags", [0, K.FLAG_FULL_R2C, K.FLAG_ZERO_PAD_UPPER_HALF,
                                   K.FLAG_FULL_R2C | K.FLAG_ZERO_PAD_UPPER_HALF])
def test_r2c(gpu, ora, N, flags):
    n_in = N // 2 if flags & K.FLAG_ZERO_PAD_UPPER_HALF else N
    x = signals.uniform(3000 + N, n_in)
    got = gpu.fft_r2c(x, flags, N)
    want = ora.fft_r2c(x, flags, N)
    assert_close(got, want, N, what=f"r2c N={N} flags={flags:#x}")
    if flags & K.FLAG_FULL_R2C:
        # conjugate symmetry of the full output (test.c:295-302)
        k = np.arange(1, N // 2)
        assert max_abs(got[k], np.conj(got[N - k])) < 1e-5 * np.sqrt(N) * 4


@pytest.mark.parametrize("N", SIZES_1D[1:])
def test_c2r(gpu, ora, N):
    X = signals.complex_uniform(4000 + N, N // 2 + 1)
    X[0] = X[0].real
    X[N // 2] = X[N // 2].real
    assert_close(gpu.fft_c2r(X, N), ora.fft_c2r(X, N), N, what=f"c2r N={N}")


@pytest.mark.parametrize("N", [2 ** e for e in range(2, 15)])
@pytest.mark.parametrize("method", [0, 1, 4, 8, 12, 13])
def test_conv(gpu, ora, N, method):
    stereo = method & 1
    a = signals.complex_uniform(5000 + N, N) if stereo else signals.uniform(5000 + N, N)
    b = signals.uniform(6000 + N, N)
    if method & 4:
        a = a[: N // 2].copy()
    if method & 8:
        b = b[: N // 2].copy()
    assert_close(gpu.conv(a, b, N, method), ora.conv(a, b, N, method), N, elem_tol=4e-6,
                 what=f"conv N={N} m={method}")


@pytest.mark.parametrize("N", [16, 256, 2048])
@pytest.mark.parametrize("method", [12, 13])
def test_conv_vs_direct_fp64(gpu, N, method):
    stereo = method & 1
    a = signals.complex_uniform(7000 + N, N // 2) if stereo else signals.uniform(7000 + N, N // 2)
    b = signals.uniform(7100 + N, N // 2)
    ref = direct_conv_f64(a, b, N)
    got = gpu.conv(a, b, N, method)
    assert rel_l2(got, ref if stereo else ref.real) < 1e-5


SIZES_2D = [(2, 2), (4, 2), (2, 8), (8, 8), (16, 4), (32, 64), (64, 16), (4, 512), (512, 4),
            (128, 256), (512, 512)]


@pytest.mark.parametrize("Nx,Ny", SIZES_2D)
@pytest.mark.parametrize("direction", [K.FORWARD, K.INVERSE])
def test_2d_c2c(gpu, ora, Nx, Ny, direction):
    x = signals.complex_uniform(8000 + Nx * 7 + Ny, Nx * Ny).reshape(Ny, Nx)
    assert_close(gpu.fft2_c2c(x, direction), ora.fft2_c2c(x, direction), Nx * Ny, what=f"2d {Nx}x{Ny}")


@pytest.mark.parametrize("Nx,Ny", [s for s in SIZES_2D if s[0] >= 4])
@pytest.mark.parametrize("full", [0, K.FLAG_FULL_R2C])
def test_2d_r2c(gpu, ora, Nx, Ny, full):
    x = signals.uniform(9000 + Nx * 7 + Ny, Nx * Ny).reshape(Ny, Nx)
    vx = Nx if full else Nx // 2 + 1
    got = gpu.fft2_r2c(x, full)[:, :vx]
    want = ora.fft2_r2c(x, full)[:, :vx]
    assert_close(got, want, Nx * Ny, what=f"2d r2c {Nx}x{Ny}")


@pytest.mark.parametrize("Nx,Ny", [s for s in SIZES_2D if s[0] >= 4])
def test_2d_c2r(gpu, ora, Nx, Ny):
    X = signals.complex_uniform(9500 + Nx * 7 + Ny, Nx * Ny).reshape(Ny, Nx)
    assert_close(gpu.fft2_c2r(X), ora.fft2_c2r(X), Nx * Ny, what=f"2d c2r {Nx}x{Ny}")


# ------------------------------------------------------------- golden vectors

def _golden_run(gpu, case):
    g = golden()
    kind = case.split("/")[0]
    x = g[case + "/in"]
    if kind in ("c2c", "r2c", "c2r", "conv"):
        N = int(case.split("/")[1][1:])
    if kind == "c2c":
        d = K.FORWARD if "/d-1/" in case else K.INVERSE
        return gpu.fft_c2c(x, d, K.FLAG_ZERO_PAD_UPPER_HALF if case.endswith("zp1") else 0, N), N
    if kind == "r2c":
        fl = (K.FLAG_FULL_R2C if "full1" in case else 0) | (K.FLAG_ZERO_PAD_UPPER_HALF if case.endswith("zp1") else 0)
        return gpu.fft_r2c(x, fl, N), N
    if kind == "c2r":
        return gpu.fft_c2r(x, N), N
    if kind == "conv":
        return gpu.conv(x, g[case + "/in2"], N, int(case.rsplit("/m", 1)[1])), N
    Nx, Ny = map(int, case.split("/")[1].split("x"))
    if kind == "c2c2d":
        return gpu.fft2_c2c(x, K.FORWARD if "/d-1" in case else K.INVERSE), Nx * Ny
    if kind == "r2c2d":
        full = "full1" in case
        return np.ascontiguousarray(gpu.fft2_r2c(x, K.FLAG_FULL_R2C if full else 0)[:, : (Nx if full else Nx // 2 + 1)]), Nx * Ny
    return gpu.fft2_c2r(x), Nx * Ny


ALL_GOLDEN = [c for p in ("c2c", "r2c", "c2r", "conv", "c2c2d", "r2c2d", "c2r2d") for c in golden_cases(p)]


@pytest.mark.parametrize("case", ALL_GOLDEN)
def test_golden_vectors(gpu, case):
    got, n = _golden_run(gpu, case)
    want = golden()[case + "/c"]
    assert_close(got, want, n, elem_tol=4e-6, what=case)


# ----------------------------------------------------- multi-pass lengths

@pytest.mark.parametrize("lg", [17, 18, 20, 22, 24])
def test_large_c2c_vs_fp64(gpu, lg):
    N = 1 << lg
    x = signals.complex_uniform(10000 + lg, N)
    ref = np.fft.fft(x.astype(np.complex128))
    got = gpu.fft_c2c(x, K.FORWARD)
    assert rel_l2(got, ref) < 2e-6
    back = gpu.fft_c2c(got, K.INVERSE)
    assert rel_l2(back / N, x) < 4e-6


@pytest.mark.parametrize("lg", [17, 20])
def test_large_vs_oracle(gpu, ora, lg):
    N = 1 << lg
    x = signals.complex_uniform(11000 + lg, N)
    for d in (K.FORWARD, K.INVERSE):
        assert_close(gpu.fft_c2c(x, d), ora.fft_c2c(x, d), N, what=f"c2c 2^{lg}")
    xh = x[: N // 2].copy()
    assert_close(gpu.fft_c2c(xh, K.FORWARD, K.FLAG_ZERO_PAD_UPPER_HALF, N),
                 ora.fft_c2c(xh, K.FORWARD, K.FLAG_ZERO_PAD_UPPER_HALF, N), N, what="zp")
    xr = signals.uniform(11100 + lg, N)
    for fl in (0, K.FLAG_FULL_R2C):
        assert_close(gpu.fft_r2c(xr, fl), ora.fft_r2c(xr, fl), N, what=f"r2c 2^{lg}")
    X = signals.complex_uniform(11200 + lg, N // 2 + 1)
    assert_close(gpu.fft_c2r(X, N), ora.fft_c2r(X, N), N, what=f"c2r 2^{lg}")


@pytest.mark.parametrize("N,method", [(1 << 16, 12), (1 << 16, 13), (1 << 18, 12), (1 << 17, 1)])
def test_large_conv(gpu, ora, N, method):
    stereo = method & 1
    a = signals.complex_uniform(12000 + N, N) if stereo else signals.uniform(12000 + N, N)
    b = signals.uniform(12100 + N, N)
    if method & 4:
        a = a[: N // 2].copy()
    if method & 8:
        b = b[: N // 2].copy()
    assert_close(gpu.conv(a, b, N, method), ora.conv(a, b, N, method), N, elem_tol=4e-6, what=f"conv {N}")


@pytest.mark.parametrize("Nx", [64, 2048])
def test_2d_persistent_columns_match_oracle(gpu, ora, Nx):
    """4096-point columns run as a persistent grid (default): the same bits as
    one launch per tile, and the oracle's results, for r2c, c2r and both c2c
    directions (64 columns: fewer tiles than SMs; 2048: several tiles per CTA)."""
    Ny = 4096
    on, off = gpu.options(persistent_tiles=1), gpu.options(persistent_tiles=0)
    x = signals.uniform(13100 + Nx, Nx * Ny).reshape(Ny, Nx)
    vx = Nx // 2 + 1
    a, b = gpu.fft2_r2c(x, opts=on), gpu.fft2_r2c(x, opts=off)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert_close(a[:, :vx], ora.fft2_r2c(x, 0)[:, :vx], Nx * Ny, what=f"2d r2c {Nx}x{Ny}")
    X = signals.complex_uniform(13200 + Nx, Nx * Ny).reshape(Ny, Nx)
    a, b = gpu.fft2_c2r(X, opts=on), gpu.fft2_c2r(X, opts=off)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert_close(a, ora.fft2_c2r(X), Nx * Ny, what=f"2d c2r {Nx}x{Ny}")
    for d in (K.FORWARD, K.INVERSE):
        a, b = gpu.fft2_c2c(X, d, opts=on), gpu.fft2_c2c(X, d, opts=off)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
        assert_close(a, ora.fft2_c2c(X, d), Nx * Ny, what=f"2d c2c {Nx}x{Ny} {d}")


def test_persistent_column_plans_created_in_any_order(gpu):
    """The persistent 4096-point column tile serves launches with the twiddle
    region (1D four-step 4096 x 4096) and without it (2D columns): a plan
    created afterwards must not lower the kernel's shared-memory limit under
    the earlier plan's launch."""
    N = 1 << 24
    four_step = gpu._plan_1d(0, N, K.FORWARD, 0, gpu.options(multipass_levels=2))
    try:
        xr = signals.uniform(14200, 2048 * 4096).reshape(4096, 2048)
        X = gpu.fft2_r2c(xr)  # one-pass persistent columns, no twiddle region
        assert rel_l2(X[:, :1025], np.fft.rfft2(xr.astype(np.float64))) < 2e-6
        x = aligned_copy(signals.complex_uniform(14300, N), np.complex64)
        y = np.zeros(N, np.complex64)
        gpu.execute_plan_1d(four_step, y.ctypes.data, x.ctypes.data)
        gpu.check("execute_plan_1d")
        assert rel_l2(y, np.fft.fft(x.astype(np.complex128))) < 2e-6
    finally:
        gpu.free_plan_1d(four_step)


def test_l2_residency_hints_change_no_bits(gpu, ora):
    """The L2 cache-policy hints (and the discard of dead intermediates) leave
    every output bit unchanged: three-level c2c 2^22, four-step r2c / c2r
    batches, 2D c2r with a discarded scratch; the hinted results also against
    the oracle / FP64."""
    on, off = gpu.options(l2_residency=1), gpu.options(l2_residency=0)
    same = lambda u, v: np.array_equal(u.view(np.uint32), v.view(np.uint32))  # noqa: E731
    N = 1 << 22
    x = signals.complex_uniform(14000, N)
    a, b = gpu.fft_c2c(x, K.FORWARD, opts=on), gpu.fft_c2c(x, K.FORWARD, opts=off)
    assert same(a, b)
    assert rel_l2(a, np.fft.fft(x.astype(np.complex128))) < 2e-6
    N = 1 << 21
    r = signals.uniform(14050, N)
    a, b = gpu.fft_r2c(r, opts=on), gpu.fft_r2c(r, opts=off)
    assert same(a, b)
    assert rel_l2(a, np.fft.rfft(r.astype(np.float64))) < 2e-6
    back, back0 = gpu.fft_c2r(a, N, opts=on), gpu.fft_c2r(a, N, opts=off)
    assert same(back, back0)
    assert rel_l2(back / N, r) < 4e-6
    Nx, Ny = 256, 4096
    X = signals.complex_uniform(14100, Nx * Ny).reshape(Ny, Nx)
    c, d = gpu.fft2_c2r(X, opts=on), gpu.fft2_c2r(X, opts=off)
    assert np.array_equal(c.view(np.uint32), d.view(np.uint32))
    assert_close(c, ora.fft2_c2r(X), Nx * Ny, what="2d c2r 256x4096")


def test_2d_4096_round_trip(gpu):
    Nx = Ny = 4096
    x = signals.normal(13000, Nx * Ny).reshape(Ny, Nx)
    X = gpu.fft2_r2c(x)
    # spot-check rows of the spectrum against FP64
    ref = np.fft.rfft2(x.astype(np.float64))
    assert rel_l2(X[:, : Nx // 2 + 1], ref) < 2e-6
    back = gpu.fft2_c2r(X)
    assert rel_l2(back / (Nx * Ny), x) < 4e-6
