"""The oracle (CPU restatement of the reference's scalar path) is pinned
against the reference library: bit-exact on the portable C tier through the
golden fixtures, and live against the reference when it was compiled here."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import bitwise_equal, direct_conv_f64, golden, golden_cases, rel_l2
from mufft_gb300 import capi as K
from mufft_gb300 import signals
from oracle.oracle import load_oracle, load_reference


@pytest.fixture(scope="module")
def ora():
    return load_oracle()


def _n(case, key="N"):
    for part in case.split("/"):
        if part.startswith(key) and part[len(key):].isdigit():
            return int(part[len(key):])
    raise KeyError(case)


def _check(case, got):
    g = golden()
    assert bitwise_equal(got, g[case + "/c"]), case
    if case + "/simd" in g:
        assert rel_l2(got, g[case + "/simd"]) <= 1e-6, case


@pytest.mark.parametrize("case", golden_cases("c2c"))
def test_c2c_golden(ora, case):
    g = golden()
    N = _n(case)
    d = K.FORWARD if "/d-1/" in case else K.INVERSE
    zp = K.FLAG_ZERO_PAD_UPPER_HALF if case.endswith("zp1") else 0
    _check(case, ora.fft_c2c(g[case + "/in"], d, zp, N))


@pytest.mark.parametrize("case", golden_cases("r2c"))
def test_r2c_golden(ora, case):
    g = golden()
    N = _n(case)
    fl = (K.FLAG_FULL_R2C if "full1" in case else 0) | (K.FLAG_ZERO_PAD_UPPER_HALF if case.endswith("zp1") else 0)
    _check(case, ora.fft_r2c(g[case + "/in"], fl, N))


@pytest.mark.parametrize("case", golden_cases("c2r"))
def test_c2r_golden(ora, case):
    g = golden()
    _check(case, ora.fft_c2r(g[case + "/in"], _n(case)))


@pytest.mark.parametrize("case", golden_cases("conv"))
def test_conv_golden(ora, case):
    g = golden()
    N = _n(case)
    m = int(case.rsplit("/m", 1)[1])
    _check(case, ora.conv(g[case + "/in"], g[case + "/in2"], N, m))


@pytest.mark.parametrize("case", golden_cases("c2c2d") + golden_cases("r2c2d") + golden_cases("c2r2d"))
def test_2d_golden(ora, case):
    g = golden()
    kind, size = case.split("/")[:2]
    Nx, Ny = map(int, size.split("x"))
    x = g[case + "/in"]
    if kind == "c2c2d":
        got = ora.fft2_c2c(x, K.FORWARD if "/d-1" in case else K.INVERSE)
    elif kind == "r2c2d":
        full = "full1" in case
        got = ora.fft2_r2c(x, K.FLAG_FULL_R2C if full else 0)[:, : (Nx if full else Nx // 2 + 1)]
    else:
        got = ora.fft2_c2r(x)
    _check(case, np.ascontiguousarray(got))


def test_plan_decomposition(ora):
    # Decompositions the reference's greedy planner produces (fft.c:325-379).
    assert ora.steps(1024, K.FORWARD) == [(8, 1), (8, 8), (8, 64), (2, 512)]
    assert ora.steps(4096, K.FORWARD) == [(8, 1), (8, 8), (8, 64), (8, 512)]
    assert ora.steps(2048, K.INVERSE) == [(2, 1), (2, 2), (4, 4), (8, 16), (8, 128), (2, 1024)]
    assert ora.steps(2, K.FORWARD) == [(2, 1)]
    assert ora.steps(16, K.FORWARD) == [(8, 1), (2, 8)]


def test_rejects_like_reference(ora):
    assert not ora.create_plan_1d_c2c(1, K.FORWARD, 0)
    assert not ora.create_plan_1d_c2c(12, K.FORWARD, 0)
    assert not ora.create_plan_1d_r2c(2, 0)
    assert not ora.create_plan_1d_c2r(2, 0)
    assert not ora.create_plan_conv(2, 0, 0)
    assert not ora.create_plan_2d_c2c(1, 4, K.FORWARD, 0)
    assert not ora.create_plan_2d_r2c(2, 4, 0)


@pytest.mark.parametrize("N", [8, 64, 512, 4096, 65536])
def test_oracle_accuracy_fp64(ora, N):
    x = signals.complex_uniform(11, N)
    ref = np.fft.fft(x.astype(np.complex128))
    assert rel_l2(ora.fft_c2c(x, K.FORWARD), ref) < 1e-6
    if N <= 512:
        assert rel_l2(ora.dft_f64(x, K.FORWARD), ref) < 1e-12


@pytest.mark.parametrize("N", [16, 128])
@pytest.mark.parametrize("method", [0, 1])
def test_oracle_conv_direct(ora, N, method):
    a = (signals.complex_uniform(12, N // 2) if method else signals.uniform(12, N // 2))
    b = signals.uniform(13, N // 2)
    m = method | K.CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_FIRST | K.CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_SECOND
    got = ora.conv(a, b, N, m)
    ref = direct_conv_f64(a, b, N)
    if not method:
        ref = ref.real
    assert rel_l2(got, ref) < 1e-6


def test_many_threads_matches_single(ora):
    x = signals.complex_uniform(14, 64 * 256).reshape(64, 256)
    many = ora.c2c_many(x, K.FORWARD, 4)
    for i in (0, 17, 63):
        assert bitwise_equal(many[i], ora.fft_c2c(x[i], K.FORWARD))


ref_lib = load_reference()


@pytest.mark.skipif(ref_lib is None, reason="reference library not compiled here (oracle/build_ref.sh)")
@pytest.mark.parametrize("N", [2048, 8192, 65536])
def test_oracle_equals_reference_live(ora, N):
    x = signals.complex_uniform(15, N)
    for d in (K.FORWARD, K.INVERSE):
        assert bitwise_equal(ora.fft_c2c(x, d), ref_lib.fft_c2c(x, d, K.FLAG_CPU_NO_SIMD))
    xr = signals.uniform(16, N)
    assert bitwise_equal(ora.fft_r2c(xr), ref_lib.fft_r2c(xr, K.FLAG_CPU_NO_SIMD))
    X = signals.complex_uniform(17, N // 2 + 1)
    assert bitwise_equal(ora.fft_c2r(X, N), ref_lib.fft_c2r(X, N, K.FLAG_CPU_NO_SIMD))
