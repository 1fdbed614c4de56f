"""GPU tests of the convolution adjoints (mufft_gb_conv_adjoint_input /
_filter) against the FP64 oracle (oracle/adjoint.py), finite differences of
the loss, and a 200-step gradient descent that recovers a hidden filter."""
from __future__ import annotations

import numpy as np
import pytest

from helpers import rel_l2
from mufft_gb300 import capi as K
from mufft_gb300 import signals
from oracle import adjoint as A

pytestmark = pytest.mark.gpu

STEREO = K.CONV_METHOD_FLAG_STEREO_MONO
PAD1 = K.CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_FIRST
PAD2 = K.CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_SECOND
ADJ_TOL = 1e-5  # relative L2 against FP64 (the bar for gradients is 1e-4)


@pytest.fixture(scope="module")
def gpu():
    import mufft_gb300
    return mufft_gb300.load()


@pytest.fixture(scope="module")
def torch():
    import torch as t
    assert t.cuda.is_available()
    return t


def _st(torch):
    return torch.cuda.current_stream().cuda_stream


class ConvPlan:
    def __init__(self, gpu, N, method):
        self.gpu, self.N, self.method = gpu, N, method
        self.stereo = bool(method & 1)
        self.p = gpu.create_plan_conv(N, 0, method)
        assert self.p, gpu.gb_last_error_string()
        self.block = gpu.conv_get_transformed_block_size(self.p) // 8

    def spectrum(self, torch, block, x_dev):
        out = torch.empty(self.block, dtype=torch.complex64, device="cuda")
        rc = self.gpu.gb_execute_conv_input_async(self.p, block, out.data_ptr(), x_dev.data_ptr(), _st(torch))
        assert rc == 0, self.gpu.gb_last_error_string()
        return out

    def free(self):
        self.gpu.free_plan_conv(self.p)


def _signal(seed, N, stereo):
    return signals.complex_uniform(seed, N) if stereo else signals.uniform(seed, N)


def _dev(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


@pytest.mark.parametrize("N", [16, 256, 4096, 1 << 16, 1 << 21])
@pytest.mark.parametrize("method", [0, STEREO, PAD1 | PAD2, STEREO | PAD2])
def test_adjoint_input_vs_fp64(gpu, torch, N, method):
    pl = ConvPlan(gpu, N, method)
    try:
        b = signals.uniform(30000 + N, N)
        g = _signal(30001 + N, N, pl.stereo)
        H = pl.spectrum(torch, K.CONV_BLOCK_SECOND, _dev(torch, b))
        dg = _dev(torch, g)
        out = torch.full((N,), float("nan"), dtype=torch.complex64 if pl.stereo else torch.float32, device="cuda")
        rc = gpu.gb_conv_adjoint_input(pl.p, out.data_ptr(), dg.data_ptr(), H.data_ptr(), _st(torch))
        assert rc == 0, gpu.gb_last_error_string()
        torch.cuda.synchronize()
    finally:
        pl.free()
    b_eff = b.astype(np.float64)
    if method & PAD2:
        b_eff[N // 2:] = 0
    ref = A.adjoint_input_f64(g, b_eff, pl.stereo)
    assert rel_l2(out.cpu().numpy(), ref) < ADJ_TOL


@pytest.mark.parametrize("N,B", [(16, 1), (1024, 7), (1 << 16, 3), (1 << 21, 2), (1 << 23, 5)])
@pytest.mark.parametrize("method", [0, STEREO | PAD1])
def test_adjoint_filter_vs_fp64(gpu, torch, N, B, method):
    """Batch sums over spectra; (2^23, 5) runs a ragged last chunk."""
    if N == 1 << 23 and not method & 1:
        pytest.skip("the ragged chunk needs the stereo spectrum size")
    pl = ConvPlan(gpu, N, method)
    try:
        firsts = np.stack([_signal(31000 + N + i, N, pl.stereo) for i in range(B)])
        grads = np.stack([_signal(32000 + N + i, N, pl.stereo) for i in range(B)])
        dA = torch.empty((B, pl.block), dtype=torch.complex64, device="cuda")
        for i in range(B):
            dA[i] = pl.spectrum(torch, K.CONV_BLOCK_FIRST, _dev(torch, firsts[i]))
        dg = _dev(torch, grads)
        out = torch.full((N,), float("nan"), dtype=torch.float32, device="cuda")
        rc = gpu.gb_conv_adjoint_filter(pl.p, out.data_ptr(), dg.data_ptr(), N, dA.data_ptr(), pl.block, B,
                                        _st(torch))
        assert rc == 0, gpu.gb_last_error_string()
        torch.cuda.synchronize()
    finally:
        pl.free()
    f_eff = firsts.astype(np.complex128 if pl.stereo else np.float64)
    if method & PAD1:
        f_eff[:, N // 2:] = 0
    ref = A.adjoint_filter_f64(grads, f_eff)
    assert rel_l2(out.cpu().numpy(), ref) < ADJ_TOL


@pytest.mark.parametrize("method", [0, STEREO])
def test_adjoint_matches_finite_differences(gpu, torch, method):
    """GPU gradients of 0.5*||conv(first, second) - target||^2 against FP64
    central differences on 256 random coordinates of each, to 1e-4 relative."""
    N, B = 1024, 2
    pl = ConvPlan(gpu, N, method)
    try:
        firsts = np.stack([_signal(33000 + i, N, pl.stereo) for i in range(B)])
        second = signals.uniform(33100, N)
        targets = np.stack([_signal(33200 + i, N, pl.stereo) for i in range(B)])
        r = np.stack([A.conv_f64(f, second, pl.stereo) for f in firsts]) - targets
        r32 = r.astype(np.complex64 if pl.stereo else np.float32)
        H = pl.spectrum(torch, K.CONV_BLOCK_SECOND, _dev(torch, second))
        dA = torch.stack([pl.spectrum(torch, K.CONV_BLOCK_FIRST, _dev(torch, f)) for f in firsts])
        dr = _dev(torch, r32)
        gf = torch.empty(N, dtype=torch.float32, device="cuda")
        assert gpu.gb_conv_adjoint_filter(pl.p, gf.data_ptr(), dr.data_ptr(), N, dA.data_ptr(), pl.block, B,
                                          _st(torch)) == 0
        gi = torch.empty(N, dtype=torch.complex64 if pl.stereo else torch.float32, device="cuda")
        assert gpu.gb_conv_adjoint_input(pl.p, gi.data_ptr(), dr[1].data_ptr(), H.data_ptr(), _st(torch)) == 0
        torch.cuda.synchronize()
    finally:
        pl.free()
    gf, gi = gf.cpu().numpy(), gi.cpu().numpy()
    scale_f, scale_i = np.abs(gf).max(), np.abs(gi).max()
    coords = np.random.default_rng(35).choice(N, 256, replace=False)
    for j in coords:
        fd = A.finite_difference(lambda s: A.loss_f64(firsts, s, targets, pl.stereo), second.astype(np.float64), j)
        assert abs(fd - gf[j]) < 1e-4 * scale_f, ("filter", j, fd, gf[j])

        def loss_first(f1):
            f = firsts.astype(f1.dtype)
            f[1] = f1
            return A.loss_f64(f, second, targets, pl.stereo)
        x1 = firsts[1].astype(np.complex128 if pl.stereo else np.float64)
        fd = A.finite_difference(loss_first, x1, j)
        assert abs(fd - gi[j]) < 1e-4 * scale_i, ("input", j, fd, gi[j])


def test_gradient_descent_recovers_filter(gpu, torch):
    """200 steps of gradient descent on the taps of a filter shared by 8 stereo
    signals (conv_input, conv_output and the filter adjoint on the GPU)."""
    N, B, T = 4096, 8, 128
    method = STEREO | PAD1 | PAD2
    t = np.arange(T)
    h_true = signals.normal(34000, T) * np.exp(-t / (T / 4))
    x = np.zeros((B, N), np.complex64)
    for i in range(B):
        x[i, : N // 2] = signals.complex_uniform(34100 + i, N // 2)
    h_pad = np.zeros(N)
    h_pad[:T] = h_true
    targets = np.stack([A.conv_f64(x[i], h_pad, True) for i in range(B)]).astype(np.complex64)
    spec = np.fft.fft(x.astype(np.complex128), axis=1)
    lr = 1.0 / float(np.max(np.sum(np.abs(spec) ** 2, axis=0)))

    pl = ConvPlan(gpu, N, method)
    try:
        dA = torch.stack([pl.spectrum(torch, K.CONV_BLOCK_FIRST, _dev(torch, x[i])) for i in range(B)])
        dt = _dev(torch, targets)
        h = torch.zeros(N, dtype=torch.float32, device="cuda")
        y = torch.empty((B, N), dtype=torch.complex64, device="cuda")
        grad = torch.empty(N, dtype=torch.float32, device="cuda")
        st = _st(torch)
        losses = []
        for step in range(200):
            H = pl.spectrum(torch, K.CONV_BLOCK_SECOND, h)
            for i in range(B):
                assert gpu.gb_execute_conv_output_async(pl.p, y[i].data_ptr(), dA[i].data_ptr(), H.data_ptr(),
                                                        st) == 0
            r = y - dt
            losses.append(0.5 * float(torch.sum(torch.abs(r) ** 2)))
            assert gpu.gb_conv_adjoint_filter(pl.p, grad.data_ptr(), r.data_ptr(), N, dA.data_ptr(), pl.block,
                                              B, st) == 0
            h[:T] -= lr * grad[:T]
        h_got = h[:T].cpu().numpy()
    finally:
        pl.free()
    assert losses[-1] < 1e-8 * losses[0], (losses[0], losses[-1])
    # monotone until the FP32 floor
    far = [i for i in range(1, len(losses)) if losses[i - 1] > 1e-6 * losses[0]]
    assert len(far) >= 5 and all(losses[i] <= losses[i - 1] for i in far), losses[:12]
    assert rel_l2(h_got, h_true) < 1e-4


@pytest.mark.parametrize("N,B", [(256, 5), (4096, 3), (1 << 17, 3), (1 << 23, 5)])
@pytest.mark.parametrize("method", [0, STEREO, PAD1 | PAD2, STEREO | PAD1])
def test_batched_conv_output_and_adjoint_vs_fp64(gpu, torch, N, B, method):
    """mufft_gb_execute_conv_output_batched and mufft_gb_conv_adjoint (one
    filter spectrum broadcast over the batch; one forward transform of each
    output gradient for both gradients) against FP64.  Single-pass (N <=
    16384: the filter is shared across transforms of one tile) and
    multi-pass sizes; (2^23, 5) runs a ragged last chunk (stereo)."""
    if N == 1 << 23 and not method & 1:
        pytest.skip("the ragged chunk needs the stereo spectrum size")
    pl = ConvPlan(gpu, N, method)
    try:
        stereo = pl.stereo
        firsts = np.stack([_signal(33000 + N + i, N, stereo) for i in range(B)])
        grads = np.stack([_signal(34000 + N + i, N, stereo) for i in range(B)])
        b = signals.uniform(35000 + N, N)
        H = pl.spectrum(torch, K.CONV_BLOCK_SECOND, _dev(torch, b))
        dA = torch.empty((B, pl.block), dtype=torch.complex64, device="cuda")
        for i in range(B):
            dA[i] = pl.spectrum(torch, K.CONV_BLOCK_FIRST, _dev(torch, firsts[i]))
        dt = torch.complex64 if stereo else torch.float32
        outs = torch.full((B, N), float("nan"), dtype=dt, device="cuda")
        rc = gpu.gb_execute_conv_output_batched(pl.p, outs.data_ptr(), N, dA.data_ptr(), pl.block, H.data_ptr(), B,
                                                _st(torch))
        assert rc == 0, gpu.gb_last_error_string()
        dg = _dev(torch, grads)
        gx = torch.full((B, N), float("nan"), dtype=dt, device="cuda")
        gh = torch.full((N,), float("nan"), dtype=torch.float32, device="cuda")
        rc = gpu.gb_conv_adjoint(pl.p, gh.data_ptr(), gx.data_ptr(), N, dg.data_ptr(), N, dA.data_ptr(), pl.block,
                                 H.data_ptr(), B, _st(torch))
        assert rc == 0, gpu.gb_last_error_string()
        # one gradient at a time gives the same numbers as both at once
        gx2 = torch.full((B, N), float("nan"), dtype=dt, device="cuda")
        rc = gpu.gb_conv_adjoint(pl.p, None, gx2.data_ptr(), N, dg.data_ptr(), N, None, 0, H.data_ptr(), B,
                                 _st(torch))
        assert rc == 0, gpu.gb_last_error_string()
        torch.cuda.synchronize()
    finally:
        pl.free()
    f_eff = firsts.astype(np.complex128 if stereo else np.float64)
    if method & PAD1:
        f_eff[:, N // 2:] = 0
    b_eff = b.astype(np.float64)
    if method & PAD2:
        b_eff[N // 2:] = 0
    got_out, got_gx = outs.cpu().numpy(), gx.cpu().numpy()
    for i in range(B):
        assert rel_l2(got_out[i], A.conv_f64(f_eff[i], b_eff, stereo)) < ADJ_TOL, i
        assert rel_l2(got_gx[i], A.adjoint_input_f64(grads[i], b_eff, stereo)) < ADJ_TOL, i
    assert rel_l2(gh.cpu().numpy(), A.adjoint_filter_f64(grads, f_eff)) < ADJ_TOL
    assert np.array_equal(got_gx.view(np.uint32), gx2.cpu().numpy().view(np.uint32))


def test_batched_adjoint_rejects_bad_arguments(gpu, torch):
    pl = ConvPlan(gpu, 1024, STEREO)
    try:
        d = torch.zeros(4 * 1024, dtype=torch.complex64, device="cuda")
        p = d.data_ptr()
        # nothing to compute; distances below one block; empty batch
        for args in [(None, None, 1024, p, 1024, p, pl.block, p, 2),
                     (p, p, 512, p, 1024, p, pl.block, p, 2),
                     (p, p, 1024, p, 1024, p, 16, p, 2),
                     (p, p, 1024, p, 1024, p, pl.block, p, 0)]:
            assert gpu.gb_conv_adjoint(pl.p, *args, _st(torch)) != 0
            gpu.gb_clear_error()
        assert gpu.gb_execute_conv_output_batched(pl.p, p, 512, p, pl.block, p, 2, _st(torch)) != 0
        gpu.gb_clear_error()
    finally:
        pl.free()


def test_adjoint_full_workload(gpu, torch):
    """The filter-fitting workload at full size: 64 stereo signals of 2^20
    frames, a 2^16-tap filter (N(0,1) * exp(-t/8192)), N = 2^21 with both
    blocks zero-padded so the circular convolution is the linear one, loss
    0.5 * sum_b ||conv(x_b, h) - y*_b||^2 with y* made by a hidden filter.
      1. Both GPU gradients (mufft_gb_conv_adjoint, all 64 signals) against
         the FP64 gradient of the same loss, relative L2 <= 1e-4.
      2. FP64 central differences of the loss (torch float64 FFTs on the GPU)
         on 256 random filter taps and 256 random input samples.
      3. 200 steps of gradient descent on the taps: the loss falls
         monotonically until it reaches the FP32 floor."""
    B, L, T = 64, 1 << 20, 1 << 16
    N = 2 * L
    method = STEREO | PAD1 | PAD2
    st = _st(torch)
    g = torch.Generator(device="cuda").manual_seed(5)
    x = torch.zeros((B, N), dtype=torch.complex64, device="cuda")
    x[:, :L].real.uniform_(-1, 1, generator=g)
    x[:, :L].imag.uniform_(-1, 1, generator=g)
    t = torch.arange(T, device="cuda", dtype=torch.float64)
    h_hidden = torch.zeros(N, dtype=torch.float64, device="cuda")
    h_hidden[:T] = torch.randn(T, device="cuda", generator=g, dtype=torch.float64) * torch.exp(-t / 8192)
    h0 = torch.zeros(N, dtype=torch.float64, device="cuda")
    h0[:T] = torch.randn(T, device="cuda", generator=g, dtype=torch.float64) * torch.exp(-t / 8192)

    # FP64 spectra of the signals; targets y* = conv(x, h_hidden) rounded to complex64
    X = torch.fft.fft(x.to(torch.complex128), dim=1)
    ystar = torch.empty((B, N), dtype=torch.complex64, device="cuda")
    Hh = torch.fft.fft(h_hidden)
    for c in range(0, B, 8):
        ystar[c:c + 8] = torch.fft.ifft(X[c:c + 8] * Hh, dim=1).to(torch.complex64)

    pl = ConvPlan(gpu, N, method)
    try:
        # ---- 1. GPU gradients at h0 against the FP64 gradient
        h32 = h0.to(torch.float32)
        H = pl.spectrum(torch, K.CONV_BLOCK_SECOND, h32)
        dA = torch.empty((B, pl.block), dtype=torch.complex64, device="cuda")
        for b in range(B):
            rc = gpu.gb_execute_conv_input_async(pl.p, K.CONV_BLOCK_FIRST, dA[b].data_ptr(), x[b].data_ptr(), st)
            assert rc == 0, gpu.gb_last_error_string()
        y = torch.empty((B, N), dtype=torch.complex64, device="cuda")
        assert gpu.gb_execute_conv_output_batched(pl.p, y.data_ptr(), N, dA.data_ptr(), pl.block, H.data_ptr(), B,
                                                  st) == 0, gpu.gb_last_error_string()
        r = y - ystar
        gh = torch.full((N,), float("nan"), dtype=torch.float32, device="cuda")
        gx = torch.full((B, N), float("nan"), dtype=torch.complex64, device="cuda")
        assert gpu.gb_conv_adjoint(pl.p, gh.data_ptr(), gx.data_ptr(), N, r.data_ptr(), N, dA.data_ptr(), pl.block,
                                   H.data_ptr(), B, st) == 0, gpu.gb_last_error_string()
        torch.cuda.synchronize()
        del y, r

        H0 = torch.fft.fft(h0)
        gh_ref = torch.zeros(N, dtype=torch.complex128, device="cuda")
        gx_err2, gx_ref2 = 0.0, 0.0
        for c in range(0, B, 8):
            R = torch.fft.fft(torch.fft.ifft(X[c:c + 8] * H0, dim=1) - ystar[c:c + 8].to(torch.complex128), dim=1)
            gh_ref += (R * torch.conj(X[c:c + 8])).sum(dim=0)
            gxr = torch.fft.ifft(R * torch.conj(H0), dim=1)
            gx_err2 += float((gx[c:c + 8].to(torch.complex128) - gxr).abs().square().sum())
            gx_ref2 += float(gxr.abs().square().sum())
            del R, gxr
        gh_ref = torch.fft.ifft(gh_ref).real
        gh_rel = float(torch.linalg.norm(gh[:T].double() - gh_ref[:T]) / torch.linalg.norm(gh_ref[:T]))
        gx_rel = (gx_err2 / gx_ref2) ** 0.5
        assert gh_rel <= 1e-4, gh_rel
        assert gx_rel <= 1e-4, gx_rel

        # ---- 2. FP64 central differences of the loss
        def loss_filter(hv):
            Hv = torch.fft.fft(hv)
            tot = 0.0
            for c in range(0, B, 8):
                d = torch.fft.ifft(X[c:c + 8] * Hv, dim=1) - ystar[c:c + 8].to(torch.complex128)
                tot += 0.5 * float(d.abs().square().sum())
            return tot

        def loss_signal(b, xv):  # the one term of the sum that x_b enters
            d = torch.fft.ifft(torch.fft.fft(xv) * H0) - ystar[b].to(torch.complex128)
            return 0.5 * float(d.abs().square().sum())

        rng = np.random.default_rng(55)
        ghc = gh.cpu().numpy()
        scale_h = float(np.abs(ghc[:T]).max())
        eps = 1e-2  # the loss is quadratic: central differences carry only rounding error
        for j in rng.choice(T, 256, replace=False):
            e = torch.zeros(N, dtype=torch.float64, device="cuda")
            e[int(j)] = eps
            fd = (loss_filter(h0 + e) - loss_filter(h0 - e)) / (2 * eps)
            assert abs(fd - ghc[j]) < 1e-4 * scale_h, ("filter", int(j), fd, float(ghc[j]))
        gxc_rows = {}
        for b, n in zip(rng.integers(0, B, 256), rng.integers(0, L, 256)):
            b, n = int(b), int(n)
            if b not in gxc_rows:
                gxc_rows[b] = gx[b].cpu().numpy()
            scale_x = float(np.abs(gxc_rows[b][:L]).max())
            xb = x[b].to(torch.complex128)
            fd = 0j
            for unit in (1.0, 1j):
                e = torch.zeros(N, dtype=torch.complex128, device="cuda")
                e[n] = eps * unit
                d = (loss_signal(b, xb + e) - loss_signal(b, xb - e)) / (2 * eps)
                fd += d * unit
            assert abs(fd - gxc_rows[b][n]) < 1e-4 * scale_x, ("input", b, n, fd, gxc_rows[b][n])
        del gx

        # ---- 3. 200 descent steps on the taps, from zero
        spec_power = torch.zeros(N, dtype=torch.float64, device="cuda")
        for c in range(0, B, 8):
            spec_power += X[c:c + 8].abs().square().sum(dim=0)
        lr = 1.0 / float(spec_power.max())
        del X
        torch.cuda.empty_cache()
        h = torch.zeros(N, dtype=torch.float32, device="cuda")
        y = torch.empty((B, N), dtype=torch.complex64, device="cuda")
        losses = []
        for step in range(200):
            H = pl.spectrum(torch, K.CONV_BLOCK_SECOND, h)
            assert gpu.gb_execute_conv_output_batched(pl.p, y.data_ptr(), N, dA.data_ptr(), pl.block, H.data_ptr(),
                                                      B, st) == 0
            y.sub_(ystar)
            losses.append(0.5 * float(y.abs().square().sum(dtype=torch.float64)))
            assert gpu.gb_conv_adjoint(pl.p, gh.data_ptr(), None, 0, y.data_ptr(), N, dA.data_ptr(), pl.block,
                                       H.data_ptr(), B, st) == 0
            h[:T].sub_(lr * gh[:T])
        h_err = float(torch.linalg.norm(h[:T].double() - h_hidden[:T]) / torch.linalg.norm(h_hidden[:T]))
    finally:
        pl.free()
    floor = 1e-9 * losses[0]
    far = [i for i in range(1, len(losses)) if losses[i - 1] > floor]
    assert len(far) >= 10 and all(losses[i] < losses[i - 1] for i in far), losses[:16]
    assert losses[-1] < 1e-6 * losses[0], (losses[0], losses[-1])
    assert h_err < 1e-3, h_err
    print(f"full adjoint workload: grad rel L2 filter {gh_rel:.2e} input {gx_rel:.2e}; "
          f"loss {losses[0]:.4e} -> {losses[-1]:.4e} in 200 steps; filter error {h_err:.2e}")
