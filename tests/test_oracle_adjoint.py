"""The FP64 adjoint oracle against central finite differences of the loss
0.5 * ||conv(first, second) - target||^2 (no GPU)."""
from __future__ import annotations

import numpy as np
import pytest

from mufft_gb300 import signals
from oracle import adjoint as A


@pytest.mark.parametrize("stereo", [False, True])
def test_adjoint_oracle_matches_finite_differences(stereo):
    N, B = 64, 3
    if stereo:
        firsts = np.stack([signals.complex_uniform(500 + i, N).astype(np.complex128) for i in range(B)])
    else:
        firsts = np.stack([signals.uniform(500 + i, N).astype(np.float64) for i in range(B)])
    second = signals.uniform(510, N).astype(np.float64)
    targets = np.stack([signals.uniform(520 + i, N).astype(np.float64) for i in range(B)])
    r = np.stack([A.conv_f64(f, second, stereo) for f in firsts]) - targets
    # filter gradient: summed over the signals
    g_filter = A.adjoint_filter_f64(r, firsts)
    for j in (0, 5, N - 1):
        fd = A.finite_difference(lambda s: A.loss_f64(firsts, s, targets, stereo), second, j)
        assert abs(fd - g_filter[j]) < 1e-6 * max(1.0, abs(fd)), j
    # input gradient of signal 1
    g_in = A.adjoint_input_f64(r[1], second, stereo)
    for j in (0, 7, N - 2):
        def loss_first(f1):
            f = firsts.copy()
            f[1] = f1
            return A.loss_f64(f, second, targets, stereo)
        fd = A.finite_difference(loss_first, firsts[1], j)
        assert abs(fd - g_in[j]) < 1e-6 * max(1.0, abs(fd)), j
