"""FP64 oracle of the convolution adjoints (test infrastructure only).

The reference has no adjoint: its convolution is the forward product
out = (1/N) IFFT(FFT(first) . FFT(second)) (fft.c:794-809, kernel.c:22-34).
These functions restate that product and its two gradients in float64
numpy, and check them against central finite differences of the loss
0.5 * ||conv(first, second) - target||^2, so the GPU adjoints are pinned to
the mathematics rather than to another implementation.

Conventions: `first` is real (MONO_MONO) or complex (STEREO_MONO), `second`
is real; complex gradients are dL/dRe + i dL/dIm.
"""
from __future__ import annotations

import numpy as np


def conv_f64(first: np.ndarray, second: np.ndarray, stereo: bool) -> np.ndarray:
    """Circular convolution of length N = len(first) (both blocks N long)."""
    a = np.asarray(first, np.complex128 if stereo else np.float64)
    b = np.asarray(second, np.float64)
    y = np.fft.ifft(np.fft.fft(a) * np.fft.fft(b))
    return y if stereo else y.real


def adjoint_input_f64(grad_output: np.ndarray, second: np.ndarray, stereo: bool) -> np.ndarray:
    """d/d first of <grad_output, conv(first, second)>: (1/N) IFFT(G conj(B))."""
    g = np.asarray(grad_output, np.complex128)
    b = np.asarray(second, np.float64)
    y = np.fft.ifft(np.fft.fft(g) * np.conj(np.fft.fft(b)))
    return y if stereo else y.real


def adjoint_filter_f64(grad_outputs: np.ndarray, firsts: np.ndarray) -> np.ndarray:
    """d/d second summed over signals: Re (1/N) IFFT(sum_b G_b conj(A_b))."""
    g = np.asarray(grad_outputs, np.complex128)
    a = np.asarray(firsts, np.complex128)
    s = (np.fft.fft(g, axis=-1) * np.conj(np.fft.fft(a, axis=-1))).reshape(-1, g.shape[-1]).sum(axis=0)
    return np.fft.ifft(s).real


def loss_f64(firsts: np.ndarray, second: np.ndarray, targets: np.ndarray, stereo: bool) -> float:
    r = np.stack([conv_f64(f, second, stereo) for f in np.atleast_2d(firsts)]) - np.atleast_2d(targets)
    return 0.5 * float(np.sum(np.abs(r) ** 2))


def finite_difference(fn, x: np.ndarray, index: int, eps: float = 1e-6) -> complex | float:
    """Central difference of scalar fn at x[index] (d/dRe + i d/dIm for complex x)."""
    x = np.array(x, copy=True)
    flat = x.reshape(-1)
    base = flat[index]
    flat[index] = base + eps
    up = fn(x)
    flat[index] = base - eps
    dn = fn(x)
    flat[index] = base
    d = (up - dn) / (2 * eps)
    if np.iscomplexobj(x):
        flat[index] = base + 1j * eps
        up = fn(x)
        flat[index] = base - 1j * eps
        dn = fn(x)
        flat[index] = base
        d = d + 1j * (up - dn) / (2 * eps)
    return d
