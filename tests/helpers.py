"""Shared helpers for the test suite: golden fixtures and error metrics."""
from __future__ import annotations

from functools import lru_cache
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden" / "golden.npz"

# Parity bar of the GPU path against the reference / oracle:
# relative L2 error <= 1e-5 for c2c, r2c, c2r and convolution.
REL_L2_TOL = 1e-5


@lru_cache(maxsize=1)
def golden() -> dict[str, np.ndarray]:
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


def golden_cases(prefix: str) -> list[str]:
    """Case names (without the /in, /c, /simd suffix) under `prefix`."""
    g = golden()
    return sorted({k.rsplit("/", 1)[0] for k in g if k.startswith(prefix + "/") and k.endswith("/in")})


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.complex128 if np.iscomplexobj(a) or np.iscomplexobj(b) else np.float64)
    b = np.asarray(b, dtype=a.dtype)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def max_abs(a, b) -> float:
    return float(np.max(np.abs(np.asarray(a, np.complex128) - np.asarray(b, np.complex128)))) if np.size(a) else 0.0


def bitwise_equal(a, b) -> bool:
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    if a.shape != b.shape or a.dtype != b.dtype:
        return False
    return bool(np.array_equal(a, b))


def direct_conv_f64(a, b, N: int):
    """Circular convolution of length N in FP64 by the O(N^2) sum (the role of
    the reference's test.c:375-403, in double precision)."""
    a = np.zeros(N, np.complex128) + np.pad(np.asarray(a, np.complex128), (0, N - len(a)))
    b = np.pad(np.asarray(b, np.float64), (0, N - len(b)))
    out = np.zeros(N, np.complex128)
    for k in range(N):
        out += a[k] * np.roll(b, k)
    return out
