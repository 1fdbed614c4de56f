"""Deterministic synthetic inputs shared by the tests, the bench and smoke().

SplitMix64 streams (the same integers on every machine and numpy version),
turned into float32 uniforms on [-1, 1) from the top 24 bits, and into
normals by Box-Muller in float64.
"""
from __future__ import annotations

import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, n: int, offset: int = 0) -> np.ndarray:
    with np.errstate(over="ignore"):
        i = np.arange(offset + 1, offset + n + 1, dtype=np.uint64)
        z = np.uint64(seed) * _M2 + i * _GAMMA
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, n: int, offset: int = 0) -> np.ndarray:
    """float32 uniform on [-1, 1): multiples of 2^-23."""
    top = (splitmix64(seed, n, offset) >> np.uint64(40)).astype(np.int64)
    return ((top - (1 << 23)).astype(np.float64) / float(1 << 23)).astype(np.float32)


def normal(seed: int, n: int, offset: int = 0) -> np.ndarray:
    """float32 standard normals (Box-Muller on two uniform streams)."""
    u = (splitmix64(seed, 2 * n, 2 * offset) >> np.uint64(11)).astype(np.float64) / float(1 << 53)
    u1 = np.maximum(u[0::2], 1e-300)
    u2 = u[1::2]
    return (np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)).astype(np.float32)


def complex_uniform(seed: int, n: int, offset: int = 0) -> np.ndarray:
    """complex64 with re, im i.i.d. uniform on [-1, 1)."""
    u = uniform(seed, 2 * n, 2 * offset)
    return u.view(np.complex64)


def complex_logmag(seed: int, n: int, lo: float = 1e-3, hi: float = 1e3) -> np.ndarray:
    """complex64 with log-uniform magnitude on [lo, hi) and uniform phase."""
    u = (splitmix64(seed, 2 * n) >> np.uint64(11)).astype(np.float64) / float(1 << 53)
    mag = np.exp(np.log(lo) + (np.log(hi) - np.log(lo)) * u[0::2])
    ph = 2.0 * np.pi * u[1::2]
    return (mag * np.exp(1j * ph)).astype(np.complex64)


def ragged_conv_requests(seed: int = 4, count: int = 512):
    """The ragged convolution mix: `count` requests with block size N = 2^e,
    e uniform on 8..16 (numpy Generator `seed`), exactly count/2 of them
    STEREO_MONO (a seeded permutation picks which); request i has an input of
    N/2 samples (uniform [-1, 1), complex for stereo, SplitMix64 seed
    20000 + i) and a filter of N/2 taps N(0,1) * exp(-t / (N/8)) (seed
    10000 + i).  Returns (N, stereo, input, filter) tuples."""
    rng = np.random.default_rng(seed)
    e = rng.integers(8, 17, count)
    stereo = np.zeros(count, bool)
    stereo[rng.permutation(count)[: count // 2]] = True
    reqs = []
    for i in range(count):
        N = 1 << int(e[i])
        t = np.arange(N // 2)
        h = (normal(10000 + i, N // 2) * np.exp(-t / (N / 8))).astype(np.float32)
        x = complex_uniform(20000 + i, N // 2) if stereo[i] else uniform(20000 + i, N // 2)
        reqs.append((N, bool(stereo[i]), x, h))
    return reqs


def ragged_fft_requests(seed: int = 6, count: int = 512, lo: int = 4, hi: int = 16):
    """The ragged transform mix: `count` requests with N = 2^e, e uniform on
    lo..hi (numpy Generator `seed`); the kind is c2c forward, c2c inverse, r2c
    or c2r with equal odds; a quarter of the c2c and r2c requests zero-pad the
    upper half of their input, half of the r2c requests write all N bins
    (FULL_R2C).  Request i's input (SplitMix64 seed 30000 + i) is uniform on
    [-1, 1): N complex (N/2 with zero padding) for c2c, N reals (N/2) for
    r2c, N/2 + 1 complex for c2r.  Returns (N, kind, direction, flags, input)
    tuples with the fft.h flag values."""
    rng = np.random.default_rng(seed)
    e = rng.integers(lo, hi + 1, count)
    choice = rng.integers(0, 4, count)
    zp = rng.random(count) < 0.25
    full = rng.random(count) < 0.5
    reqs = []
    for i in range(count):
        N = 1 << int(e[i])
        kind = 0 if choice[i] < 2 else int(choice[i]) - 1
        direction = 1 if choice[i] == 1 else -1
        flags = 0
        if kind != 2 and zp[i]:
            flags |= 1 << 17       # MUFFT_FLAG_ZERO_PAD_UPPER_HALF
        if kind == 1 and full[i]:
            flags |= 1 << 16       # MUFFT_FLAG_FULL_R2C
        n_in = N // 2 if flags & (1 << 17) else N
        if kind == 0:
            x = complex_uniform(30000 + i, n_in)
        elif kind == 1:
            x = uniform(30000 + i, n_in)
        else:
            x = complex_uniform(30000 + i, N // 2 + 1)
        reqs.append((N, kind, direction, flags, x))
    return reqs
