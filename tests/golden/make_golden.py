"""Generates tests/golden/golden.npz with the reference muFFT library itself.

Run in a checkout that has the reference sources (it compiles them with
oracle/build_ref.sh into oracle/_ref/ first):

    python tests/golden/make_golden.py [reference_dir]

Every case stores its input and the reference's output for the portable C
tier (flags | MUFFT_FLAG_CPU_NO_SIMD, the only tier an Arm host has), and on
x86 also the output of the default SIMD tier.  Inputs come from
mufft_gb300.signals, so they are reproducible without the file.  The cases
follow the sweeps of the reference's test.c:490-579, capped at N = 1024
(1D) and 64 x 64 (2D) to keep the fixture small; larger sizes are compared
live against the oracle.
"""
from __future__ import annotations

import platform
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from mufft_gb300 import capi as K  # noqa: E402
from mufft_gb300 import signals  # noqa: E402

OUT = Path(__file__).resolve().parent / "golden.npz"


def main():
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py REFERENCE_SOURCE_DIR")
    ref_dir = sys.argv[1]
    subprocess.run([str(ROOT / "oracle" / "build_ref.sh"), ref_dir], check=True)
    from oracle.oracle import load_reference
    ref = load_reference()
    x86 = platform.machine().lower() in ("x86_64", "amd64")
    tiers = [("c", K.FLAG_CPU_NO_SIMD)] + ([("simd", 0)] if x86 else [])
    d: dict[str, np.ndarray] = {}
    seed = 100

    def put(name, inp, fn, inp2=None):
        d[name + "/in"] = inp
        if inp2 is not None:
            d[name + "/in2"] = inp2
        for tier, fl in tiers:
            d[name + "/" + tier] = fn(fl)

    sizes_1d = [2 ** e for e in range(1, 11)]
    for N in sizes_1d:
        seed += 1
        x = signals.complex_uniform(seed, N)
        for dirn in (K.FORWARD, K.INVERSE):
            put(f"c2c/N{N}/d{dirn}/zp0", x, lambda fl: ref.fft_c2c(x, dirn, fl))
            xh = x[: N // 2].copy()
            put(f"c2c/N{N}/d{dirn}/zp1", xh,
                lambda fl: ref.fft_c2c(xh, dirn, fl | K.FLAG_ZERO_PAD_UPPER_HALF, N))
        if N < 4:
            continue
        xr = signals.uniform(seed + 5000, N)
        for full in (0, K.FLAG_FULL_R2C):
            put(f"r2c/N{N}/full{int(bool(full))}/zp0", xr, lambda fl: ref.fft_r2c(xr, fl | full))
            xrh = xr[: N // 2].copy()
            put(f"r2c/N{N}/full{int(bool(full))}/zp1", xrh,
                lambda fl: ref.fft_r2c(xrh, fl | full | K.FLAG_ZERO_PAD_UPPER_HALF, N))
        X = signals.complex_uniform(seed + 6000, N // 2 + 1)
        X[0] = X[0].real
        X[N // 2] = X[N // 2].real
        put(f"c2r/N{N}", X, lambda fl: ref.fft_c2r(X, N, fl))
        for method in (0, 1, 12, 13):
            stereo = method & 1
            a = signals.complex_uniform(seed + 7000, N) if stereo else signals.uniform(seed + 7000, N)
            b = signals.uniform(seed + 8000, N)
            if method & 4:
                a = a[: N // 2].copy()
            if method & 8:
                b = b[: N // 2].copy()
            put(f"conv/N{N}/m{method}", a, lambda fl: ref.conv(a, b, N, method, fl), inp2=b)

    for Nx, Ny in [(2, 2), (4, 2), (2, 8), (8, 8), (16, 4), (32, 64), (64, 16), (4, 64)]:
        seed += 1
        x = signals.complex_uniform(seed, Nx * Ny).reshape(Ny, Nx)
        for dirn in (K.FORWARD, K.INVERSE):
            put(f"c2c2d/{Nx}x{Ny}/d{dirn}", x, lambda fl: ref.fft2_c2c(x, dirn, fl))
    for Nx, Ny in [(4, 2), (4, 4), (8, 16), (32, 8), (64, 32), (16, 2), (64, 64)]:
        seed += 1
        x = signals.uniform(seed, Nx * Ny).reshape(Ny, Nx)
        for full in (0, K.FLAG_FULL_R2C):
            vx = Nx if full else Nx // 2 + 1
            put(f"r2c2d/{Nx}x{Ny}/full{int(bool(full))}", x,
                lambda fl: ref.fft2_r2c(x, fl | full)[:, :vx].copy())
        X = signals.complex_uniform(seed + 9000, Nx * Ny).reshape(Ny, Nx)
        put(f"c2r2d/{Nx}x{Ny}", X, lambda fl: ref.fft2_c2r(X, fl))

    np.savez_compressed(OUT, **d)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes, {len(d)} arrays)")


if __name__ == "__main__":
    main()
