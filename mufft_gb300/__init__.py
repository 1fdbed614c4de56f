"""GB300-native muFFT: the muFFT C API served by hand-written sm_103a kernels.

The product is the C-ABI library libmufft_gb300.so (include/fft.h,
include/mufft_gb300.h).  This package builds it (`build.build()`), loads it
(`load()`), and mirrors its API in Python through ctypes (`capi.MuFFT`).
There is no Python or CPU fallback: `load()` raises when the library has not
been built.
"""
from __future__ import annotations

from pathlib import Path

from .capi import *  # noqa: F401,F403  (constants and MuFFT)
from .capi import MuFFT

LIB_PATH = Path(__file__).resolve().parent / "libmufft_gb300.so"
_lib: MuFFT | None = None


def load() -> MuFFT:
    """The library binding (cached).  Raises if libmufft_gb300.so is missing."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is not built; run `python -m mufft_gb300.build` "
                "or `python -c 'import __graft_entry__ as g; g.build()'`")
        _lib = MuFFT(LIB_PATH, "mufft_", gb_extensions=True)
    return _lib
