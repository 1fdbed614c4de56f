"""Python loader for the oracle (and, where it was built, the reference).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py -- never by the mufft_gb300 package.

  load_oracle()     -> MuFFT binding of oracle/_build/libmufft_oracle.so, the
                       C restatement of the reference's scalar path (compiled
                       here on demand with gcc; works on x86 and Arm)
  load_reference()  -> MuFFT binding of oracle/_ref/libmufft_ref.so, the
                       reference library compiled from its own sources by
                       oracle/build_ref.sh, or None where it was not built
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

import sys
sys.path.insert(0, str(Path(__file__).resolve().parent.parent))
from mufft_gb300.capi import MuFFT  # noqa: E402

HERE = Path(__file__).resolve().parent
ORACLE_SRC = HERE / "mufft_oracle.c"
ORACLE_SO = HERE / "_build" / "libmufft_oracle.so"
REF_SO = HERE / "_ref" / "libmufft_ref.so"


def build_oracle(force: bool = False) -> Path:
    if ORACLE_SO.exists() and not force and ORACLE_SO.stat().st_mtime >= ORACLE_SRC.stat().st_mtime:
        return ORACLE_SO
    ORACLE_SO.parent.mkdir(exist_ok=True)
    tmp = ORACLE_SO.with_suffix(f".so.{os.getpid()}")
    cmd = [os.environ.get("CC", "gcc"), "-std=c99", "-O3", "-fPIC", "-ffp-contract=off", "-shared",
           "-pthread", "-o", str(tmp), str(ORACLE_SRC), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


class Oracle(MuFFT):
    def __init__(self):
        super().__init__(build_oracle(), "oracle_")
        f = self.lib.oracle_plan_1d_steps
        f.restype = C.c_uint
        f.argtypes = [C.c_void_p, C.POINTER(C.c_uint), C.POINTER(C.c_uint), C.c_uint]
        f = self.lib.oracle_execute_plan_1d_many
        f.restype = None
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint, C.c_size_t, C.c_size_t, C.c_uint]
        f = self.lib.oracle_dft_f64
        f.restype = None
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_uint, C.c_int]
        f = self.lib.oracle_convolve
        f.restype = None
        f.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_uint]

    def steps(self, N: int, direction: int, flags: int = 0) -> list[tuple[int, int]]:
        """(radix, p) of each pass the greedy planner picks (fft.c:325-379)."""
        plan = self.create_plan_1d_c2c(N, direction, flags)
        if not plan:
            raise ValueError(f"no plan for N={N}")
        r = (C.c_uint * 32)()
        p = (C.c_uint * 32)()
        n = self.lib.oracle_plan_1d_steps(plan, r, p, 32)
        self.free_plan_1d(plan)
        return [(r[i], p[i]) for i in range(n)]

    def dft_f64(self, x: np.ndarray, direction: int) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.complex128)
        out = np.zeros_like(x)
        self.lib.oracle_dft_f64(out.ctypes.data, x.ctypes.data, x.size, direction)
        return out

    def c2c_many(self, x: np.ndarray, direction: int, threads: int, flags: int = 0) -> np.ndarray:
        """Batched c2c over rows of x on `threads` host threads."""
        x = np.ascontiguousarray(x, dtype=np.complex64)
        B, N = x.shape
        out = np.empty_like(x)
        plan = self.create_plan_1d_c2c(N, direction, flags)
        self.lib.oracle_execute_plan_1d_many(plan, out.ctypes.data, x.ctypes.data, B, N * 8, N * 8, threads)
        self.free_plan_1d(plan)
        return out


_oracle: Oracle | None = None


def load_oracle() -> Oracle:
    global _oracle
    if _oracle is None:
        _oracle = Oracle()
    return _oracle


def load_reference() -> MuFFT | None:
    if not REF_SO.exists():
        return None
    return MuFFT(REF_SO, "mufft_")
