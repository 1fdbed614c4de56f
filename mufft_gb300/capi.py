"""ctypes mirror of the muFFT C API (fft.h) and the GB300 extensions.

`MuFFT(path, prefix)` binds any library that exports the fft.h functions
under `prefix` ("mufft_" for libmufft_gb300.so and for the reference library;
the oracle uses "oracle_").  Method names are the C names without the
prefix, with the same arguments and the same NULL-on-error behaviour, so a
test written against one library runs unchanged against the others.  The
numpy helpers at the bottom (`fft_c2c`, `fft_r2c`, ...) wrap the
create / execute / free sequence the reference's own tests use (test.c).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

FORWARD = -1
INVERSE = 1
FLAG_CPU_ANY = 0
FLAG_CPU_NO_SIMD = (1 << 16) - 1
FLAG_CPU_NO_AVX = 1 << 0
FLAG_CPU_NO_SSE3 = 1 << 1
FLAG_CPU_NO_SSE = 1 << 2
FLAG_FULL_R2C = 1 << 16
FLAG_ZERO_PAD_UPPER_HALF = 1 << 17
# mufft_gb300.h extension flags
FLAG_SPLIT_BF16X3 = 1 << 24
FLAG_SPLIT_BF16X2 = 1 << 25
FLAG_AUTOTUNE = 1 << 26
CONV_METHOD_FLAG_MONO_MONO = 0
CONV_METHOD_FLAG_STEREO_MONO = 1
CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_FIRST = 1 << 2
CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_SECOND = 1 << 3
CONV_BLOCK_FIRST = 0
CONV_BLOCK_SECOND = 1

_vp = C.c_void_p
_u = C.c_uint
_i = C.c_int
_sz = C.c_size_t

# (name, restype, argtypes) of every fft.h entry point.
FFT_H = [
    ("create_plan_1d_c2c", _vp, [_u, _i, _u]),
    ("create_plan_1d_r2c", _vp, [_u, _u]),
    ("create_plan_1d_c2r", _vp, [_u, _u]),
    ("execute_plan_1d", None, [_vp, _vp, _vp]),
    ("free_plan_1d", None, [_vp]),
    ("create_plan_conv", _vp, [_u, _u, _u]),
    ("execute_conv_input", None, [_vp, _u, _vp, _vp]),
    ("conv_get_transformed_block_size", _sz, [_vp]),
    ("execute_conv_output", None, [_vp, _vp, _vp, _vp]),
    ("free_plan_conv", None, [_vp]),
    ("create_plan_2d_c2c", _vp, [_u, _u, _i, _u]),
    ("create_plan_2d_r2c", _vp, [_u, _u, _u]),
    ("create_plan_2d_c2r", _vp, [_u, _u, _u]),
    ("execute_plan_2d", None, [_vp, _vp, _vp]),
    ("free_plan_2d", None, [_vp]),
]
MEMORY_H = [
    ("alloc", _vp, [_sz]),
    ("calloc", _vp, [_sz]),
    ("free", None, [_vp]),
    ("get_convolve_func", _vp, [_u]),
]
# mufft_gb300.h (prefix mufft_gb_)
GB_H = [
    ("last_error", _i, []),
    ("last_error_string", C.c_char_p, []),
    ("clear_error", None, []),
    ("create_plan_1d_c2c_batched", _vp, [_u, _i, _u, _u, _sz, _sz]),
    ("create_plan_1d_r2c_batched", _vp, [_u, _u, _u, _sz, _sz]),
    ("create_plan_1d_c2r_batched", _vp, [_u, _u, _u, _sz, _sz]),
    ("execute_plan_1d_async", _i, [_vp, _vp, _vp, _vp]),
    ("execute_plan_1d_launches_async", _i, [_vp, _vp, _vp, _u, _u, _vp]),
    ("execute_plan_1d_host_pipeline", _i, [_vp, _vp, _vp, _u]),
    ("execute_plan_2d_async", _i, [_vp, _vp, _vp, _vp]),
    ("execute_conv_input_async", _i, [_vp, _u, _vp, _vp, _vp]),
    ("execute_conv_output_async", _i, [_vp, _vp, _vp, _vp, _vp]),
    ("plan_1d_launches", _u, [_vp]),
    ("plan_2d_launches", _u, [_vp]),
    ("execute_plan_2d_launches_async", _i, [_vp, _vp, _vp, _u, _u, _vp]),
    ("plan_1d_describe", _i, [_vp, C.c_char_p, _sz]),
    ("plan_2d_describe", _i, [_vp, C.c_char_p, _sz]),
    ("describe_schedule_1d", _i, [_u, _i, _i, _u, _u, _vp, C.c_char_p, _sz]),
    ("describe_schedule_2d", _i, [_i, _u, _u, _i, _u, _vp, C.c_char_p, _sz]),
    ("options_init", None, [_vp]),
    ("create_plan_1d", _vp, [_i, _u, _i, _u, _u, _sz, _sz, _vp]),
    ("create_plan_2d", _vp, [_i, _u, _u, _i, _u, _vp]),
    ("create_plan_conv", _vp, [_u, _u, _u, _vp]),
    ("list_tiles", _i, [C.c_char_p, _sz]),
    ("execute_c2c_noalloc", _i, [_u, _i, _vp, _vp, _vp]),
    ("conv_adjoint_input", _i, [_vp, _vp, _vp, _vp, _vp]),
    ("conv_adjoint_filter", _i, [_vp, _vp, _vp, _sz, _vp, _sz, _u, _vp]),
    ("conv_adjoint", _i, [_vp, _vp, _vp, _sz, _vp, _sz, _vp, _sz, _vp, _u, _vp]),
    ("execute_conv_output_batched", _i, [_vp, _vp, _sz, _vp, _sz, _vp, _u, _vp]),
    ("autotune_1d", _i, [_i, _u, _i, _u, _u, _vp, _sz]),
    ("autotune_save", _i, [C.c_char_p]),
    ("autotune_load", _i, [C.c_char_p]),
    ("autotune_clear", None, []),
    ("create_stream_conv", _vp, [_u, _u, _vp, _u, _u, _vp]),
    ("stream_conv_input", _vp, [_vp]),
    ("stream_conv_output", _vp, [_vp]),
    ("stream_conv_process", _i, [_vp, _vp]),
    ("stream_conv_reset", _i, [_vp, _vp]),
    ("stream_conv_ranges", _u, [_vp]),
    ("stream_conv_fused", _i, [_vp]),
    ("stream_conv_status", _i, [_vp]),
    ("stream_conv_inject_timeout", _i, [_vp, _i]),
    ("free_stream_conv", None, [_vp]),
    ("create_conv_batch", _vp, [_vp, _u, _u, _vp]),
    ("execute_conv_batch", _i, [_vp, _vp]),
    ("conv_batch_split_size", _u, [_vp]),
    ("conv_batch_class_size", _u, [_vp]),
    ("conv_batch_status", _i, [_vp]),
    ("free_conv_batch", None, [_vp]),
    ("create_fft_batch", _vp, [_vp, _u, _u, _vp]),
    ("execute_fft_batch", _i, [_vp, _vp]),
    ("fft_batch_status", _i, [_vp]),
    ("fft_batch_describe", _i, [_vp, C.c_char_p, _sz]),
    ("free_fft_batch", None, [_vp]),
    ("device_alloc", _vp, [_sz]),
    ("device_free", None, [_vp]),
    ("memcpy", _i, [_vp, _vp, _sz]),
    ("device_synchronize", _i, []),
]

CONVOLVE_FUNC = C.CFUNCTYPE(None, _vp, _vp, _vp, C.c_float, _u)


class ConvRequest(C.Structure):
    """mufft_gb_conv_request (include/mufft_gb300.h)."""
    _fields_ = [("N", C.c_uint), ("method", C.c_uint), ("input", C.c_void_p), ("filter", C.c_void_p),
                ("output", C.c_void_p)]


class FftRequest(C.Structure):
    """mufft_gb_fft_request (include/mufft_gb300.h)."""
    _fields_ = [("N", C.c_uint), ("kind", C.c_int), ("direction", C.c_int), ("flags", C.c_uint),
                ("input", C.c_void_p), ("output", C.c_void_p)]


class TileChoice(C.Structure):
    """mufft_gb_tile_choice (include/mufft_gb300.h)."""
    _fields_ = [("L", C.c_uint), ("load_across", C.c_int), ("store_across", C.c_int),
                ("transforms_per_tile", C.c_uint), ("elems_per_thread", C.c_uint), ("cluster_ctas", C.c_uint)]


MAX_TILE_CHOICES = 8


class Options(C.Structure):
    """mufft_gb_options (include/mufft_gb300.h): per-plan schedule choices."""
    _fields_ = [("size", C.c_uint), ("multipass_levels", C.c_int), ("twiddle_table", C.c_int),
                ("fused_passes", C.c_int), ("tma", C.c_int), ("tile_occupancy", C.c_int), ("stream_tiles", C.c_int),
                ("split_engine", C.c_int), ("columns_2d", C.c_int), ("conv_split", C.c_uint),
                ("conv_classes", C.c_uint), ("stream_conv_ranges", C.c_uint), ("stream_conv_fused", C.c_int),
                ("fft_split", C.c_uint), ("ntiles", C.c_uint), ("tiles", TileChoice * MAX_TILE_CHOICES),
                ("persistent_tiles", C.c_int), ("l2_residency", C.c_int)]


class MuFFTError(RuntimeError):
    pass


def aligned_empty(shape, dtype, align: int = 64) -> np.ndarray:
    """Uninitialised numpy array whose data starts on an `align`-byte boundary
    (muFFT's contract for every buffer, fft_internal.h:38)."""
    dtype = np.dtype(dtype)
    n = int(np.prod(shape)) if np.ndim(shape) else int(shape)
    raw = np.empty(n * dtype.itemsize + align, np.uint8)
    off = (-raw.ctypes.data) % align
    return raw[off: off + n * dtype.itemsize].view(dtype).reshape(shape)


def aligned_zeros(shape, dtype) -> np.ndarray:
    a = aligned_empty(shape, dtype)
    a[...] = 0
    return a


def aligned_copy(x, dtype) -> np.ndarray:
    x = np.asarray(x, dtype=dtype)
    a = aligned_empty(x.shape, dtype)
    a[...] = x
    return a


def _ptr(a) -> int:
    """Address of a numpy array or torch tensor (or an int address)."""
    if isinstance(a, int):
        return a
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()


class MuFFT:
    """Binding of one library exporting the muFFT API under `prefix`."""

    def __init__(self, path: str | Path, prefix: str = "mufft_", gb_extensions: bool = False):
        self.path = str(path)
        self.lib = C.CDLL(self.path)
        self.prefix = prefix
        self.symbols: list[str] = []
        for name, res, args in FFT_H:
            self._bind(prefix + name, name, res, args)
        for name, res, args in MEMORY_H:
            if hasattr(self.lib, prefix + name):
                self._bind(prefix + name, name, res, args)
        self.gb = gb_extensions
        if gb_extensions:
            for name, res, args in GB_H:
                self._bind("mufft_gb_" + name, "gb_" + name, res, args)

    def _bind(self, cname: str, pyname: str, res, args):
        f = getattr(self.lib, cname)
        f.restype = res
        f.argtypes = args
        setattr(self, pyname, f)
        self.symbols.append(cname)

    # ---------------------------------------------------------- options
    def options(self, tiles=(), **fields) -> "Options":
        """mufft_gb_options with the library's defaults, then `fields` set
        (names as in the C struct); `tiles`: (L, load_across, store_across,
        transforms_per_tile, elems_per_thread, cluster_ctas) tuples."""
        o = Options()
        self.gb_options_init(C.byref(o))
        for k, v in fields.items():
            if not hasattr(o, k) or k in ("size", "tiles", "ntiles"):
                raise AttributeError(f"no option {k}")
            setattr(o, k, v)
        for i, t in enumerate(tiles):
            o.tiles[i] = TileChoice(*t)
        o.ntiles = len(tiles)
        return o

    # ----------------------------------------------------------- errors
    def check(self, what: str = "call"):
        if self.gb:
            code = self.gb_last_error()
            if code:
                msg = self.gb_last_error_string().decode()
                self.gb_clear_error()
                raise MuFFTError(f"{what}: error {code}: {msg}")

    def _plan(self, p, what):
        if not p:
            if self.gb:
                self.check(what)
            raise MuFFTError(f"{what} returned NULL")
        return p

    # ---------------------------------------------------- numpy helpers
    def _plan_1d(self, kind: int, N: int, direction: int, flags: int, opts):
        """opts: mufft_gb_options for the GB300 library (None: the fft.h creator)."""
        if opts is not None:
            return self._plan(self.gb_create_plan_1d(kind, N, direction, flags, 1, 0, 0, C.byref(opts)),
                              "gb_create_plan_1d")
        if kind == 0:
            return self._plan(self.create_plan_1d_c2c(N, direction, flags), "create_plan_1d_c2c")
        if kind == 1:
            return self._plan(self.create_plan_1d_r2c(N, flags), "create_plan_1d_r2c")
        return self._plan(self.create_plan_1d_c2r(N, flags), "create_plan_1d_c2r")

    def fft_c2c(self, x: np.ndarray, direction: int, flags: int = 0, N: int | None = None, opts=None) -> np.ndarray:
        x = aligned_copy(x, np.complex64)
        N = N or x.shape[-1]
        plan = self._plan_1d(0, N, direction, flags, opts)
        out = aligned_zeros(N, np.complex64)
        try:
            self.execute_plan_1d(plan, _ptr(out), _ptr(x))
            self.check("execute_plan_1d")
        finally:
            self.free_plan_1d(plan)
        return out

    def fft_r2c(self, x: np.ndarray, flags: int = 0, N: int | None = None, opts=None) -> np.ndarray:
        x = aligned_copy(x, np.float32)
        N = N or x.shape[-1]
        plan = self._plan_1d(1, N, FORWARD, flags, opts)
        nout = N if flags & FLAG_FULL_R2C else N // 2 + 1
        out = aligned_zeros(nout, np.complex64)
        try:
            self.execute_plan_1d(plan, _ptr(out), _ptr(x))
            self.check("execute_plan_1d")
        finally:
            self.free_plan_1d(plan)
        return out

    def fft_c2r(self, X: np.ndarray, N: int, flags: int = 0, opts=None) -> np.ndarray:
        X = aligned_copy(X, np.complex64)
        assert X.shape[-1] >= N // 2 + 1
        plan = self._plan_1d(2, N, INVERSE, flags, opts)
        out = aligned_zeros(N, np.float32)
        try:
            self.execute_plan_1d(plan, _ptr(out), _ptr(X))
            self.check("execute_plan_1d")
        finally:
            self.free_plan_1d(plan)
        return out

    def conv(self, a: np.ndarray, b: np.ndarray, N: int, method: int, flags: int = 0) -> np.ndarray:
        """Full muFFT convolution sequence: transform both blocks, multiply, inverse."""
        stereo = (method & 1) == CONV_METHOD_FLAG_STEREO_MONO
        a = aligned_copy(a, np.complex64 if stereo else np.float32)
        b = aligned_copy(b, np.float32)
        plan = self._plan(self.create_plan_conv(N, flags, method), "create_plan_conv")
        try:
            nblk = self.conv_get_transformed_block_size(plan) // 8
            b0 = aligned_zeros(nblk, np.complex64)
            b1 = aligned_zeros(nblk, np.complex64)
            out = aligned_zeros(N, np.complex64 if stereo else np.float32)
            self.execute_conv_input(plan, CONV_BLOCK_FIRST, _ptr(b0), _ptr(a))
            self.execute_conv_input(plan, CONV_BLOCK_SECOND, _ptr(b1), _ptr(b))
            self.execute_conv_output(plan, _ptr(out), _ptr(b0), _ptr(b1))
            self.check("conv")
        finally:
            self.free_plan_conv(plan)
        return out

    def _plan_2d(self, kind: int, Nx: int, Ny: int, direction: int, flags: int, opts):
        if opts is not None:
            return self._plan(self.gb_create_plan_2d(kind, Nx, Ny, direction, flags, C.byref(opts)),
                              "gb_create_plan_2d")
        if kind == 0:
            return self._plan(self.create_plan_2d_c2c(Nx, Ny, direction, flags), "create_plan_2d_c2c")
        if kind == 1:
            return self._plan(self.create_plan_2d_r2c(Nx, Ny, flags), "create_plan_2d_r2c")
        return self._plan(self.create_plan_2d_c2r(Nx, Ny, flags), "create_plan_2d_c2r")

    def fft2_c2c(self, x: np.ndarray, direction: int, flags: int = 0, opts=None) -> np.ndarray:
        """opts: mufft_gb_options for the GB300 library (None: the fft.h creator)."""
        x = aligned_copy(x, np.complex64)
        Ny, Nx = x.shape
        plan = self._plan_2d(0, Nx, Ny, direction, flags, opts)
        out = aligned_zeros((Ny, Nx), np.complex64)
        try:
            self.execute_plan_2d(plan, _ptr(out), _ptr(x))
            self.check("execute_plan_2d")
        finally:
            self.free_plan_2d(plan)
        return out

    def fft2_r2c(self, x: np.ndarray, flags: int = 0, opts=None) -> np.ndarray:
        """Returns the Ny x Nx complex output buffer (valid columns Nx/2 + 1, or Nx with FULL_R2C)."""
        x = aligned_copy(x, np.float32)
        Ny, Nx = x.shape
        plan = self._plan_2d(1, Nx, Ny, FORWARD, flags, opts)
        out = aligned_zeros((Ny, Nx), np.complex64)
        try:
            self.execute_plan_2d(plan, _ptr(out), _ptr(x))
            self.check("execute_plan_2d")
        finally:
            self.free_plan_2d(plan)
        return out

    def fft2_c2r(self, X: np.ndarray, flags: int = 0, opts=None) -> np.ndarray:
        """X: Ny x Nx complex buffer (first Nx/2 + 1 columns read); returns Ny x Nx reals."""
        X = aligned_copy(X, np.complex64)
        Ny, Nx = X.shape
        plan = self._plan_2d(2, Nx, Ny, INVERSE, flags, opts)
        out = aligned_zeros(2 * Nx * Ny, np.float32)  # the reference's scratch contract (fft.h:258-260)
        try:
            self.execute_plan_2d(plan, _ptr(out), _ptr(X))
            self.check("execute_plan_2d")
        finally:
            self.free_plan_2d(plan)
        return out[: Nx * Ny].reshape(Ny, Nx)
