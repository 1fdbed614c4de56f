"""C-ABI checks that need no GPU: the library loads, exports exactly what
include/*.h declares, validates arguments like the reference, and plans the
GPU schedule on the host."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import pytest

import mufft_gb300
from mufft_gb300 import capi as K

ROOT = Path(__file__).resolve().parents[1]


def _has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def declared_functions() -> set[str]:
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(mufft_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


@pytest.fixture(scope="module")
def lib():
    return mufft_gb300.load()


def test_library_exports_every_declared_symbol(lib):
    declared = declared_functions()
    assert len(declared) >= 38
    for name in sorted(declared):
        assert hasattr(lib.lib, name), f"{name} declared in include/ but not exported"


def test_reference_api_complete(lib):
    # Every function of the reference fft.h (fft.h:86-297) is present.
    ref_api = {"mufft_create_plan_1d_c2c", "mufft_create_plan_1d_r2c", "mufft_create_plan_1d_c2r",
               "mufft_execute_plan_1d", "mufft_free_plan_1d", "mufft_create_plan_conv",
               "mufft_execute_conv_input", "mufft_conv_get_transformed_block_size",
               "mufft_execute_conv_output", "mufft_free_plan_conv", "mufft_get_convolve_func",
               "mufft_create_plan_2d_c2c", "mufft_create_plan_2d_r2c", "mufft_create_plan_2d_c2r",
               "mufft_execute_plan_2d", "mufft_free_plan_2d", "mufft_alloc", "mufft_calloc", "mufft_free"}
    assert ref_api <= declared_functions()
    for name in ref_api:
        assert hasattr(lib.lib, name)


def test_constants_match_reference():
    h = (ROOT / "include" / "fft.h").read_text()
    want = {"MUFFT_FORWARD": "(-1)", "MUFFT_INVERSE": "(1)", "MUFFT_FLAG_CPU_ANY": "(0)",
            "MUFFT_FLAG_CPU_NO_SIMD": "((1 << 16) - 1)", "MUFFT_FLAG_FULL_R2C": "(1 << 16)",
            "MUFFT_FLAG_ZERO_PAD_UPPER_HALF": "(1 << 17)",
            "MUFFT_CONV_METHOD_FLAG_STEREO_MONO": "1",
            "MUFFT_CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_FIRST": "(1 << 2)",
            "MUFFT_CONV_METHOD_FLAG_ZERO_PAD_UPPER_HALF_SECOND": "(1 << 3)",
            "MUFFT_CONV_BLOCK_SECOND": "1"}
    for k, v in want.items():
        m = re.search(rf"#define {k}\s+(.+)", h)
        assert m and m.group(1).strip() == v, k


def test_extension_flags_match_header():
    h = (ROOT / "include" / "mufft_gb300.h").read_text()
    for name, val in (("MUFFT_GB_FLAG_SPLIT_BF16X3", K.FLAG_SPLIT_BF16X3),
                      ("MUFFT_GB_FLAG_SPLIT_BF16X2", K.FLAG_SPLIT_BF16X2)):
        m = re.search(rf"#define {name}\s+\(1u << (\d+)\)", h)
        assert m and (1 << int(m.group(1))) == val, name
    # no overlap with the reference's flag bits (fft.h:52-65)
    assert K.FLAG_SPLIT_BF16X3 & (K.FLAG_CPU_NO_SIMD | K.FLAG_FULL_R2C | K.FLAG_ZERO_PAD_UPPER_HALF) == 0


def test_split_precision_schedule_and_rejections(lib):
    buf = C.create_string_buffer(4096)
    for N, limbs, flag in ((4096, 3, K.FLAG_SPLIT_BF16X3), (256, 2, K.FLAG_SPLIT_BF16X2)):
        mma_sync = lib.options(split_engine=1)  # one CTA per 4096 points
        assert lib.gb_describe_schedule_1d(N, 0, K.FORWARD, flag, 65536, C.byref(mma_sync), buf, 4096) == 0
        d = buf.value.decode()
        assert d.startswith(f"split_tc N={N} bf16x{limbs} mma.sync"), d
        assert f"grid={65536 * N // 4096}" in d, d
        # tcgen05 (the default): persistent, two CTAs per SM
        assert lib.gb_describe_schedule_1d(N, 0, K.FORWARD, flag, 65536, None, buf, 4096) == 0
        d = buf.value.decode()
        assert d.startswith(f"split_tc N={N} bf16x{limbs} tcgen05 grid=304"), d
    bad = lib.options(split_engine=2)
    assert lib.gb_describe_schedule_1d(4096, 0, K.FORWARD, K.FLAG_SPLIT_BF16X3, 1, C.byref(bad), buf, 4096) == -1
    lib.gb_clear_error()
    for N, kind, flags in ((1024, 0, K.FLAG_SPLIT_BF16X3), (4096, 1, K.FLAG_SPLIT_BF16X3),
                           (4096, 0, K.FLAG_SPLIT_BF16X2 | K.FLAG_ZERO_PAD_UPPER_HALF)):
        assert lib.gb_describe_schedule_1d(N, kind, K.FORWARD, flags, 1, None, buf, 4096) == -2, (N, kind, flags)
        lib.gb_clear_error()


def test_autotune_argument_checks(lib, tmp_path):
    buf = C.create_string_buffer(256)
    assert lib.gb_autotune_1d(3, 1024, K.FORWARD, 0, 1, buf, 256) == -1
    lib.gb_clear_error()
    assert lib.gb_autotune_1d(0, 1000, K.FORWARD, 0, 1, buf, 256) == -1  # not a power of two
    lib.gb_clear_error()
    assert lib.gb_autotune_1d(0, 4096, K.FORWARD, K.FLAG_SPLIT_BF16X3, 1, buf, 256) == -2
    lib.gb_clear_error()
    assert lib.gb_autotune_load(str(tmp_path / "missing").encode()) == -1
    junk = tmp_path / "junk.txt"
    junk.write_text("not a cache\n")
    assert lib.gb_autotune_load(str(junk).encode()) == -1
    lib.gb_clear_error()
    lib.gb_autotune_clear()
    if not _has_gpu():
        assert lib.gb_autotune_1d(0, 1 << 20, K.FORWARD, 0, 1, buf, 256) == -3
        lib.gb_clear_error()
    # the autotune flag alone changes nothing in a described schedule
    assert _sched(lib, 1 << 20, 0, flags=K.FLAG_AUTOTUNE) == _sched(lib, 1 << 20, 0)


def test_stream_conv_validates_on_host(lib):
    import numpy as np
    h = np.ones(10, np.float32)
    for block, taps in ((1000, 10), (1, 10), (256, 0)):
        assert not lib.gb_create_stream_conv(block, 0, h.ctypes.data, taps, 0, None)
        assert lib.gb_last_error() == -1
        lib.gb_clear_error()
    assert not lib.gb_stream_conv_input(None) and not lib.gb_stream_conv_output(None)
    assert lib.gb_stream_conv_process(None, None) == -1
    lib.gb_clear_error()
    lib.gb_free_stream_conv(None)


def test_null_frees_are_noops(lib):
    lib.free_plan_1d(None)
    lib.free_plan_2d(None)
    lib.free_plan_conv(None)
    lib.free(None)


@pytest.mark.parametrize("N", [0, 1, 3, 12, 1000])
def test_invalid_sizes_rejected(lib, N):
    assert not lib.create_plan_1d_c2c(N, K.FORWARD, 0)
    assert lib.gb_last_error() == -1  # MUFFT_GB_ERR_INVALID, decided before any device use
    lib.gb_clear_error()
    assert not lib.create_plan_1d_r2c(N, 0)
    assert not lib.create_plan_conv(N, 0, 0)
    assert not lib.create_plan_2d_c2c(N, 4, K.FORWARD, 0)
    lib.gb_clear_error()


def test_reference_edge_rejections(lib):
    # r2c/c2r need N >= 4 (the inner complex transform of N/2 = 1 fails).
    for f in (lib.create_plan_1d_r2c, lib.create_plan_1d_c2r):
        assert not f(2, 0)
        assert lib.gb_last_error() == -1
        lib.gb_clear_error()
    assert not lib.create_plan_1d_c2c(64, 0, 0)  # direction must be +-1
    assert lib.gb_last_error() == -1
    assert not lib.create_plan_2d_r2c(2, 8, 0)
    lib.gb_clear_error()


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device path")
def test_valid_plan_without_gpu_reports_no_device(lib):
    assert not lib.create_plan_1d_c2c(1024, K.FORWARD, 0)
    assert lib.gb_last_error() == -3  # MUFFT_GB_ERR_NO_DEVICE
    lib.gb_clear_error()


def test_conv_batch_validates_requests_on_host(lib):
    """Request checks run before any device work (no GPU needed)."""
    fake = 0x10000
    cases = [(1000, 0, (fake, fake, fake), -1), (1 << 18, 0, (fake, fake, fake), -2),
             (16, 0, (fake, fake, fake), -2), (1 << 17, K.CONV_METHOD_FLAG_STEREO_MONO, (fake, fake, fake), -2),
             (1024, 0, (fake, None, fake), -1)]
    for N, method, ptrs, code in cases:
        reqs = (K.ConvRequest * 1)(K.ConvRequest(N, method, *ptrs))
        assert not lib.gb_create_conv_batch(reqs, 1, 0, None)
        assert lib.gb_last_error() == code, (N, method)
        lib.gb_clear_error()
    assert not lib.gb_create_conv_batch(None, 0, 0, None)
    assert lib.gb_last_error() == -1
    lib.gb_clear_error()
    lib.gb_free_conv_batch(None)


def _sched(lib, N, kind, direction=K.FORWARD, flags=0, batch=1, opts=None):
    buf = C.create_string_buffer(4096)
    rc = lib.gb_describe_schedule_1d(N, kind, direction, flags, batch, C.byref(opts) if opts else None, buf, 4096)
    assert rc == 0, (rc, lib.gb_last_error_string())
    return buf.value.decode()


def test_single_pass_schedule(lib):
    s = _sched(lib, 1024, 0, batch=4096)  # one transform per tile
    assert s.count("tile") == 1 and "L=1024 R=16 C=1 " in s and "grid=4096x1" in s, s
    s = _sched(lib, 4096, 0, K.INVERSE)
    assert "conj=3" in s
    s = _sched(lib, 8192, 1, flags=K.FLAG_ZERO_PAD_UPPER_HALF)
    assert "L=4096" in s and "+half" in s and "epi=r2c" in s
    s = _sched(lib, 8192, 2)
    assert "pro=c2r" in s


def test_multipass_schedules(lib):
    parts = _sched(lib, 1 << 24, 0, opts=lib.options(multipass_levels=2)).split("; ")
    assert len(parts) == 2
    assert "L=4096" in parts[0] and "across/across" in parts[0] and "epi=twiddle" in parts[0]
    assert "L=4096" in parts[1] and "along/across" in parts[1]
    parts = _sched(lib, 1 << 24, 0, opts=lib.options(multipass_levels=3, fused_passes=0)).split("; ")
    assert len(parts) == 3
    assert all("L=256" in p for p in parts)
    assert "epi=twiddle" in parts[0] and "epi=twiddle" in parts[1]
    assert "along/across" in parts[2] and "grid=16x256" in parts[2]
    parts = _sched(lib, 1 << 24, 0, opts=lib.options(multipass_levels=3, fused_passes=1)).split("; ")
    assert len(parts) == 2 and "L=256" in parts[0] and parts[1].startswith("fused_bc")
    assert "blocks=16 ring=4" in parts[1]
    buf = C.create_string_buffer(64)
    bad = lib.options(multipass_levels=5)
    assert lib.gb_describe_schedule_1d(1 << 24, 0, K.FORWARD, 0, 1, C.byref(bad), buf, 64) == -1
    lib.gb_clear_error()
    s = _sched(lib, 1 << 21, 1)  # r2c of 2^21 reals = 2^20 complex + in-place fix-up
    assert s.split("; ")[-1].startswith("r2c_fixup")


def test_schedule_options_in_dry_runs(lib):
    """Resident-CTA caps pad the tile launches' shared memory; streaming row
    tiles run as a persistent grid (both measured slower on GB300, off by
    default); options apply to the one call they are passed to."""
    s = _sched(lib, 1024, 0, batch=4096, opts=lib.options(tile_occupancy=2))
    assert "smem=115712" in s, s          # (233472 / 2 - 1024) rounded to 128 bytes
    s = _sched(lib, 1024, 0, batch=4096, opts=lib.options(stream_tiles=1))
    assert "tile+stream" in s and "grid=152x1" in s, s
    s = _sched(lib, 1024, 0, batch=4096)
    assert "+stream" not in s and "smem=8704" in s, s
    s = _sched(lib, 1024, 0, batch=4096, opts=lib.options(tiles=[(1024, 0, 0, 4, 16, 1)]))
    assert "L=1024 R=16 C=4 " in s and "grid=1024x1" in s and "smem=34816" in s, s
    # 4096-point column tiles (one 1024-thread CTA per SM) run as a persistent
    # grid by default; the other tiles keep one launch per tile
    s = _sched(lib, 1 << 24, 0, opts=lib.options(multipass_levels=2))
    first, second = s.split("; ")
    assert first.startswith("tile+persistent L=4096 R=16 C=4") and "grid=152x1" in first, s
    assert "+persistent" not in second, s
    s = _sched(lib, 1 << 24, 0, opts=lib.options(multipass_levels=2, persistent_tiles=0))
    assert "+persistent" not in s and "grid=1024x1" in s, s
    assert "+persistent" not in _sched(lib, 1 << 24, 0)


def test_options_struct_layout_matches_the_header(lib):
    """mufft_gb_options_init writes sizeof(mufft_gb_options) into `size`:
    the ctypes mirror has the same size, and the fields after the tile choices
    (appended later) land where the library reads them."""
    o = K.Options()
    lib.gb_options_init(C.byref(o))
    assert o.size == C.sizeof(K.Options)
    assert (o.persistent_tiles, o.l2_residency, o.fft_split, o.ntiles) == (-1, -1, 8192, 0)


def _sched2d(lib, kind, Nx, Ny, opts=None):
    buf = C.create_string_buffer(4096)
    rc = lib.gb_describe_schedule_2d(kind, Nx, Ny, K.FORWARD, 0, C.byref(opts) if opts else None, buf, 4096)
    assert rc == 0, (rc, lib.gb_last_error_string())
    return buf.value.decode().split("; ")


def test_2d_schedules_without_a_gpu(lib):
    """2D schedules: one-row row tiles; 4096-row columns as one persistent
    pass, or -- for real grids at least 4096 wide (c2c: 8192) with the L2
    hints, and from 8192 rows always -- as a two-pass four-step of 64-column
    tiles whose intermediates stay in L2 (D: dropped once read)."""
    rows, c1, c2 = _sched2d(lib, 1, 4096, 4096)
    assert rows.startswith("tile L=2048 R=16 C=1 ") and "epi=r2c" in rows and rows.endswith("l2=FL")
    assert "L=64 R=16 C=64" in c1 and "by_row" in c1 and c1.endswith("l2=L")
    assert "L=64 R=16 C=64" in c2 and c2.endswith("l2=SD")
    c1, c2, rows = _sched2d(lib, 2, 4096, 4096)
    assert c1.endswith("l2=FL") and c2.endswith("l2=LD") and "pro=c2r" in rows and rows.endswith("l2=SD")
    rows, col = _sched2d(lib, 0, 4096, 4096)  # c2c at 4096 wide: one persistent column pass
    assert col.startswith("tile+persistent L=4096 R=16 C=4")
    rows, col = _sched2d(lib, 1, 2048, 4096)
    assert col.startswith("tile+persistent L=4096") and rows.startswith("tile L=1024 R=16 C=1 ")
    assert len(_sched2d(lib, 1, 4096, 4096, lib.options(columns_2d=1))) == 2
    assert len(_sched2d(lib, 1, 4096, 4096, lib.options(l2_residency=0))) == 2
    assert len(_sched2d(lib, 0, 1024, 8192)) == 3
    buf = C.create_string_buffer(64)
    assert lib.gb_describe_schedule_2d(1, 3, 4, K.FORWARD, 0, None, buf, 64) == -1
    lib.gb_clear_error()
    assert lib.gb_describe_schedule_2d(5, 4, 4, K.FORWARD, 0, None, buf, 64) == -1
    lib.gb_clear_error()


def test_l2_residency_hints_in_schedules(lib):
    """Multi-pass intermediates carry L2 cache-policy hints by default: the
    first pass streams its input and keeps its output (F, L), the last drops
    the intermediate once read and streams its output (D, S; no S before an
    r2c fix-up, which reads that output); single passes carry none."""
    a, b, c = _sched(lib, 1 << 24, 0).split("; ")
    assert a.endswith("l2=FL") and b.endswith("l2=L") and c.endswith("l2=SD"), (a, b, c)
    p1, p2, fix = _sched(lib, 1 << 21, 1).split("; ")
    assert p1.endswith("l2=FL") and p2.endswith("l2=D") and fix.startswith("r2c_fixup"), (p1, p2)
    assert "l2=" not in _sched(lib, 1 << 24, 0, opts=lib.options(l2_residency=0))
    assert "l2=" not in _sched(lib, 4096, 0, batch=64)
    buf = C.create_string_buffer(64)
    for v in (2, -2):
        o = lib.options(l2_residency=v)
        assert lib.gb_describe_schedule_1d(1024, 0, K.FORWARD, 0, 1, C.byref(o), buf, 64) == -1
        lib.gb_clear_error()
    buf = C.create_string_buffer(64)
    for bad in (dict(tile_occupancy=-1), dict(tile_occupancy=33), dict(stream_tiles=2), dict(stream_conv_fused=3),
                dict(stream_conv_ranges=1 << 21), dict(conv_split=1000), dict(twiddle_table=3), dict(tma=3),
                dict(columns_2d=3), dict(persistent_tiles=2), dict(persistent_tiles=-2)):
        o = lib.options(**bad)
        assert lib.gb_describe_schedule_1d(1024, 0, K.FORWARD, 0, 1, C.byref(o), buf, 64) == -1, bad
        lib.gb_clear_error()
    o = lib.options(tiles=[(1024, 0, 0, 3, 0, 0)])  # no such tile
    assert lib.gb_describe_schedule_1d(1024, 0, K.FORWARD, 0, 1, C.byref(o), buf, 64) == -1
    lib.gb_clear_error()
    o = lib.options()
    o.size = 4  # not initialised by mufft_gb_options_init
    assert lib.gb_describe_schedule_1d(1024, 0, K.FORWARD, 0, 1, C.byref(o), buf, 64) == -1
    lib.gb_clear_error()
    d = lib.options()
    assert (d.multipass_levels, d.twiddle_table, d.conv_split, d.conv_classes, d.stream_conv_fused,
            d.persistent_tiles, d.l2_residency) == (0, -1, 65536, 16384, 1, -1, -1)


def test_batched_convolution_entry_points_validate_on_host(lib):
    assert lib.gb_execute_conv_output_batched(None, None, 0, None, 0, None, 1, None) == -1
    lib.gb_clear_error()
    assert lib.gb_conv_adjoint(None, None, None, 0, None, 0, None, 0, None, 1, None) == -1
    lib.gb_clear_error()
    assert lib.gb_stream_conv_ranges(None) == 0 and lib.gb_stream_conv_fused(None) == 0
    assert lib.gb_stream_conv_status(None) == -1
    lib.gb_clear_error()


def test_fft_batch_validates_requests_on_host(lib):
    """Request checks run before any device work (no GPU needed)."""
    fake = 0x10000
    cases = [(1000, 0, -1, 0, fake, fake, -1),          # not a power of two
             (2, 1, -1, 0, fake, fake, -1),             # real kinds need N >= 4
             (1024, 3, -1, 0, fake, fake, -1),          # no such kind
             (1024, 0, 0, 0, fake, fake, -1),           # c2c direction
             (1024, 0, -1, 1 << 24, fake, fake, -1),    # flag the batch does not take
             (1024, 0, -1, 0, fake + 4, fake, -1),      # misaligned input
             (1024, 0, -1, 0, None, fake, -1),
             (1 << 17, 0, -1, 0, fake, fake, -2),       # c2c longer than 65536
             (1 << 18, 1, -1, 0, fake, fake, -2)]       # r2c longer than 131072
    for N, kind, direction, flags, pin, pout, code in cases:
        reqs = (K.FftRequest * 1)(K.FftRequest(N, kind, direction, flags, pin, pout))
        assert not lib.gb_create_fft_batch(reqs, 1, 0, None)
        assert lib.gb_last_error() == code, (N, kind, direction, flags)
        lib.gb_clear_error()
    assert not lib.gb_create_fft_batch(None, 0, 0, None)
    assert lib.gb_last_error() == -1
    lib.gb_clear_error()
    bad = lib.options(fft_split=4096)
    reqs = (K.FftRequest * 1)(K.FftRequest(1024, 0, -1, 0, fake, fake))
    assert not lib.gb_create_fft_batch(reqs, 1, 0, C.byref(bad))
    assert lib.gb_last_error() == -1
    lib.gb_clear_error()
    assert lib.gb_execute_fft_batch(None, None) == -1
    assert lib.gb_fft_batch_status(None) == -1
    lib.gb_clear_error()
    lib.gb_free_fft_batch(None)


def test_host_pipeline_validates_on_host(lib):
    assert lib.gb_execute_plan_1d_host_pipeline(None, None, None, 0) == -1
    lib.gb_clear_error()
