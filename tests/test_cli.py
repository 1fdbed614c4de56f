"""The muFFT-style command-line benchmark (mufft_gb300/cli/mufft_bench.c):
it builds, keeps bench.c's argument contract, and prints the reference
library's lines next to its own when MUFFT_REFERENCE_LIB is set."""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

import pytest

from mufft_gb300.build import build_cli

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def cli():
    return str(build_cli())


def test_usage_matches_reference_contract(cli):
    for args in (["1"], ["1", "2", "3", "4"]):
        r = subprocess.run([cli, *args], capture_output=True, text=True)
        assert r.returncode == 1 and "Usage:" in r.stderr and "[iterations] [Nx] [Ny]" in r.stderr


def test_one_size_lines(cli):
    env = dict(os.environ)
    ref = ROOT / "oracle" / "_ref" / "libmufft_ref.so"
    if ref.exists():
        env["MUFFT_REFERENCE_LIB"] = str(ref)
    r = subprocess.run([cli, "20", "256"], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    assert any(l.startswith("muFFT-GB300 C2C:") and "000256" in l for l in lines)
    assert any(l.startswith("muFFT-GB300 conv stereo:") for l in lines)
    if ref.exists():
        c2c = [l for l in lines if l.startswith("muFFT C2C:")]
        assert c2c and "Mflops" in c2c[0]
    r = subprocess.run([cli, "5", "64", "32"], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0
    assert any("0064 by 0032" in l for l in r.stdout.splitlines())


@pytest.mark.gpu
def test_gpu_lines_report_mflops(cli):
    r = subprocess.run([cli, "200", "4096"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    for tag in ("muFFT-GB300 C2C:", "muFFT-GB300 device C2C:", "muFFT-GB300 R2C-C2R:"):
        line = [l for l in r.stdout.splitlines() if l.startswith(tag)]
        assert line and "Mflops" in line[0] and "unavailable" not in line[0], r.stdout
