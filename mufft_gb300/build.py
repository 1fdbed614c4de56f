"""Builds libmufft_gb300.so in-tree with nvcc for sm_103a.

Every translation unit under csrc/ is compiled in parallel into
mufft_gb300/_build/ and linked into mufft_gb300/libmufft_gb300.so (the CUDA
runtime is linked statically, so the library only needs the driver).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
INCLUDE = PKG.parent / "include"
BUILD = PKG / "_build"
LIB = PKG / "libmufft_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", f"-I{INCLUDE}", f"-I{CSRC}"]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    raise RuntimeError("nvcc not found (set CUDA_HOME or put nvcc on PATH)")


def sources() -> list[Path]:
    return sorted(p for p in CSRC.iterdir() if p.suffix in (".cu", ".cpp"))


def _compile(src: Path, verbose: bool) -> tuple[Path, str]:
    obj = BUILD / (src.stem + ".o")
    deps = [src, *CSRC.glob("*.h"), *CSRC.glob("*.cuh"), *INCLUDE.glob("*.h")]
    if obj.exists() and obj.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return obj, ""
    cmd = [nvcc(), *ARCH, *COMMON, "-c", str(src), "-o", str(obj)]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr[:4000]}")
    return obj, res.stderr


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    BUILD.mkdir(exist_ok=True)
    srcs = sources()
    jobs = jobs or min(len(srcs), max(1, os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for (o, log), s in zip(results, srcs):
            if log:
                print(f"== {s.name}\n{log}", file=sys.stderr)
    newest = max(o.stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-Xlinker", f"--version-script={CSRC / 'exports.map'}",
               "-o", str(tmp), *map(str, objs)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
    return LIB


CLI_SRC = PKG / "cli" / "mufft_bench.c"
CLI = PKG / "mufft-bench"


def build_cli() -> Path:
    """The muFFT-style command-line benchmark (plain C against the library)."""
    lib = build()
    deps = [CLI_SRC, lib, *INCLUDE.glob("*.h")]
    if CLI.exists() and CLI.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return CLI
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("no C compiler for the command-line benchmark")
    cmd = [cc, "-O2", "-std=c11", "-D_POSIX_C_SOURCE=200809L", f"-I{INCLUDE}", str(CLI_SRC), "-o", str(CLI),
           f"-L{PKG}", "-lmufft_gb300", f"-Wl,-rpath,{PKG}", "-ldl", "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"mufft-bench build failed:\n{res.stdout}\n{res.stderr[:4000]}")
    return CLI


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
    print(build_cli())
