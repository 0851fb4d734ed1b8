"""Build recipe of the native library (libffcz.so) and the fftz CLI.

Every translation unit is compiled by nvcc for sm_103a only, in parallel,
into ``ffcz_gb300/_build/``; nothing is installed outside the source tree.
Usage: ``python -m ffcz_gb300.build`` (or ``build()`` from Python).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
# FFCZ_BUILD_DIR / FFCZ_NVCC_FLAGS build variants (other tile or twiddle
# settings) next to the default library without touching it.
OUT = Path(os.environ.get("FFCZ_BUILD_DIR", str(PKG / "_build")))
EXTRA = os.environ.get("FFCZ_NVCC_FLAGS", "").split()
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB_SOURCES = ["solver.cu", "static_kernels.cu", "static_kernels_fc.cu", "static_kernels_tc.cu", "static_kernels_pipe.cu", "static_kernels_f64.cu", "static_kernels_f64s.cu", "huffman.cu", "decode.cu", "base.cu", "legacy_kernels.cu", "noalloc.cu", "fft_plan.cpp",
               "huffman_host.cpp", "capi_misc.cpp", "container.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _flags(src: Path) -> list[str]:
    common = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC", f"-I{ROOT / 'include'}", f"-I{CSRC}"] + EXTRA
    if src.suffix == ".cu":
        return common + ARCH + ["-lineinfo", "-Xptxas", "-warn-spills"]
    return common


def _compile(src: Path, obj: Path, verbose: bool) -> tuple[Path, str]:
    cmd = [nvcc(), "-c", str(src), "-o", str(obj)] + _flags(src)
    if verbose and src.suffix == ".cu":
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compiles libffcz.so and the fftz CLI; returns the library path."""
    OUT.mkdir(parents=True, exist_ok=True)
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((ROOT / "include").glob("*"))
    jobs = []
    objs = []
    for name in LIB_SOURCES:
        src = CSRC / name
        obj = OUT / (name + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append((src, obj))
    logs = []
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for obj, log in ex.map(lambda j: _compile(j[0], j[1], verbose), jobs):
            logs.append(log)
    lib = OUT / "libffcz.so"
    if force or jobs or not lib.exists():
        cmd = [nvcc(), "-shared", "-o", str(lib)] + [str(o) for o in objs] + ARCH + ["-ldl", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    cli_src = CSRC / "fftz_main.cu"
    cli = OUT / "fftz"
    if cli_src.exists() and (force or _stale(cli, [cli_src, lib] + headers)):
        cmd = [nvcc(), str(cli_src), "-o", str(cli), "-std=c++17", "-O2", f"-I{ROOT / 'include'}"] + ARCH + [
            f"-L{OUT}", "-lffcz", f"-Xlinker", f"-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose:
        for log in logs:
            if log.strip():
                print(log, file=sys.stderr)
    return lib


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(OUT / "libffcz.so")
