"""Builds the CUDA library ``helio_gb300/_lib/libhelio_gb300.so`` for sm_103a.

Each translation unit under ``csrc/`` is compiled by nvcc in parallel
(``-gencode arch=compute_103a,code=sm_103a -lineinfo -O3``) and linked into one
shared library with a plain C ABI (include/helio_gb300.h). The library links the
shared CUDA runtime and nothing from PyTorch.

Usage: ``python -m helio_gb300.build [--force] [--verbose]``.
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
OUT_DIR = PKG / "_lib"
BUILD_DIR = PKG / "_build"
LIB_NAME = "libhelio_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = sorted(CSRC.glob("*.cu"))
HEADERS = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [ROOT / "include" / "helio_gb300.h"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build helio_gb300")


def cuda_lib_dir() -> str:
    root = Path(nvcc()).resolve().parent.parent
    for cand in (root / "lib64", root / "targets" / "sbsa-linux" / "lib", root / "targets" / "x86_64-linux" / "lib"):
        if (cand / "libcudart.so").exists() or list(cand.glob("libcudart.so*")):
            return str(cand)
    return str(root / "lib64")


def lib_path() -> Path:
    return OUT_DIR / LIB_NAME


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(src: Path, verbose: bool) -> Path:
    obj = BUILD_DIR / (src.stem + ".o")
    if not _stale(obj, [src, *HEADERS]):
        return obj
    cmd = [
        nvcc(), *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
        "-I", str(ROOT / "include"), "-c", str(src), "-o", str(obj),
    ]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        print(r.stderr, flush=True)
    return obj


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile every CUDA translation unit and link the shared library."""
    OUT_DIR.mkdir(exist_ok=True)
    BUILD_DIR.mkdir(exist_ok=True)
    if force:
        for o in BUILD_DIR.glob("*.o"):
            o.unlink()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(SOURCES), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    out = lib_path()
    if force or _stale(out, objs):
        tmp = out.with_suffix(f".{os.getpid()}.tmp")
        libdir = cuda_lib_dir()
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "shared", "-o", str(tmp), *map(str, objs),
               "-L", libdir, f"-Xlinker=-rpath,{libdir}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, out)
    return out


if __name__ == "__main__":
    p = build(force="--force" in sys.argv, verbose="--verbose" in sys.argv)
    print(p)
