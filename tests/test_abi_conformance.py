"""Builds tests/abi_conformance.cpp — a plain C++ client of include/helio_gb300.h, as a
Rust, cgo or JNI binding would be — against the library and runs it: the entry points
that need no GPU on CPU, the whole ABI contract on a GPU."""
import subprocess
from pathlib import Path

import pytest

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent


@pytest.fixture(scope="module")
def conformance_exe(built_library, tmp_path_factory):
    from helio_gb300 import build

    cuda_root = Path(build.nvcc()).resolve().parent.parent
    lib_dir = Path(built_library).parent
    exe = tmp_path_factory.mktemp("abi") / "abi_conformance"
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", str(HERE / "abi_conformance.cpp"), "-I", str(ROOT / "include"),
           "-I", str(cuda_root / "include"), "-L", str(lib_dir), "-lhelio_gb300", "-L", build.cuda_lib_dir(),
           "-lcudart", f"-Wl,-rpath,{lib_dir}", f"-Wl,-rpath,{build.cuda_lib_dir()}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_abi_conformance_without_gpu(conformance_exe):
    r = subprocess.run([str(conformance_exe), "cpu"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "checks passed" in r.stdout


@pytest.mark.gpu
def test_abi_conformance_on_gpu(conformance_exe):
    r = subprocess.run([str(conformance_exe), "gpu"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "FAIL" not in r.stdout
