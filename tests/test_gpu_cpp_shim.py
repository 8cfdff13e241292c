"""The C++ shim (include/cgx_cabana.hpp): reference-shaped p2g / g2p from C++
through libcgx, checked against the oracle inside tests/cpp/shim_parity.cpp.
The CPU test only compiles it; the GPU test links and runs it."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "shim_parity.cpp")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _cxx():
    return shutil.which("g++") or "g++"


def test_shim_header_compiles():
    subprocess.run([_cxx(), "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(CUDA, "include"), SRC], check=True)


@pytest.mark.gpu
def test_shim_parity_runs(tmp_path):
    from oracle import oracle as O
    O.lib()  # builds liboracle.so if needed
    lib_dir = os.path.join(ROOT, "cabana_gb300")
    orc_dir = os.path.join(ROOT, "oracle", "_build")
    exe = tmp_path / "shim_parity"
    subprocess.run([_cxx(), "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(CUDA, "include"), SRC, "-L", lib_dir, "-lcgx", "-L", orc_dir, "-loracle",
                    "-L", os.path.join(CUDA, "lib64"), "-lcudart", f"-Wl,-rpath,{lib_dir}:{orc_dir}",
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "OK" in out.stdout
