"""kissfft_gb300::kissfft<T> (include/kissfft_cuda.hh), the reference's C++
facade (kissfft.hh) over the GPU library.

The check program tests/cxx/facade_check.cpp is compiled against the header
and the core library (CPU: it must compile and link) and run on a GPU,
where every check must stay within its bound against a long-double DFT.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def build_check(tmp_path):
    from kissfft_gb300 import build
    if not os.path.exists(build.core_lib()):
        build.build()
    exe = str(tmp_path / "facade_check")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"), "-I",
           os.path.join(CUDA, "include"), os.path.join(ROOT, "tests", "cxx", "facade_check.cpp"), "-o", exe,
           "-L", build.LIB, "-lkissfft_gb300", "-L", os.path.join(CUDA, "lib64"), "-lcudart",
           "-Wl,-rpath," + build.LIB]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_facade_compiles_and_links(tmp_path):
    assert os.path.exists(build_check(tmp_path))


@pytest.mark.gpu
def test_facade_against_direct_dft(tmp_path):
    exe = build_check(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "ALL OK" in r.stdout, r.stdout + r.stderr
