"""The C++ mirror (include/refrakt.hpp) compiles against the C ABI and runs the reference's call
pattern: host part here, the walker pool and draw on a GPU."""
import os
import subprocess

import pytest

from conftest import ROOT


def _build(rk, tmp_path):
    exe = str(tmp_path / "host_api")
    lib_dir = os.path.dirname(rk.LIB_PATH)
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include",
           os.path.join(ROOT, "tests", "cpp", "host_api.cpp"), "-o", exe, "-L", lib_dir, "-lrefrakt_gb300",
           "-L", "/usr/local/cuda/lib64", "-lcudart", "-Wl,-rpath," + lib_dir]
    subprocess.run(cmd, check=True)
    return exe


def test_cpp_client_host(rk, tmp_path):
    exe = _build(rk, tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr


@pytest.mark.gpu
def test_cpp_client_gpu(rk, tmp_path):
    exe = _build(rk, tmp_path)
    r = subprocess.run([exe, "--gpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr
