"""Runs the reference's known-answer tests through the C++ host mirror
(include/particular_cuda.hpp) on the GPU (tests/cpp/kat_test.cpp)."""
import subprocess

import pytest

pytestmark = pytest.mark.gpu



def test_cpp_host_mirror_kats(native_lib):
    from conftest import load_cpp_build
    exe = load_cpp_build().build()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL OK" in r.stdout
