"""Builds the C++ known-answer test program (tests/cpp/kat_test.cpp) against the
in-tree libparticular_cuda.so, into tests/cpp/_build/kat_test."""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "_build", "kat_test")
LIB_DIR = os.path.join(ROOT, "particular_gb300", "lib")


def build(force=False):
    src = os.path.join(HERE, "kat_test.cpp")
    deps = [src, os.path.join(ROOT, "include", "particular_cuda.hpp"),
            os.path.join(ROOT, "include", "particular_cuda.h")]
    if (not force and os.path.exists(OUT)
            and all(os.path.getmtime(d) <= os.path.getmtime(OUT) for d in deps)):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-Wall", "-Wextra",
           f"-I{os.path.join(ROOT, 'include')}", src, "-o", OUT, f"-L{LIB_DIR}",
           "-lparticular_cuda", f"-Wl,-rpath,{LIB_DIR}"]
    subprocess.check_call(cmd)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
