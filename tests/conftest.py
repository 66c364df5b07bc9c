import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import build, oracle as O
    build.build()
    return O


@pytest.fixture(scope="session")
def native_lib():
    """The native library, built if needed (nvcc cross-compiles without a GPU)."""
    from particular_gb300 import build_native, _native
    build_native.build()
    return _native.lib()


@pytest.fixture(scope="session")
def res(native_lib):
    """A CUDA context on device 0 (GPU tests only)."""
    from particular_gb300 import CudaResources
    r = CudaResources(0)
    yield r
    r.close()


def load_cpp_build():
    """tests/cpp/build.py, loaded by path (it builds the C++ KAT program)."""
    import importlib.util
    path = os.path.join(ROOT, "tests", "cpp", "build.py")
    spec = importlib.util.spec_from_file_location("pt_cpp_kat_build", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod
