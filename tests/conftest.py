import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# sources of the reference project (read only; absent where the GPU tests run)
REF_SRC = os.environ.get("LIGHTER_REF_SRC", "/root/reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the bake kernels)")


@pytest.fixture(scope="session")
def built():
    """Compile the GPU library and the CPU oracle (incremental)."""
    from lighter_gb300 import build
    build.build_library()
    build.build_oracle()
    return True


@pytest.fixture(scope="session")
def oracle(built):
    from lighter_gb300 import load_library
    return load_library(os.path.join(ROOT, "oracle", "liblighter_oracle.so"))


@pytest.fixture(scope="session")
def gpu(built):
    from lighter_gb300 import library
    return library()


@pytest.fixture(scope="session")
def ref(built):
    """The reference compiled from its own sources, where they exist."""
    from lighter_gb300 import load_library
    path = os.path.join(ROOT, "oracle", "_ref", "liblighter_ref.so")
    if not os.path.exists(path):
        pytest.skip("reference build (oracle/_ref) not available here")
    return load_library(path)


def has_cuda_device() -> bool:
    return os.path.exists("/dev/nvidia0") or os.path.exists("/dev/nvidiactl")
