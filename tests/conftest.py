"""Shared test set-up: import paths, the `gpu` marker, builds of the oracle and the library."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "ark-cpp-mpi_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "tests", "golden")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def port():
    """The C restatement of the reference step (built on first use)."""
    import oracle

    oracle.build(port=True, ref=False)
    return oracle


@pytest.fixture(scope="session")
def ark():
    """The GPU library's ctypes binding (built on first use; loads without a GPU)."""
    import ark_build

    ark_build.build()
    import arkgpu

    arkgpu.lib()
    return arkgpu


@pytest.fixture(autouse=True)
def _bounds_checked_build_clean(request):
    """Under the bounds-checked library (ARK_GPU_LIB pointing at lib_check/), every GPU test also
    asserts that its kernels recorded no out-of-range index (ark_bounds_check)."""
    yield
    if not os.environ.get("ARK_GPU_LIB") or "gpu" not in request.keywords:
        return
    import arkgpu

    # ARK_GPU_LIB names the bounds-checked build: an ordinary library there (status 6) fails too
    hits, value, bound, line = arkgpu.bounds_check(reset=True)
    assert hits == 0, f"{hits} out-of-range kernel indices; first {value} (bound {bound}) at csrc line {line}"
