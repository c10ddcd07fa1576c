import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "3bem_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Compile the oracle (and the library when missing) once per session."""
    from oracle import oracle
    oracle.build()
    lib = os.path.join(ROOT, "3bem_gb300", "lib", "libtbem_gpu.so")
    if not os.path.exists(lib):
        import importlib.util
        spec = importlib.util.spec_from_file_location(
            "tbem_build", os.path.join(ROOT, "3bem_gb300", "build.py"))
        m = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(m)
        m.build()
    yield
