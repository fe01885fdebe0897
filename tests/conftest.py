import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "many-lights-gi_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the CUDA kernels through the C ABI")


@pytest.fixture(scope="session", autouse=True)
def _built_libraries():
    """Build the oracle, libmlgi.so and libmlgi_checked.so once per session (no-ops when up to date)."""
    import importlib.util

    for path in (os.path.join(ROOT, "oracle", "build.py"), os.path.join(PKG, "build.py")):
        spec = importlib.util.spec_from_file_location("_b_" + os.path.basename(os.path.dirname(path)), path)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        getattr(mod, "build_all", mod.build)()
    yield


@pytest.fixture(autouse=True)
def _no_index_violations(request):
    """Under the bounds-checked library (MLGI_CHECKED=1), every GPU test must end with no index
    violation recorded by any kernel it ran."""
    yield
    if os.environ.get("MLGI_CHECKED") == "1" and request.node.get_closest_marker("gpu"):
        import mlgi

        ctx = mlgi.Context(0)
        try:
            ctx.check_device_status()
        finally:
            ctx.close()
