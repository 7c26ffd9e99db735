import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "isspa-force-cuda_gb300"), os.path.join(ROOT, "oracle"), ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Build the engine library and the oracle once per session."""
    import build as engine_build
    import oracle

    engine_build.build()
    oracle.build()
    yield


@pytest.fixture(scope="session")
def has_gpu(_built):
    import isspa_gb300 as ig

    return ig.abi.device_count() > 0


@pytest.fixture(autouse=True)
def _gpu_guard(request, has_gpu):
    if request.node.get_closest_marker("gpu") and not has_gpu:
        pytest.skip("no CUDA device in this process")


@pytest.fixture(scope="session")
def adi2():
    import isspa_gb300 as ig

    return ig.System.from_config(os.path.join(GOLDEN, "adi2_config.txt"))
