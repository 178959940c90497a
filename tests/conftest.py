import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built librast")


@pytest.fixture(scope="session")
def port():
    import oracle
    return oracle.Port()


@pytest.fixture(scope="session")
def reference():
    import oracle
    if not os.path.exists(oracle.REF_SO):
        if oracle.reference_tree() is not None:
            oracle.build(with_reference=True)
        else:
            pytest.skip("the reference sources are not present on this machine (set RAST_REFERENCE)")
    return oracle.Reference()


@pytest.fixture(scope="session")
def renderer():
    from rasteriser_gb300 import abi
    r = abi.Renderer(0)
    yield r
    r.close()
