import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def pma_lib():
    from porousmediaanalysis_gb300 import build, capi
    build.build()
    return capi.lib()


@pytest.fixture(scope="session")
def ctx(pma_lib):
    import torch
    import porousmediaanalysis_gb300 as pma
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    c = pma.Context(0)
    c.set_throat_numbering(reference=True)  # parity: the reference's own shared-type ids
    yield c
    c.close()


@pytest.fixture(scope="session")
def ref_cases():
    import json
    with open(os.path.join(GOLDEN, "ref_cases.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def example_golden():
    import json
    with open(os.path.join(GOLDEN, "example.json")) as f:
        return json.load(f)
