import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def built_lib():
    """Builds (if stale) and returns the path of libsandengine_gb300.so."""
    from sandengine_gb300.build import build
    return build()


@pytest.fixture(scope="session")
def se(built_lib):
    import sandengine_gb300
    return sandengine_gb300


def ruleset_text(name: str) -> str:
    from sandengine_gb300.workloads import ruleset_text as rt
    if name == "reference":
        with open(os.path.join(GOLDEN, "reference_materials.yaml")) as f:
            return f.read()
    return rt(name)


@pytest.fixture(scope="session")
def rulesets():
    return {n: ruleset_text(n) for n in ("reference", "four_materials", "twelve_materials")}


@pytest.fixture(scope="session")
def ports(rulesets):
    from oracle.build import Port
    return {n: Port(t) for n, t in rulesets.items()}
