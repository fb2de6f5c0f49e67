import importlib.util
import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def load_package():
    """Import gradpower.jl_gb300/ as the package `gradpower_gb300`."""
    if "gradpower_gb300" in sys.modules:
        return sys.modules["gradpower_gb300"]
    pkg = os.path.join(ROOT, "gradpower.jl_gb300")
    spec = importlib.util.spec_from_file_location("gradpower_gb300", os.path.join(pkg, "__init__.py"),
                                                  submodule_search_locations=[pkg])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["gradpower_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def load_oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # noqa: E402
    return oracle


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


load_package()


@pytest.fixture(scope="session")
def gp():
    return load_package()


@pytest.fixture(scope="session")
def orc():
    return load_oracle()


@pytest.fixture(scope="session")
def golden_cases():
    with open(os.path.join(GOLDEN, "cases.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_known():
    with open(os.path.join(GOLDEN, "known.json")) as f:
        return json.load(f)
