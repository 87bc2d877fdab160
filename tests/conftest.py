import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__ as entry  # noqa: E402


def _reference_root():
    """The reference tree's root, as the oracle's build recipe locates it
    (PGSVT_REFERENCE, else the recipe's default)."""
    spec = importlib.util.spec_from_file_location(
        "_oracle_build_paths", os.path.join(ROOT, "oracle", "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.REFERENCE_ROOT


REFERENCE = _reference_root()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def pkg():
    return entry.load_package()


@pytest.fixture(scope="session")
def oracle():
    return entry.load_oracle()


@pytest.fixture(scope="session")
def capi(pkg):
    pkg._capi.load()
    return pkg._capi


def reference_available():
    return os.path.isdir(os.path.join(REFERENCE, "src"))
