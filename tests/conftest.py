"""Shared test setup: the `gpu` marker, and loaders for the engine package
(its directory name is not a Python identifier) and for the oracle."""
from __future__ import annotations

import importlib.util
import pathlib
import sys

import pytest

REPO = pathlib.Path(__file__).resolve().parent.parent


def load_engine():
    if "pito_codecs_gb300" in sys.modules:
        return sys.modules["pito_codecs_gb300"]
    pkg = REPO / "pito-codecs_gb300"
    spec = importlib.util.spec_from_file_location("pito_codecs_gb300", pkg / "__init__.py",
                                                  submodule_search_locations=[str(pkg)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["pito_codecs_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


def load_oracle():
    if "pyoracle" in sys.modules:
        return sys.modules["pyoracle"]
    spec = importlib.util.spec_from_file_location("pyoracle", REPO / "oracle" / "pyoracle.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules["pyoracle"] = mod
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the engine's kernels")


@pytest.fixture(scope="session")
def engine():
    return load_engine()


@pytest.fixture(scope="session")
def oracle():
    return load_oracle()


@pytest.fixture(scope="session")
def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
