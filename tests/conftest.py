"""Shared test set-up: the gpu marker, and loaders for the product binding
(171026-1-3dhlld-cyli-gal_gb300/mhdgpu.py) and the oracle (oracle/pyoracle.py)."""
import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "171026-1-3dhlld-cyli-gal_gb300")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def _load(name, path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def load_mhdgpu(build=True):
    if "mhdgpu" in sys.modules:
        return sys.modules["mhdgpu"]
    if build:
        b = _load("mhd_build", os.path.join(PKG, "build.py"))
        b.build()
    return _load("mhdgpu", os.path.join(PKG, "mhdgpu.py"))


def have_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def reference_tree_present():
    import build_ref
    return build_ref.available()


@pytest.fixture(scope="session")
def M():
    return load_mhdgpu()


@pytest.fixture(scope="session")
def P():
    import pyoracle
    pyoracle.build_oracle()
    return pyoracle
