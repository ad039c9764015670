"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on
the CPU (oracle, generators, host logic, ABI surface)."""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "unnamed-voxel-tracer_gb300"
sys.path.insert(0, str(PKG))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


def _load(name: str, path: Path):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def vtlib():
    """The CUDA library, built in-tree if stale."""
    _load("vt_build", PKG / "build.py").build()
    import vt
    vt.load()
    return vt


@pytest.fixture(scope="session")
def oracle(vtlib):
    import oracle_py
    oracle_py.load()
    return oracle_py


@pytest.fixture(scope="session")
def ctx(vtlib):
    c = vtlib.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="session")
def vt(vtlib):
    return vtlib
