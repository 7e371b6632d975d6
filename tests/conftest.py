"""Shared fixtures: the package under test (loaded from its directory, whose
name is not a Python identifier) and the CPU oracle."""
import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "lagrangianvoronoi.jl_gb300")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))


def load_package():
    if "lvgpu" in sys.modules:
        return sys.modules["lvgpu"]
    spec = importlib.util.spec_from_file_location("lvgpu", os.path.join(PKG_DIR, "__init__.py"),
                                                  submodule_search_locations=[PKG_DIR])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["lvgpu"] = mod
    spec.loader.exec_module(mod)
    return mod


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built liblvgpu.so")


@pytest.fixture(scope="session")
def lv():
    mod = load_package()
    from importlib import import_module
    build = import_module("lvgpu.build")
    build.build()
    return mod


@pytest.fixture(scope="session")
def oracle():
    import lvref
    lvref.build()
    return lvref
