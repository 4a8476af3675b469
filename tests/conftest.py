"""Shared test set-up: the `gpu` marker, and loaders for the package (its
folder name, elpaso-core_gb300, is not an identifier) and for the oracle."""
import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


def load_package():
    name = "elpaso_core_gb300"
    if name in sys.modules:
        return sys.modules[name]
    path = os.path.join(ROOT, "elpaso-core_gb300", "__init__.py")
    spec = importlib.util.spec_from_file_location(name, path, submodule_search_locations=[os.path.dirname(path)])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def elp():
    return load_package()


@pytest.fixture(scope="session")
def meshes(elp):
    import importlib
    return importlib.import_module("elpaso_core_gb300.meshes")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as orc
    return orc


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "elements.npz")))
