import importlib.util
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built sm_103a library")


def load_package():
    """Import the package directory ``qdk-chemistry_gb300`` as ``qdk_chemistry_gb300``."""
    name = "qdk_chemistry_gb300"
    if name in sys.modules:
        return sys.modules[name]
    pkg_dir = os.path.join(ROOT, "qdk-chemistry_gb300")
    spec = importlib.util.spec_from_file_location(name, os.path.join(pkg_dir, "__init__.py"),
                                                  submodule_search_locations=[pkg_dir])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def pkg():
    return load_package()


@pytest.fixture(scope="session")
def oracle():
    import oracle as orc
    orc.build()
    return orc


@pytest.fixture(scope="session")
def known():
    with open(os.path.join(GOLDEN, "known_answers.json")) as f:
        return json.load(f)


def load_fcidump(name):
    pkg = load_package()
    d = np.load(os.path.join(GOLDEN, name + "_fcidump.npz"))
    return pkg.integrals.integrals_from_lines(int(d["norb"]), d["idx"], d["vals"], int(d["nelec"]), int(d["ms2"]))


@pytest.fixture(scope="session")
def h2o():
    return load_fcidump("h2o_ccpvdz")


@pytest.fixture(scope="session")
def n2_6e6o():
    return load_fcidump("n2_6e6o")


@pytest.fixture(scope="session")
def n2_14e18o():
    return load_fcidump("n2_14e18o")
