"""Shared test setup.

* registers the ``gpu`` marker (tests that need a GB300);
* loads the package from the ``dem-sphsource_gb300`` directory as
  ``dem_sphsource_gb300`` and puts the repository root on sys.path (for
  ``oracle``, the test-only checker).
"""
import importlib.util
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def load_package():
    name = "dem_sphsource_gb300"
    if name in sys.modules:
        return sys.modules[name]
    d = os.path.join(ROOT, "dem-sphsource_gb300")
    spec = importlib.util.spec_from_file_location(name, os.path.join(d, "__init__.py"),
                                                  submodule_search_locations=[d])
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built CUDA library")


@pytest.fixture(scope="session")
def ds():
    return load_package()


@pytest.fixture(scope="session")
def scenes():
    load_package()
    import dem_sphsource_gb300.scenes as s
    return s
