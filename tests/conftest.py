import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O

    O.lib()
    return O


@pytest.fixture(scope="session")
def gpu_lib():
    """The built CUDA library; builds it in-tree if it is missing."""
    from mmo_gb300 import build, lib

    if not os.path.exists(lib.LIB_PATH):
        build.build()
    return lib.load()


@pytest.fixture(scope="session")
def scorer_factory(gpu_lib):
    from mmo_gb300.ff import UFFScorer

    made = []

    def make(prot=None, lig=None, physics=None):
        from mmo_gb300.ff import Physics

        s = UFFScorer(0, physics or Physics())
        if prot is not None:
            s.set_protein(prot)
        if lig is not None:
            s.set_ligand(lig)
        made.append(s)
        return s

    yield make
    for s in made:
        s.close()


def scaled_err(e, e64, scale):
    """|E - E64| / max(|E64|, scale): scale is the sum of |pair energies|,
    which conditions totals that cancel to near zero."""
    return abs(float(e) - float(e64)) / max(abs(float(e64)), float(scale), 1e-300)


@pytest.fixture
def rng():
    return np.random.default_rng(12345)
