import importlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = "moving-mesh-reconstruction_gb300"
for p in (ROOT, os.path.join(ROOT, PKG), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libmmh_gb300.so")


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def mmh():
    importlib.import_module(PKG)
    import mmh as M
    M.lib()
    return M


@pytest.fixture(scope="session")
def fields():
    import fields as F
    return F


def smooth_field(n, amp, seed, ns=-2.0):
    """Smooth zero-mean random field (the log of a lognormal density) scaled by amp."""
    import fields as F
    rho = F.lognormal_density(n, sigma=1.0, ns=ns, seed=seed)
    g = np.log(rho)
    g = g - g.mean()
    return np.asfortranarray(g * amp)
