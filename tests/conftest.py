"""Shared fixtures: markers, the oracle, and paired GPU / oracle models."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libssgb300.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def ss():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import streamsculptor_gb300 as ss
    ss._abi.load()
    return ss


G = 4.498502151469553e-12

# C1 workload: NFW + Miyamoto-Nagai + Hernquist, progenitor at present day
MW3 = dict(nfw=(5.4e11, 15.62), mn=(6.8e10, 3.0, 0.28), hern=(5e9, 1.0))
PROG_WF = np.array([12.0, 0.0, 4.0, 0.0, 0.18, 0.04])


def mw3_gpu(ss):
    from streamsculptor_gb300 import potential as P
    u = ss.usys
    return P.Potential_Combine([P.NFWPotential(m=5.4e11, r_s=15.62, units=u),
                                P.MiyamotoNagaiDisk(m=6.8e10, a=3.0, b=0.28, units=u),
                                P.HernquistPotential(m=5e9, r_s=1.0, units=u)], units=u)


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))
