import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")
CASES = ["lj864", "ljatm864", "atmlist500", "fene375", "edge_box", "atm2b864", "thermo864", "ibi864"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built engine")


def load_case(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def case_system(z):
    from komd_gb300 import lattice
    return lattice.System(r=z["r0"].copy(), v=z["v0"].copy(), m=z["m"], eps=z["eps"], sig=z["sig"],
                          mol_id=z["mol_id"], low=z["low"], high=z["high"])


@pytest.fixture(scope="session")
def oracle_lib():
    import pyoracle
    pyoracle.build()
    return pyoracle
