import os
import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(REPO / "ipcc2021-final_gb300"))
sys.path.insert(0, str(REPO / "oracle"))
GOLDEN = REPO / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session")
def oracle():
    from oracle import Oracle
    return Oracle()


def load_golden(name):
    z = np.load(GOLDEN / name)
    out = {k: z[k] for k in z.files}
    out["dims"] = tuple(int(v) for v in out["dims"])
    out["gauge"] = [np.ascontiguousarray(g) for g in out["gauge"]]
    out["mass"] = float(out["mass"])
    return out


@pytest.fixture(scope="session")
def golden4():
    return load_golden("wilson_4x4x4x4.npz")


@pytest.fixture(scope="session")
def golden6():
    return load_golden("wilson_6x4x2x4.npz")


@pytest.fixture(scope="session")
def wd():
    import wilson_gb300
    return wilson_gb300


@pytest.fixture(scope="session")
def ctx(wd):
    c = wd.Context(0)
    yield c
    c.close()
