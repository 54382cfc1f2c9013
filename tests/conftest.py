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


@pytest.fixture(scope="session")
def digest8(wd):
    """The 8^3x16 fixture: digests of the reference's outputs plus its seeded
    inputs regenerated with the package's host generator."""
    z = np.load(GOLDEN / "wilson_8x8x8x16_digest.npz")
    d = {k: z[k] for k in z.files}
    dims = tuple(int(v) for v in d["dims"])
    d["dims"] = dims
    d["mass"] = float(d["mass"])
    d["stride"] = int(d["stride"])
    d["gauge"] = wd.gen_gauge(dims, seed=int(d["gauge_seed"]), eps=float(d["eps"]))
    d["src"] = wd.gen_source(dims, seed=int(d["source_seed"]))
    return d


def digest_error(d, name, v) -> float:
    """Largest of the relative errors of v's L2 norm and of its sampled
    entries against the fixture's digest of `name`."""
    ref = d[f"{name}_sample"]
    e_sample = np.linalg.norm(v[::d["stride"]] - ref) / np.linalg.norm(ref)
    e_norm = abs(np.linalg.norm(v) - float(d[f"{name}_norm"])) / float(d[f"{name}_norm"])
    return float(max(e_sample, e_norm))
