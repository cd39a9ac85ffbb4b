import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "threephotons.jl_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden_sh():
    with open(os.path.join(GOLDEN, "sh_values.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def config1():
    d = np.load(os.path.join(GOLDEN, "config1.npz"))
    out = {k: d[k] for k in d.files}
    out["params"] = json.loads(str(d["params"]))
    return out


@pytest.fixture(scope="session")
def config1_hist(config1):
    from tp3.structure import loadHistograms
    return loadHistograms(config1["counts"].astype(np.float64), config1["params"]["K"])
