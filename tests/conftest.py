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
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


def golden_names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".npz"))


def load_golden(name):
    d = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    meta = json.loads(bytes(d.pop("meta")).decode())
    case = meta["case"]
    case["periodic"] = tuple(case["periodic"])
    case["length"] = tuple(case["length"])
    case["bc"] = [(t, dens, tuple(vel), ps) for t, dens, vel, ps in case["bc"]]
    case["blocks"] = {int(k): [tuple(b) for b in v] for k, v in case.get("blocks", {}).items()}
    case["bc_kinds"] = [(t, dens, tuple(vel), ps) for t, dens, vel, ps in case.get("bc_kinds", [])]
    case["bc_split"] = {int(k): tuple(v) for k, v in case.get("bc_split", {}).items()}
    d["case"] = case
    d["meta"] = meta
    d["iteration"] = int(d["scalars"][0])
    d["time"] = float(d["scalars"][1])
    d["dt"] = float(d["scalars"][2])
    return d


@pytest.fixture(scope="session")
def tslib():
    from turbostructred_gb300 import build, capi
    build.build()
    return capi.load()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build_oracle()
    return oracle
