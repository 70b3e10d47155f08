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
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


GOLDEN_SETS = ["toy", "c1_small", "zipf_long", "edge_080", "edge_090"]


def load_golden(name):
    sets = []
    with open(os.path.join(GOLDEN, f"{name}.sets.txt")) as f:
        for line in f:
            line = line.strip()
            if line:
                sets.append([int(x) for x in line.split()])
    sizes = np.array([len(s) for s in sets], dtype=np.uint32)
    tokens = np.array([t for s in sets for t in s], dtype=np.uint32)
    starts = np.zeros(len(sets), dtype=np.uint32)
    if len(sets):
        starts[1:] = np.cumsum(sizes[:-1])
    with open(os.path.join(GOLDEN, f"{name}.json")) as f:
        results = json.load(f)["results"]
    return tokens, starts, sizes, {float(k): v for k, v in results.items()}


@pytest.fixture(scope="session")
def golden():
    return {name: load_golden(name) for name in GOLDEN_SETS}


@pytest.fixture(scope="session")
def ctx():
    import hyset_gb300 as hs
    c = hs.Context(0)
    yield c
    c.close()
