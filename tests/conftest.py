import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds on CPU")


def load_golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


class GoldenPartition:
    """Partition record in the shape NetworkLikelihood expects."""

    def __init__(self, d):
        self.tip_states = np.array(d["tip_states"], dtype=np.uint32)
        self.weights = np.array(d["weights"], dtype=np.float64)
        self.freqs = np.array(d["freqs"], dtype=np.float64)
        self.exch = np.array(d["exch"], dtype=np.float64)
        self.alpha = float(d["alpha"])
        self.states = int(d.get("states", 4))
        self.rate_cats = 4


def golden_cases():
    ref = load_golden("reference_cases.json")["cases"]
    syn = load_golden("synthetic_cases.json")["cases"]
    pro = load_golden("protein_cases.json")["cases"]
    return ref + syn + pro


@pytest.fixture(scope="session")
def cases():
    return golden_cases()
