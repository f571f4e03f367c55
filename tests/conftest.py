import glob
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


def golden_names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def load_golden(name):
    """A fixture's problem (with the model's infinite-sites penalty it ran with) and data."""
    import numpy as np

    from argweaver_gb300.problem import Problem

    prob = Problem.load(os.path.join(GOLDEN, name + ".prob"))
    gold = np.load(os.path.join(GOLDEN, name + ".npz"))
    if "infsites_penalty" in gold.files:
        prob.infsites_penalty = float(gold["infsites_penalty"])
    return prob, gold
