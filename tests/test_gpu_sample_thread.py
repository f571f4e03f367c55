"""The threading step on the GPU (arghmm_sample_thread, sample_thread.cpp:1010-1023):
forward, traceback and recombinations on the device, the thread added on the host. Bar:
after the same srand(seed), the grown ARG is the reference's (trees, SPRs, block lengths,
node mappings)."""

import glob
import os

import numpy as np
import pytest

from argweaver_gb300 import refapi
from argweaver_gb300.problem import Problem
from conftest import GOLDEN, load_golden

pytestmark = pytest.mark.gpu

NAMES = sorted(os.path.basename(p)[:-5] for p in glob.glob(os.path.join(GOLDEN, "samplethread", "*.prob")))


@pytest.mark.parametrize("name", NAMES)
def test_sample_thread_matches_reference(name):
    prob, _ = load_golden(name)
    ref = Problem.load(os.path.join(GOLDEN, "samplethread", name + ".prob"))
    refapi.srand(int(np.load(os.path.join(GOLDEN, "samplethread", name + ".npz"))["seed"]))
    out = refapi.arghmm_sample_thread(prob)
    np.testing.assert_array_equal(out.ptrees, ref.ptrees)
    np.testing.assert_array_equal(out.ages, ref.ages)
    np.testing.assert_array_equal(out.sprs[1:], ref.sprs[1:])
    np.testing.assert_array_equal(out.blocklens, ref.blocklens)
    np.testing.assert_array_equal(out.mapping[1:], ref.mapping[1:])

