"""The internal-branch resampling step's host half (sample_arg_thread_internal,
sample_thread.cpp:635-692): after srand(seed), the oracle's traceback on the first seqlen
draws (last column first) and its recombination sampler on the draws after them, regrafted
by add_arg_thread_path on the host, give the reference's whole ARG. This pins the order in
which the device step spends the draws and the regraft that follows it."""

import os

import numpy as np
import pytest

import pyoracle
from argweaver_gb300 import refapi
from conftest import GOLDEN, load_golden

NAMES = sorted(f[:-4] for f in os.listdir(os.path.join(GOLDEN, "samplethreadinternal")) if f.endswith(".npz"))


@pytest.mark.parametrize("name", NAMES)
def test_internal_step_on_the_oracle_matches_reference(name):
    prob, _ = load_golden(name)
    ref = np.load(os.path.join(GOLDEN, "samplethreadinternal", name + ".npz"))
    L = prob.seqlen
    draws = pyoracle.rand_uniforms(int(ref["seed"]), 3 * L + 2)[::-1]  # in draw order
    fw, _ = pyoracle.forward(prob)
    path = pyoracle.traceback(prob, fw, draws[:L][::-1].copy())
    pos, node, time, _ = pyoracle.sample_recombinations(prob, path, draws[L:].copy())
    got = refapi.add_arg_thread_path(prob, path, pos, node, time)
    assert got["ptrees"].shape == ref["ptrees"].shape
    for key in ("ptrees", "ages", "blocklens", "root_child0"):
        np.testing.assert_array_equal(got[key], ref[key], err_msg=key)
    np.testing.assert_array_equal(got["sprs"][1:], ref["sprs"][1:])
    np.testing.assert_array_equal(got["mapping"][1:], ref["mapping"][1:])
