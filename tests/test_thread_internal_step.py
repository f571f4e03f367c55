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
from argweaver_gb300.problem import Problem
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


def test_cut_then_rethread_chain_on_the_oracle():
    """The Gibbs step's internal-branch move end to end on the host: a uniform removal path,
    the cut, the cut ARG as an internal problem (the oracle accepts it and threads it), the
    regraft of the sampled thread; the ARG is whole again and covers the region."""
    full = Problem.load(os.path.join(GOLDEN, "addthread", "dsmc_k8_s12.prob"))
    refapi.srand(77)
    path, _ = refapi.sample_arg_removal_path_uniform(full)
    cut = refapi.as_problem(full, refapi.remove_arg_thread_path(full, path), internal=True)
    L = cut.seqlen
    draws = pyoracle.rand_uniforms(78, 3 * L + 2)[::-1]
    fw, _ = pyoracle.forward(cut)
    thread = pyoracle.traceback(cut, fw, draws[:L][::-1].copy())
    pos, node, time, _ = pyoracle.sample_recombinations(cut, thread, draws[L:].copy())
    arg = refapi.add_arg_thread_path(cut, thread, pos, node, time)
    roots = np.argmax(arg["ptrees"] == -1, axis=1)
    assert np.all((arg["ptrees"] == -1).sum(axis=1) == 1)
    assert np.all(arg["ages"][np.arange(len(roots)), roots] < full.ntimes)  # no virtual root
    assert int(arg["blocklens"].sum()) == int(np.sum(full.blocklens))
    # and the regrown ARG is again a whole ARG over the same leaves: its tree lengths and
    # state spaces are well formed
    again = refapi.as_problem(full, arg)
    assert again.nnodes == full.nnodes
    assert all(len(s) > 0 for s in refapi.get_state_spaces(again))
