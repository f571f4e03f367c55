"""get_state_spaces (states.cpp:228-251): each tree's external states, node index order and
times from the node's age to its parent's (the root's to ntimes - 2); the counts are
arghmm_get_nstates', and the states are those the forward tables are laid out by (the
oracle's per-tree state counts)."""

import numpy as np
import pytest

import pyoracle
from argweaver_gb300 import refapi
from conftest import load_golden


@pytest.mark.parametrize("name", ["dsmc_k8_s11", "dsmc_k10_T16", "sim1_c20"])
def test_state_spaces(name):
    prob, _ = load_golden(name)
    spaces = refapi.get_state_spaces(prob)
    ns = pyoracle.nstates(prob)
    starts = np.concatenate([[0], np.cumsum(prob.blocklens)[:-1]])
    assert [len(s) for s in spaces] == [int(ns[i]) for i in starts]
    for b, st in enumerate(spaces):
        par, age = prob.ptrees[b], prob.ages[b]
        want = [(i, t) for i in range(prob.nnodes)
                for t in range(age[i], (prob.ntimes - 2 if par[i] == -1 else age[par[i]]) + 1)]
        assert [tuple(x) for x in st.tolist()] == want


@pytest.mark.parametrize("name", ["cut_k10_s3", "large_cut_k50_s19"])
def test_internal_state_counts_follow_the_root_child_order(name):
    """arghmm_get_nstates(internal=True) on a trees handle that keeps each root's child[0]
    (the cut subtree): the oracle's per-column counts, the layout of every internal table
    the C ABI returns."""
    prob, _ = load_golden(name)
    assert prob.internal
    trees = refapi.LocalTrees(prob.normalized())
    try:
        got = refapi.get_nstates(trees, prob.ntimes, True, prob.seqlen)
    finally:
        trees.close()
    np.testing.assert_array_equal(np.maximum(got, 0), pyoracle.nstates(prob))
