"""The reference's dense helper matrices through the C ABI (GPU): new_transition_probs,
new_transition_probs_switch and new_emissions (trans.cpp:1190-1251, emit.cpp:1288-1307)
against the reference's own outputs on the same trees (tests/golden/helpers, which the
oracle reproduces exactly: test_oracle_golden.py), in the reference's state order and in a
shuffled one.

Bars: log transition and switch entries within 1e-12 absolute (1e-12 relative in the
probability), zero probabilities (-inf) in the same places; emissions within 1e-12
relative.
"""

import os

import numpy as np
import pytest

from argweaver_gb300 import refapi
from argweaver_gb300.problem import Problem
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

NAMES = ["k8_s11", "k10_T32", "k17_missing"]


def load(name):
    d = os.path.join(GOLDEN, "helpers")
    return Problem.load(os.path.join(d, name + ".prob")), np.load(os.path.join(d, name + ".npz"))


def coal_states(prob, b):
    """get_coal_states (states.cpp:53-74): nodes in index order, each from its age to its
    parent's (the root's to ntimes - 2)."""
    par, age = prob.ptrees[b], prob.ages[b]
    return np.array([(v, t) for v in range(prob.nnodes)
                     for t in range(age[v], (prob.ntimes - 2 if par[v] == -1 else age[par[v]]) + 1)],
                    dtype=np.int32)


def assert_log_close(a, b):
    assert a.shape == b.shape
    np.testing.assert_array_equal(np.isinf(a), np.isinf(b))
    f = np.isfinite(b)
    err = float(np.max(np.abs(a[f] - b[f]))) if f.any() else 0.0
    assert err <= 1e-12, err


@pytest.mark.parametrize("name", NAMES)
def test_new_transition_probs(name):
    prob, gold = load(name)
    st = coal_states(prob, 0)
    got = refapi.new_transition_probs(prob.ptrees[0], prob.ages[0], st, prob.times,
                                      prob.popsizes, prob.rho)
    assert_log_close(got, gold["trans"])
    perm = np.random.default_rng(1).permutation(len(st))
    got = refapi.new_transition_probs(prob.ptrees[0], prob.ages[0], st[perm], prob.times,
                                      prob.popsizes, prob.rho)
    assert_log_close(got, gold["trans"][np.ix_(perm, perm)])


@pytest.mark.parametrize("name", NAMES)
def test_new_transition_probs_switch(name):
    prob, gold = load(name)
    o = 0
    rng = np.random.default_rng(2)
    for b, (S1, S2) in enumerate(gold["switch_sizes"], start=1):
        ref = gold["switch"][o:o + S1 * S2].reshape(S1, S2)
        o += S1 * S2
        s1, s2 = coal_states(prob, b - 1), coal_states(prob, b)
        args = (prob.ptrees[b], prob.ptrees[b - 1], prob.sprs[b], prob.ages[b], prob.ages[b - 1])
        got = refapi.new_transition_probs_switch(*args, s1, s2, prob.times, prob.popsizes,
                                                 prob.rho)
        assert_log_close(got, ref)
        p1, p2 = rng.permutation(S1), rng.permutation(S2)
        got = refapi.new_transition_probs_switch(*args, s1[p1], s2[p2], prob.times,
                                                 prob.popsizes, prob.rho)
        assert_log_close(got, ref[np.ix_(p1, p2)])


@pytest.mark.parametrize("name", NAMES)
def test_new_emissions(name):
    prob, gold = load(name)
    L0 = int(prob.blocklens[0])
    st = coal_states(prob, 0)
    seqs = prob.seqs[:, :L0]
    got = refapi.new_emissions(st, prob.ptrees[0], prob.ages[0], seqs, prob.times, prob.mu)
    ref = gold["emit"]
    assert got.shape == ref.shape
    assert float(np.max(np.abs(got - ref) / ref)) <= 1e-12
    perm = np.random.default_rng(3).permutation(len(st))
    got = refapi.new_emissions(st[perm], prob.ptrees[0], prob.ages[0], seqs, prob.times, prob.mu)
    assert float(np.max(np.abs(got - ref[:, perm]) / ref[:, perm])) <= 1e-12


def test_a_pair_that_is_no_state_is_an_error():
    prob, _ = load("k8_s11")
    st = coal_states(prob, 0)
    st[3] = (st[3][0], prob.ntimes)  # a time above every branch
    with pytest.raises(ValueError, match="not a coalescence state"):
        refapi.new_transition_probs(prob.ptrees[0], prob.ages[0], st, prob.times,
                                    prob.popsizes, prob.rho)
