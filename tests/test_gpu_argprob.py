"""Probabilities of a whole ARG on the GPU (arghmm_likelihood, arghmm_prior_prob,
arghmm_tree_prior_prob, arghmm_joint_prob: total_prob.cpp:315-382) through the reference's
C ABI. Bar: within 1e-12 (relative) of the reference's outputs on its own fixtures, and of
the oracle on larger ARGs (the per-site and per-tree terms are the reference's arithmetic;
only the order of the final sums differs)."""

import os

import numpy as np
import pytest

import pyoracle
from argweaver_gb300 import api, refapi
from argweaver_gb300.problem import Problem
from argweaver_gb300.sim import simulate
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

NAMES = ["full_k10", "full_k24_T16", "full_k12_masked", "thread_k8"]


@pytest.mark.parametrize("name", NAMES)
def test_arg_probabilities_match_reference(name):
    prob = Problem.load(os.path.join(GOLDEN, "argprob", name + ".prob"))
    gold = np.load(os.path.join(GOLDEN, "argprob", name + ".npz"))
    before = api.kernel_launches()
    lik = refapi.arghmm_likelihood(prob)
    assert api.kernel_launches() > before
    np.testing.assert_allclose(lik, gold["likelihood"], rtol=1e-12)
    np.testing.assert_allclose(refapi.arghmm_prior_prob(prob), gold["prior"], rtol=1e-12)
    np.testing.assert_allclose(refapi.arghmm_tree_prior_prob(prob), gold["tree_prior"],
                               rtol=1e-12)
    np.testing.assert_allclose(refapi.arghmm_joint_prob(prob), gold["joint"], rtol=1e-12)


@pytest.mark.parametrize("k,L,T,missing,seed", [(40, 20000, 20, 0.01, 5), (90, 8000, 32, 0.0, 6),
                                                (6, 30000, 16, 0.05, 7)])
def test_arg_probabilities_match_oracle(k, L, T, missing, seed):
    prob = simulate(k, L, seed, ntimes=T, missing=missing, add_thread=False)
    lik, prior, tprior = pyoracle.arg_prob(prob)
    np.testing.assert_allclose(refapi.arghmm_likelihood(prob), lik, rtol=1e-12)
    np.testing.assert_allclose(refapi.arghmm_prior_prob(prob), prior, rtol=1e-12)
    # the first-tree prior's alternating series (prob_coal_counts, total_prob.cpp:108-127)
    # cancels: with many lineages it turns the last-bit difference between CUDA's exp and
    # the host's into ~1e-11 of the result (the reference's own value carries the same
    # error), so the bar for that term at these sizes is 1e-9
    np.testing.assert_allclose(refapi.arghmm_tree_prior_prob(prob), tprior, rtol=1e-9)


def test_arg_probability_edges():
    base = simulate(6, 500, 3, add_thread=False)
    # a single-node ARG: log(.25) per site, as the reference's special case
    one = Problem(times=base.times, popsizes=base.popsizes, rho=base.rho, mu=base.mu,
                  ptrees=np.array([[-1]], dtype=np.int32), ages=np.array([[0]], dtype=np.int32),
                  sprs=np.full((1, 4), -1, dtype=np.int32), blocklens=np.array([300], dtype=np.int32),
                  seqs=base.seqs[:1, :300].copy())
    assert refapi.arghmm_likelihood(one) == np.log(.25) * 300
    # a tree whose leaves do not come first is rejected, not evaluated
    bad = Problem(**dict(base.__dict__))
    pt = bad.ptrees.copy()
    pt[0, [0, base.nnodes - 1]] = pt[0, [base.nnodes - 1, 0]]
    bad.ptrees = pt
    with pytest.raises(ValueError):
        refapi.arghmm_likelihood(bad)


@pytest.mark.parametrize("name,ext,c", [("k8", "", 10), ("k16_missing", ".gz", 4)])
def test_probabilities_of_an_arg_read_from_files(name, ext, c):
    # sites + SMC files through the host readers, then the device: the reference's values
    # for the ARG its own readers built from the same files
    from argweaver_gb300 import formats as fm
    fix = os.path.join(GOLDEN, "formats")
    ref = Problem.load(os.path.join(fix, f"{name}_c{c}.prob"))
    gold = np.load(os.path.join(fix, f"{name}_c{c}.npz"))
    prob, _ = fm.read_arg(os.path.join(fix, name + ".sites" + ext),
                          os.path.join(fix, name + ".smc" + ext), c, times=ref.times)
    np.testing.assert_allclose(refapi.arghmm_likelihood(prob), gold["likelihood"], rtol=1e-12)
    np.testing.assert_allclose(refapi.arghmm_prior_prob(prob), gold["prior"], rtol=1e-12)
    np.testing.assert_allclose(refapi.arghmm_joint_prob(prob), gold["joint"], rtol=1e-12)
