"""The CPU restatement (oracle/) against the compiled reference's outputs.

The fixtures in tests/golden/ were produced by the reference's own threading HMM
(tests/golden/make_golden.py). The forward table must match them to 1e-13 relative
(bit-identical on the host that made them) and the sampled path exactly.

The backward pass is new (the reference has none for the threading HMM). On single-tree
problems it must equal, to 1e-12, the exact dense backward recursion over the reference's
own dense transition matrix and emissions (trans.cpp:136, emit.cpp:650), and track the
reference's log-space backward_alg (hmm.cpp:48) to 2e-3: backward_alg sums with logsum
(common.h:182-202), which drops terms more than e^-15 below the largest, so its error
grows by about S*e^-15 per column.
"""

import os

import numpy as np
import pytest

import pyoracle
from argweaver_gb300.problem import Problem
from conftest import GOLDEN, golden_names, load_golden

NAMES = golden_names()


def load(name):
    return load_golden(name)


def weights(n):
    k = np.arange(n, dtype=np.int64)
    return 1.0 + ((k * 2654435761) % 1000) / 1000.0


def column_checks(ns, fw, gold, rtol):
    off = pyoracle.offsets(ns)
    L = ns.shape[0]
    colsum = np.array([fw[off[i]:off[i + 1]].sum() for i in range(L)])
    colwsum = np.array([(fw[off[i]:off[i + 1]] * weights(off[i + 1] - off[i])).sum()
                        for i in range(L)])
    np.testing.assert_allclose(colsum, gold["colsum"], rtol=rtol, atol=0)
    np.testing.assert_allclose(colwsum, gold["colwsum"], rtol=rtol, atol=0)
    rows = np.concatenate([fw[off[i]:off[i + 1]] for i in gold["rows"]])
    np.testing.assert_allclose(rows, gold["rowvals"], rtol=rtol, atol=1e-300)


@pytest.mark.parametrize("name", NAMES)
def test_nstates(name):
    prob, gold = load(name)
    np.testing.assert_array_equal(pyoracle.nstates(prob), gold["nstates"])
    np.testing.assert_array_equal(prob.nstates_per_column(), gold["nstates"])


@pytest.mark.parametrize("name", NAMES)
def test_forward_matches_reference(name):
    prob, gold = load(name)
    fw, lnl = pyoracle.forward(prob)
    column_checks(gold["nstates"], fw, gold, rtol=1e-13)
    assert np.isfinite(lnl) and lnl < 0


@pytest.mark.parametrize("name", NAMES)
def test_traceback_matches_reference(name):
    prob, gold = load(name)
    fw, _ = pyoracle.forward(prob)
    path = pyoracle.traceback(prob, fw, gold["uniforms"])
    np.testing.assert_array_equal(path, gold["path"])


def test_rand_uniforms_match_fixture():
    # glibc's rand() after srand(seed) gives the uniforms stored with each fixture
    prob, gold = load(NAMES[0])
    u = pyoracle.rand_uniforms(int(gold["seed"]), prob.seqlen)
    np.testing.assert_array_equal(u, gold["uniforms"])


@pytest.mark.parametrize("name", [n for n in NAMES if n.startswith("single_")])
def test_backward_matches_dense_reference(name):
    prob, gold = load(name)
    bw = pyoracle.backward(prob)
    ns = gold["nstates"]
    off = pyoracle.offsets(ns)
    P = np.exp(gold["dense_trans"])
    E = np.exp(gold["dense_emit"])
    L = prob.seqlen
    exact = np.full(P.shape[0], 1.0 / P.shape[0])
    for i in range(L - 1, -1, -1):
        if i < L - 1:
            exact = P @ (E[i + 1] * exact)
            exact /= exact.sum()
        np.testing.assert_allclose(bw[off[i]:off[i + 1]], exact, rtol=1e-12, atol=0)
        d = np.exp(gold["dense_bw"][i] - gold["dense_bw"][i].max())
        d /= d.sum()
        np.testing.assert_allclose(bw[off[i]:off[i + 1]], d, rtol=2e-3, atol=0)


@pytest.mark.parametrize("name", [n for n in NAMES if n.startswith("single_")])
def test_dense_hmm_matches_reference(name):
    # the generic HMM of hmm.cpp over the reference's own dense matrix and emissions: the
    # restatement follows its operation order, so the tables and the drawn path agree
    _, gold = load(name)
    trans, emit = gold["dense_trans"], gold["dense_emit"]
    fw = pyoracle.dense_forward(trans, emit, emit[0])
    np.testing.assert_allclose(fw, gold["dense_fw"], rtol=1e-13, atol=0)
    bw = pyoracle.dense_backward(trans, emit, np.zeros(trans.shape[0]))
    np.testing.assert_allclose(bw, gold["dense_bw"], rtol=1e-13, atol=1e-300)
    L = emit.shape[0]
    u = pyoracle.rand_uniforms(int(gold["seed"]), L)  # u[L-1] drew the last column
    path = pyoracle.dense_sample(trans, gold["dense_fw"], u, int(gold["dense_path"][-1]))
    np.testing.assert_array_equal(path, gold["dense_path"])


@pytest.mark.parametrize("name", ["s37_n160", "s5_n64"])
def test_dense_hmm_random_matrices_match_reference(name):
    gold = np.load(os.path.join(GOLDEN, "densehmm", name + ".npz"))
    trans, emit = gold["dense_trans"], gold["dense_emit"]
    S = trans.shape[0]
    assert np.isinf(trans).any() or S < 10  # zero transitions reach the logsum as -inf
    fw = pyoracle.dense_forward(trans, emit, emit[0] - np.log(S))
    np.testing.assert_allclose(fw, gold["dense_fw"], rtol=1e-13, atol=0)
    bw = pyoracle.dense_backward(trans, emit, np.zeros(S))
    np.testing.assert_allclose(bw, gold["dense_bw"], rtol=1e-13, atol=1e-300)
    u = pyoracle.rand_uniforms(int(gold["seed"]), emit.shape[0])
    path = pyoracle.dense_sample(trans, gold["dense_fw"], u, int(gold["dense_path"][-1]))
    np.testing.assert_array_equal(path, gold["dense_path"])
    assert len(set(path.tolist())) > S // 2


@pytest.mark.parametrize("name", NAMES)
def test_posterior_properties(name):
    prob, gold = load(name)
    fw, _ = pyoracle.forward(prob)
    bw = pyoracle.backward(prob)
    post = pyoracle.posterior(prob, fw, bw)
    ns = gold["nstates"]
    off = pyoracle.offsets(ns)
    sums = np.add.reduceat(post, off[:-1])
    np.testing.assert_allclose(sums, 1.0, rtol=1e-12)
    assert np.all(post >= 0)
    # at the last column the backward is flat, so the posterior is the forward column
    L = prob.seqlen
    np.testing.assert_allclose(post[off[L - 1]:], fw[off[L - 1]:], rtol=1e-12, atol=1e-300)


ARGPROB = ["full_k10", "full_k24_T16", "full_k12_masked", "thread_k8"]


@pytest.mark.parametrize("name", ARGPROB)
def test_arg_probabilities_match_reference(name):
    # calc_arg_likelihood / calc_arg_prior / calc_tree_prior (total_prob.cpp), restated in
    # the reference's order: equal to its outputs on the same host
    prob = Problem.load(os.path.join(GOLDEN, "argprob", name + ".prob"))
    gold = np.load(os.path.join(GOLDEN, "argprob", name + ".npz"))
    lik, prior, tprior = pyoracle.arg_prob(prob)
    np.testing.assert_allclose(lik, gold["likelihood"], rtol=1e-13)
    np.testing.assert_allclose(prior, gold["prior"], rtol=1e-13)
    np.testing.assert_allclose(tprior, gold["tree_prior"], rtol=1e-13)
    np.testing.assert_allclose(lik + prior, gold["joint"], rtol=1e-13)



HELPERS = ["k8_s11", "k10_T32", "k17_missing"]


def load_helpers(name):
    d = os.path.join(GOLDEN, "helpers")
    return Problem.load(os.path.join(d, name + ".prob")), np.load(os.path.join(d, name + ".npz"))


def switch_matrices(gold):
    out, o = [], 0
    for S1, S2 in gold["switch_sizes"]:
        out.append(gold["switch"][o:o + S1 * S2].reshape(S1, S2))
        o += S1 * S2
    return out


@pytest.mark.parametrize("name", HELPERS)
def test_dense_helpers_match_reference(name):
    """The oracle's dense log transition and switch matrices (TransMatrix::get,
    TransMatrixSwitch::get) and its emissions against the reference's new_transition_probs,
    new_transition_probs_switch and new_emissions on the same trees: identical, zero
    probabilities (-inf) in the same places."""
    prob, gold = load_helpers(name)
    np.testing.assert_array_equal(pyoracle.dense_matrices(prob, 0), gold["trans"])
    for b, ref in enumerate(switch_matrices(gold), start=1):
        _, sw = pyoracle.dense_matrices(prob, b, switch=True)
        np.testing.assert_array_equal(sw, ref)
    S0, L0 = gold["trans"].shape[0], gold["emit"].shape[0]
    em = pyoracle.emissions(prob)[:L0 * S0].reshape(L0, S0)
    np.testing.assert_array_equal(em, gold["emit"])
    # the reference's brute-force checks of these matrices (transition and switch rows
    # against sums over SPRs, emissions against per-state Felsenstein) passed on these trees
    assert gold["self_checks"].tolist() == [1] * (len(switch_matrices(gold)) + 2)
