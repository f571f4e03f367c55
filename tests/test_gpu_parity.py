"""Parity of the CUDA path with the oracle and the reference (GPU only).

Bars:
  FP64 forward table        <= 1e-12 relative to the oracle, per cell, and to the
                             reference's column checksums in tests/golden
  sampled path (FP64)       identical to the reference's, given the same uniforms
  posterior marginals FP64  <= 1e-10 relative to the oracle's forward-backward
  log-likelihood            <= 1e-12 relative to the oracle
  FP32 posterior            <= 1e-5 absolute (max over cells) of the FP64 posterior
The reference-compatible entry points (arghmm_forward_alg, arghmm_sample_posterior, ...)
are exercised through the same ctypes prototypes the reference declares.
"""

import os

import numpy as np
import pytest

import pyoracle
from argweaver_gb300 import api, refapi
from argweaver_gb300.problem import Problem
from argweaver_gb300.sim import simulate
from conftest import GOLDEN, golden_names, load_golden

pytestmark = pytest.mark.gpu

NAMES = golden_names()
EXTERNAL_DEFAULT_MAP = [n for n in NAMES if n.startswith(("dsmc_", "single_"))]


def load(name):
    return load_golden(name)


def weights(n):
    k = np.arange(n, dtype=np.int64)
    return 1.0 + ((k * 2654435761) % 1000) / 1000.0


def max_rel(a, b, floor=1e-300):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))


@pytest.mark.parametrize("name", NAMES)
def test_forward_fp64_matches_oracle_and_reference(name):
    prob, gold = load(name)
    r = api.run_batch([prob])[0]
    fw_o, lnl_o = pyoracle.forward(prob)
    assert r.forward.shape == fw_o.shape
    assert max_rel(r.forward, fw_o) <= 1e-12
    assert abs(r.loglik - lnl_o) <= 1e-12 * abs(lnl_o)
    ns = gold["nstates"]
    off = pyoracle.offsets(ns)
    colsum = np.add.reduceat(r.forward, off[:-1])
    np.testing.assert_allclose(colsum, gold["colsum"], rtol=1e-12)
    colw = np.array([(r.forward[off[i]:off[i + 1]] * weights(off[i + 1] - off[i])).sum()
                     for i in range(prob.seqlen)])
    np.testing.assert_allclose(colw, gold["colwsum"], rtol=1e-12)
    rows = np.concatenate([r.forward[off[i]:off[i + 1]] for i in gold["rows"]])
    np.testing.assert_allclose(rows, gold["rowvals"], rtol=1e-12, atol=1e-300)


@pytest.mark.parametrize("name", NAMES)
def test_sampled_path_matches_reference(name):
    prob, gold = load(name)
    path = api.sample_path(prob, uniforms=gold["uniforms"])
    np.testing.assert_array_equal(path, gold["path"])


@pytest.mark.parametrize("name", NAMES)
def test_posterior_fp64_matches_oracle(name):
    prob, _ = load(name)
    post = api.posterior(prob)
    fw, _ = pyoracle.forward(prob)
    bw = pyoracle.backward(prob)
    ref = pyoracle.posterior(prob, fw, bw)
    big = ref > 1e-200
    assert max_rel(post[big], ref[big]) <= 1e-10
    assert np.max(np.abs(post - ref)) <= 1e-14


@pytest.mark.parametrize("name", NAMES)
def test_fp32_close_to_fp64(name):
    prob, _ = load(name)
    r32, r64 = (api.run_batch([prob], precision=p, want_posterior=True)[0]
                for p in ("fp32", "fp64"))
    assert np.max(np.abs(r32.posterior - r64.posterior)) <= 1e-5
    assert abs(r32.loglik - r64.loglik) <= 1e-5 * abs(r64.loglik)


@pytest.mark.parametrize("k,seed", [(59, 11), (31, 12), (63, 13)])
def test_fp32_close_to_fp64_long(k, seed):
    """The FP32 bar on long problems (20,000 columns, 0.5% missing calls): the FP32
    column step converges to its own fixed point within each tree, so errors that are
    invisible on short fixtures show here first."""
    prob = simulate(k, 20000, seed=seed, missing=0.005)
    r32, r64 = (api.run_batch([prob], precision=p, want_forward=False, want_posterior=True)[0]
                for p in ("fp32", "fp64"))
    assert np.max(np.abs(r32.posterior - r64.posterior)) <= 1e-5
    assert abs(r32.loglik - r64.loglik) <= 1e-5 * abs(r64.loglik)


def _split_mismatches(prob, u):
    r = api.run_batch([prob], precision="fp32", want_path=True, uniforms=[u])[0]
    ref = pyoracle.traceback_split(prob, r.forward.astype(np.float64), u, given=r.path)
    return int(np.count_nonzero(ref != r.path))


@pytest.mark.parametrize("name", NAMES)
def test_fp32_path_matches_decomposed_oracle(name):
    """FP32 traceback: every column's draw equals the oracle's decomposed draw given the
    GPU's own next state and FP32 forward table; the oracle computes in FP64, so a draw may
    differ only where the uniform falls within rounding of a boundary."""
    prob, gold = load(name)
    assert _split_mismatches(prob, gold["uniforms"]) <= 1


@pytest.mark.parametrize("k,L,seed", [(40, 5000, 21), (63, 3000, 22)])
def test_fp32_path_matches_decomposed_oracle_larger(k, L, seed):
    prob = simulate(k, L, seed=seed, missing=0.005)
    u = np.random.default_rng(seed).random(prob.seqlen)
    assert _split_mismatches(prob, u) <= 2


def test_fp32_paths_sample_the_posterior():
    """Empirical state marginals of 2000 FP32 paths (one batch, independent uniforms)
    against the FP64 posterior marginals: within 5 sigma + 2e-3 at every cell."""
    prob = simulate(6, 120, seed=8, missing=0.005)
    n = 2000
    rng = np.random.default_rng(3)
    us = [rng.random(prob.seqlen) for _ in range(n)]
    rs = api.run_batch([prob] * n, precision="fp32", want_forward=False, want_path=True,
                       uniforms=us)
    post = api.posterior(prob)
    off = pyoracle.offsets(pyoracle.nstates(prob))
    counts = np.zeros_like(post)
    for r in rs:
        counts[off[:-1] + r.path] += 1
    emp = counts / n
    sig = np.sqrt(post * (1.0 - post) / n)
    assert np.all(np.abs(emp - post) <= 5.0 * sig + 2e-3)


@pytest.mark.parametrize("name", EXTERNAL_DEFAULT_MAP)
def test_c_abi_forward_alg(name):
    prob, gold = load(name)
    rows = refapi.arghmm_forward_alg(prob)
    fw_o, _ = pyoracle.forward(prob)
    assert max_rel(np.concatenate(rows), fw_o) <= 1e-12
    np.testing.assert_array_equal([len(r) for r in rows], np.maximum(gold["nstates"], 1))


def test_c_abi_forward_alg_given_prior():
    prob, gold = load("dsmc_k8_s11")
    S0 = int(gold["nstates"][0])
    prior = np.random.default_rng(3).random(S0)
    rows = refapi.arghmm_forward_alg(prob, prior=prior)
    np.testing.assert_array_equal(rows[0], prior)


@pytest.mark.parametrize("name", EXTERNAL_DEFAULT_MAP)
def test_c_abi_sample_posterior_with_srand(name):
    prob, gold = load(name)
    refapi.srand(int(gold["seed"]))
    path = refapi.arghmm_sample_posterior(prob)
    # expected (node, time) from the reference's state index path, column by column
    exp = np.zeros((prob.seqlen, 2), dtype=np.int64)
    pos = 0
    for b in range(prob.ntrees):
        par, age = prob.ptrees[b], prob.ages[b]
        states = []
        for v in range(prob.nnodes):
            top = prob.ntimes - 2 if par[v] == -1 else age[par[v]]
            states += [(v, t) for t in range(age[v], top + 1)]
        for i in range(pos, pos + prob.blocklens[b]):
            exp[i] = states[gold["path"][i]]
        pos += prob.blocklens[b]
    np.testing.assert_array_equal(path, exp)


@pytest.mark.parametrize("name", EXTERNAL_DEFAULT_MAP[:3])
def test_c_abi_backward_and_posterior(name):
    prob, _ = load(name)
    bw = np.concatenate(refapi.arghmm_backward_alg(prob))
    bw_o = pyoracle.backward(prob)
    assert max_rel(bw, bw_o) <= 1e-10
    post = np.concatenate(refapi.arghmm_posterior_marginals(prob))
    fw_o, _ = pyoracle.forward(prob)
    ref = pyoracle.posterior(prob, fw_o, bw_o)
    assert np.max(np.abs(post - ref)) <= 1e-14


def test_internal_c_abi_sample_thread():
    # leaf cut: a single-leaf subtree (index order of the virtual root's children holds)
    full = simulate(8, 1200, 77, add_thread=False)
    prob = _leaf_cut(full)
    refapi.srand(5)
    path = refapi.arghmm_sample_arg_thread_internal(prob)
    fw, _ = pyoracle.forward(prob)
    u = pyoracle.rand_uniforms(5, prob.seqlen)
    np.testing.assert_array_equal(path, pyoracle.traceback(prob, fw, u))


def _leaf_cut(full: Problem) -> Problem:
    """Cut leaf 0's branch in every tree: its parent becomes the virtual root (age
    ntimes+1) with children (leaf 0, rest of the tree), as remove_arg_thread_path leaves
    a leaf removal (thread.cpp:1481). Only trees whose SPRs avoid leaf 0 and its parent are
    kept, so the SPRs stay valid."""
    T = full.ntimes
    keep = []
    for b in range(full.ntrees):
        if b > 0:
            rn, cn = full.sprs[b, 0], full.sprs[b, 2]
            p0 = full.ptrees[b - 1, 0]
            if rn in (0, p0) or cn in (0, p0) or full.ptrees[b - 1, rn] == p0:
                break
        keep.append(b)
    B = len(keep)
    ptrees = full.ptrees[:B].copy()
    ages = full.ages[:B].copy()
    for b in range(B):
        par = ptrees[b]
        p = par[0]
        sib = [v for v in range(full.nnodes) if par[v] == p and v != 0][0]
        gp = par[p]
        par[sib] = gp
        if gp == -1:
            main = sib
        else:
            main = int(np.nonzero(par == -1)[0][0])
        par[p] = -1
        par[main] = p
        ages[b, p] = T + 1
    L = int(full.blocklens[:B].sum())
    sprs = full.sprs[:B].copy()
    return Problem(times=full.times, popsizes=full.popsizes, rho=full.rho, mu=full.mu,
                   ptrees=ptrees, ages=ages, sprs=sprs, blocklens=full.blocklens[:B].copy(),
                   seqs=full.seqs[:, :L].copy(), internal=True)


def test_batch_matches_single_runs():
    probs = [load(n)[0] for n in NAMES]
    batch = api.run_batch(probs, want_posterior=True)
    for p, rb in zip(probs, batch):
        r1 = api.run_batch([p], want_posterior=True)[0]
        np.testing.assert_array_equal(rb.forward, r1.forward)
        np.testing.assert_array_equal(rb.posterior, r1.posterior)
        assert rb.loglik == r1.loglik


def test_edge_cases_single_column_blocks_and_tiny_problems():
    # every block one column long; a one-column problem
    prob = simulate(5, 300, 9)
    bl = np.ones(prob.ntrees, dtype=np.int32)
    tiny = Problem(times=prob.times, popsizes=prob.popsizes, rho=prob.rho, mu=prob.mu,
                   ptrees=prob.ptrees, ages=prob.ages, sprs=prob.sprs, blocklens=bl,
                   seqs=prob.seqs[:, :prob.ntrees].copy())
    one = Problem(times=prob.times, popsizes=prob.popsizes, rho=prob.rho, mu=prob.mu,
                  ptrees=prob.ptrees[:1], ages=prob.ages[:1], sprs=prob.sprs[:1],
                  blocklens=np.array([1], np.int32), seqs=prob.seqs[:, :1].copy())
    for p in (tiny, one):
        r = api.run_batch([p], want_path=True, want_posterior=True,
                          uniforms=[np.full(p.seqlen, 0.5)])[0]
        fw_o, _ = pyoracle.forward(p)
        assert max_rel(r.forward, fw_o) <= 1e-12
        np.testing.assert_array_equal(r.path, pyoracle.traceback(p, fw_o, np.full(p.seqlen, 0.5)))


def test_all_missing_column_data_is_prior():
    # every call 'N': emissions are 1, the posterior is the prior chain's marginal
    prob = simulate(6, 500, 12)
    prob.seqs[:] = ord("N")
    r = api.run_batch([prob], want_posterior=True)[0]
    fw_o, lnl_o = pyoracle.forward(prob)
    assert max_rel(r.forward, fw_o) <= 1e-12
    assert abs(r.loglik - lnl_o) <= 1e-9


@pytest.mark.parametrize("name", ["dsmc_k8_s11", "dsmc_k17_missing", "cut_k10_s3"])
def test_conditioned_path_matches_oracle(name):
    """awg_sample_path_conditioned (the conditioned samplers' forward and traceback): a
    first column holding 1 at a chosen state and a given last state give the oracle's path on
    its forward table with that first column, the last column taking no draw; each alone
    too."""
    prob, _ = load(name)
    ns = pyoracle.nstates(prob)
    S0, SL = max(int(ns[0]), 1), max(int(ns[-1]), 1)
    rng = np.random.default_rng(17)
    u = rng.random(prob.seqlen)
    prior = np.zeros(S0)
    prior[S0 // 3] = 1.0
    last = (2 * SL) // 3
    for pr, ls in ((prior, last), (prior, -1), (None, last)):
        path = api.sample_path_conditioned(prob, prior=pr, last_state=ls, uniforms=u)
        fw, _ = pyoracle.forward(prob, prior=pr)
        ref = pyoracle.traceback_last(prob, fw, u, ls)
        np.testing.assert_array_equal(path, ref)
        if pr is not None:
            assert path[0] == S0 // 3
        if ls >= 0:
            assert path[-1] == ls


def test_conditioned_path_rand_order():
    """With no uniforms the draws come from libc rand() in the reference's order: one per
    column from the last drawn column down to column 0 (none for a given last state)."""
    prob, _ = load("dsmc_k8_s12")
    ns = pyoracle.nstates(prob)
    last = max(int(ns[-1]), 1) - 1
    refapi.srand(41)
    path = api.sample_path_conditioned(prob, last_state=last)
    fw, _ = pyoracle.forward(prob)
    # rand_uniforms(seed, n): the draws of a traceback over n columns, last column first,
    # indexed by column; column L-1 takes none here, so columns 0..L-2 take them
    u = np.zeros(prob.seqlen)
    u[:-1] = pyoracle.rand_uniforms(41, prob.seqlen - 1)
    np.testing.assert_array_equal(path, pyoracle.traceback_last(prob, fw, u, last))


@pytest.mark.parametrize("name", ["dsmc_k8_s11", "dsmc_k10_T32", "cut_k10_s3", "single_k7_s41",
                                  "dsmc_k17_missing"])
def test_c_abi_forward_alg_slow_dense_step(name):
    """arghmm_forward_alg(slow=True): the reference's dense S x S test step
    (arghmm_forward_block_slow, sample_thread.cpp:301-337) gives the structured step's
    table within rounding (the reference's own test compares the two, test_hmm.py:314-349)."""
    prob, _ = load(name)
    rows = refapi.arghmm_forward_alg(prob, slow=True)
    fw_o, _ = pyoracle.forward(prob)
    assert max_rel(np.concatenate(rows), fw_o) <= 1e-12
