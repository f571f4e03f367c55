"""Parity at the configurations' scale (GPU only).

The fixtures in tests/golden pin the oracle to the compiled reference, up to k = 48 and
an internal cut of a k = 50 ARG; here the CUDA path is held to the oracle on the shapes the
benchmark configurations run, including the launch variants only large state counts reach:

  config 1, largest shape   k = 64, 100,000 columns (about 500 states, 4.9e7 cells)
  config 2, prefix          k = 100, 30,000 columns (about 700 states), the forward kernel
                            with 2, 4 and 8 states per owner thread
  config 4, extreme         k = 200, ntimes = 32 (about 1,500 states)
  beyond the configs        a 130-leaf caterpillar tree at ntimes = 32 (3,899 states): more
                            states than the register kernel holds, so the shared-memory
                            forward kernel and the FP32 full-scan traceback run
  config 3 shape            an internal-branch cut of a k = 50 ARG along a uniform removal
                            path, the cut subtrees holding several leaves

Bars, as for the fixtures: FP64 forward table <= 1e-12 relative per cell and the
log-likelihood <= 1e-12 relative to the oracle; the FP64 sampled path identical to the
oracle's reference scan given the same uniforms; FP64 posterior <= 1e-10 relative to the
oracle's forward-backward (cells above 1e-200) and 1e-13 absolute; FP32 against FP64: posterior marginals
within 1e-5 absolute and, on cells whose FP64 marginal is at least POST_FLOOR, within
POST_REL relative; FP32 tracebacks draw, column by column given the GPU's own next state,
what the oracle draws on the GPU's FP32 table except where a uniform falls within rounding
of a boundary.
"""

import numpy as np
import pytest

import pyoracle
from argweaver_gb300 import api, refapi
from argweaver_gb300.problem import Problem
from argweaver_gb300.sim import simulate

pytestmark = pytest.mark.gpu

POST_FLOOR = 1e-3
POST_REL = 1e-5


def max_rel(a, b, floor=1e-300):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))


_oracle_cache = {}


def oracle(key, prob, posterior=False):
    """The oracle's forward table, log-likelihood and (optionally) posterior, cached per
    test problem."""
    if key not in _oracle_cache:
        fw, lnl = pyoracle.forward(prob)
        _oracle_cache[key] = {"fw": fw, "lnl": lnl}
    d = _oracle_cache[key]
    if posterior and "post" not in d:
        d["post"] = pyoracle.posterior(prob, d["fw"], pyoracle.backward(prob))
    return d


def check_fp64(key, prob, u, kpt=0):
    api.set_schedule(kpt=kpt)
    try:
        r = api.run_batch([prob], want_forward=True, want_path=True, uniforms=[u])[0]
    finally:
        api.set_schedule()
    o = oracle(key, prob)
    assert r.forward.shape == o["fw"].shape
    rel = max_rel(r.forward, o["fw"])
    assert rel <= 1e-12, f"FP64 forward max rel {rel:.3e}"
    assert abs(r.loglik - o["lnl"]) <= 1e-12 * abs(o["lnl"])
    path = pyoracle.traceback(prob, o["fw"], u)
    np.testing.assert_array_equal(r.path, path)
    return r


def check_fp32_posterior(prob):
    """FP32 against FP64 posterior marginals: max absolute error, and max relative error on
    cells whose FP64 marginal is at least POST_FLOOR."""
    a = api.run_batch([prob], precision="fp32", want_forward=False, want_posterior=True)[0]
    b = api.run_batch([prob], precision="fp64", want_forward=False, want_posterior=True)[0]
    err = np.abs(a.posterior - b.posterior)
    big = b.posterior >= POST_FLOOR
    abs_err = float(err.max())
    rel_err = float(np.max(err[big] / b.posterior[big]))
    print(f"fp32 posterior: max abs {abs_err:.3e}, max rel (>= {POST_FLOOR:g}) {rel_err:.3e}, "
          f"{int(big.sum())} cells above the floor")
    assert abs_err <= 1e-5
    assert rel_err <= POST_REL
    assert abs(a.loglik - b.loglik) <= 1e-5 * abs(b.loglik)
    return b


def split_mismatches(prob, u, kpt=0):
    """FP32 decomposed traceback against the oracle's decomposed draw, per column given the
    GPU's own next state and FP32 table."""
    api.set_schedule(kpt=kpt)
    try:
        r = api.run_batch([prob], precision="fp32", want_path=True, uniforms=[u])[0]
    finally:
        api.set_schedule()
    ref = pyoracle.traceback_split(prob, r.forward.astype(np.float64), u, given=r.path)
    return int(np.count_nonzero(ref != r.path))


# ---- config 1's largest shape --------------------------------------------------------

@pytest.fixture(scope="module")
def c1():
    return simulate(63, 100000, seed=101, missing=0.005)


def test_config1_largest_fp64_forward_path(c1):
    u = np.random.default_rng(1).random(c1.seqlen)
    check_fp64("c1", c1, u)


def test_config1_largest_fp64_posterior(c1):
    post = api.posterior(c1)
    ref = oracle("c1", c1, posterior=True)["post"]
    big = ref > 1e-200
    assert max_rel(post[big], ref[big]) <= 1e-10
    # over 100,000 columns the backward's rounding reaches a few 1e-14 absolute
    assert np.max(np.abs(post - ref)) <= 1e-13


def test_config1_largest_fp32(c1):
    check_fp32_posterior(c1)
    u = np.random.default_rng(2).random(c1.seqlen)
    assert split_mismatches(c1, u) <= 3


# ---- config 2's shape, every register-kernel width --------------------------------------

@pytest.fixture(scope="module")
def c2():
    return simulate(99, 30000, seed=102, missing=0.0)


@pytest.mark.parametrize("kpt", [2, 4, 8])
def test_config2_prefix_fp64_per_width(c2, kpt):
    u = np.random.default_rng(3).random(c2.seqlen)
    check_fp64("c2", c2, u, kpt=kpt)


@pytest.mark.parametrize("kpt", [2, 4, 8])
def test_config2_prefix_fp32_per_width(c2, kpt):
    u = np.random.default_rng(4).random(c2.seqlen)
    assert split_mismatches(c2, u, kpt=kpt) <= 2


def test_config2_prefix_fp32_posterior(c2):
    check_fp32_posterior(c2)


# ---- config 4's extreme: k = 200, ntimes = 32 --------------------------------------------

@pytest.fixture(scope="module")
def c4():
    return simulate(199, 3000, seed=104, ntimes=32, missing=0.005)


@pytest.mark.parametrize("kpt", [0, 8])
def test_config4_extreme_fp64(c4, kpt):
    assert c4.nstates_per_tree().max() > 1400
    u = np.random.default_rng(5).random(c4.seqlen)
    check_fp64("c4", c4, u, kpt=kpt)


def test_config4_extreme_fp32(c4):
    check_fp32_posterior(c4)
    u = np.random.default_rng(6).random(c4.seqlen)
    assert split_mismatches(c4, u) <= 2


# ---- beyond the register kernel: the shared-memory forward and the FP32 full scan -------

@pytest.fixture(scope="module")
def wide():
    """A single tree of 130 leaves in a caterpillar whose internal nodes are all old (time
    indices 26-30 of 32): every leaf spans about 28 time points, 3,899 states in all, more
    than the register-resident forward kernel holds (3,072), with 259 nodes. FP32 only: the
    FP64 emission kernel's shared memory holds about 1,800 states at this node count."""
    base = simulate(5, 50, seed=1, ntimes=32)
    nl = 130
    nn = 2 * nl - 1
    par = np.full(nn, -1, np.int32)
    age = np.zeros(nn, np.int32)
    prev = 0
    for j in range(nl - 1):
        v = nl + j
        par[prev] = v
        par[j + 1] = v
        age[v] = 26 + (j * 5) // (nl - 1)
        prev = v
    L = 300
    # sparse differences, as in real alignments (a column where every base is random would
    # take the pruning's partials down to about 4^-131, below FP32's range)
    rng = np.random.default_rng(5)
    consensus = rng.integers(0, 4, size=L)
    calls = np.tile(consensus, (nl + 1, 1))
    hit = rng.random(calls.shape) < 0.01
    calls[hit] = rng.integers(0, 4, size=int(hit.sum()))
    seqs = np.frombuffer(b"ACGT", np.uint8)[calls]
    p = Problem(times=base.times, popsizes=base.popsizes, rho=base.rho, mu=base.mu,
                ptrees=par[None, :].copy(), ages=age[None, :].copy(),
                sprs=np.full((1, 4), -1, np.int32), blocklens=np.array([L], np.int32),
                seqs=np.ascontiguousarray(seqs))
    assert p.nstates_per_tree().max() > 8 * 384
    return p


def test_wide_fp32_fallback_kernel_and_full_scan_traceback(wide):
    """FP32 with more states than the register kernel holds: the shared-memory forward
    kernel, and a traceback that scans every state as the reference does. Forward columns
    against the oracle's within FP32 tolerance; per column, given the GPU's own next state,
    the draw is the oracle's scan on the same FP32 table; posterior against the oracle's."""
    u = np.random.default_rng(8).random(wide.seqlen)
    r = api.run_batch([wide], precision="fp32", want_path=True, uniforms=[u])[0]
    o = oracle("wide", wide, posterior=True)
    off = pyoracle.offsets(pyoracle.nstates(wide))
    f32 = r.forward.astype(np.float64)
    assert np.max(np.abs(f32 - o["fw"])) <= 1e-5
    ref = pyoracle.traceback(wide, f32, u, given=r.path)
    assert int(np.count_nonzero(ref != r.path)) <= 2
    post = api.run_batch([wide], precision="fp32", want_forward=False, want_posterior=True)[0]
    assert np.max(np.abs(post.posterior - o["post"])) <= 1e-5
    assert off[-1] == f32.size


# ---- config 3's shape: a multi-leaf internal cut of a k = 50 ARG ------------------------

def cut_leaves(prob: Problem) -> int:
    nleaves = (prob.nnodes + 1) // 2
    best = 0
    for b in range(prob.ntrees):
        par, top = prob.ptrees[b], int(prob.root_child0[b])
        n = 0
        for v in range(nleaves):
            x = v
            while x != -1 and x != top:
                x = par[x]
            n += x == top
        best = max(best, n)
    return best


@pytest.fixture(scope="module")
def c3():
    """The first seeded k = 50 ARG (20,000 columns) whose uniform removal path (after
    srand(seed)) cuts subtrees of several leaves and leaves at least 30 states per column
    on average, cut as arg-sample cuts it (maxtime ntimes + 1). Along such a path the cut
    subtree changes from tree to tree, up to most of the leaves."""
    for seed in range(1, 60):
        full = simulate(50, 20000, seed=3000 + seed, add_thread=False, missing=0.01)
        refapi.srand(seed)
        path, _ = refapi.sample_arg_removal_path_uniform(full)
        cut = refapi.as_problem(full, refapi.remove_arg_thread_path(full, path), internal=True)
        if cut_leaves(cut) >= 3 and cut.cells() >= 30 * cut.seqlen:
            return cut
    pytest.fail("no seed gave a multi-leaf cut")


def test_config3_multileaf_cut_fp64(c3):
    u = np.random.default_rng(9).random(c3.seqlen)
    check_fp64("c3", c3, u)


def test_config3_multileaf_cut_fp32(c3):
    check_fp32_posterior(c3)
    u = np.random.default_rng(10).random(c3.seqlen)
    assert split_mismatches(c3, u) <= 2


# ---- FP32 paths as samples of the posterior, at the benchmark's state counts -----------

def test_fp32_paths_sample_the_posterior_at_scale():
    """3,000 FP32 paths of one k = 64, 1,500-column problem (about 500 states per column)
    drawn by the traceback alone from one resident FP32 forward table, fresh uniforms each:
    every cell's empirical frequency within 5 sigma + 2e-3 of the FP64 posterior marginal,
    and the mean total-variation distance between a column's empirical and posterior
    distributions within 1.25x its expectation under exact sampling (a biased sampler at
    this state count moves the mean well beyond that)."""
    from argweaver_gb300.server import Server

    prob = simulate(63, 1500, seed=105, missing=0.005)
    post = api.posterior(prob)
    off = pyoracle.offsets(pyoracle.nstates(prob))
    assert np.diff(off).mean() > 400
    n = 3000
    rng = np.random.default_rng(11)
    counts = np.zeros_like(post)
    cols = np.arange(prob.seqlen)
    with Server(device_bytes=2 << 30, max_inflight=1, max_batch=1) as srv:
        t = srv.submit(prob, precision="fp32", resident=True)
        assert srv.wait(t, timeout=120) is not None
        for _ in range(n):
            path = srv.resample(t, rng.random(prob.seqlen))
            counts[off[cols] + path] += 1
        srv.release(t)
    emp = counts / n
    sig = np.sqrt(post * (1.0 - post) / n)
    assert np.all(np.abs(emp - post) <= 5.0 * sig + 2e-3)
    # E|emp - p| ~ sqrt(2 / pi) * sigma for the cells with enough mass to be near normal
    tv = 0.5 * np.add.reduceat(np.abs(emp - post), off[:-1])
    expect = 0.5 * np.add.reduceat(np.sqrt(2.0 / np.pi) * sig, off[:-1])
    assert tv.mean() <= 1.25 * expect.mean(), (tv.mean(), expect.mean())
