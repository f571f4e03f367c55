"""Schedules do not change results (GPU only).

The persistent work-stealing per-tree kernels, the forward kernel's CTA size (states per
owner thread), the instance groups of the pipelined schedule and CUDA-graph replay are
execution choices: every sum has an order fixed by the tree, so each choice must give the
same tables, paths and log-likelihoods bit for bit. Also: a repeated batch replays its
captured graph, and the autotuner's choice is one of its candidates and is then used.
"""

import numpy as np
import pytest

from argweaver_gb300 import api
from argweaver_gb300.sim import simulate

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def batch():
    rng = np.random.default_rng(5)
    probs = [simulate(int(rng.integers(6, 30)), int(rng.integers(300, 1500)), seed=100 + i,
                      missing=0.005) for i in range(20)]
    us = [np.random.default_rng(200 + i).random(p.seqlen) for i, p in enumerate(probs)]
    return probs, us


def run(probs, us, precision):
    rs = api.run_batch(probs, precision=precision, want_path=True, uniforms=us)
    return [(r.forward.copy(), r.path.copy(), r.loglik) for r in rs]


def same(a, b):
    for (f1, p1, l1), (f2, p2, l2) in zip(a, b):
        np.testing.assert_array_equal(f1, f2)
        np.testing.assert_array_equal(p1, p2)
        assert l1 == l2


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_schedules_give_identical_results(batch, precision):
    probs, us = batch
    api.set_graphs(False)
    api.set_schedule(0, 8, 1, False)
    ref = run(probs, us, precision)
    try:
        for kpt, div, chunk, pers in [(0, 8, 1, True), (0, 4, 4, True), (4, 16, 2, True),
                                      (2, 2, 8, False), (1, 8, 1, True)]:
            api.set_schedule(kpt, div, chunk, pers)
            same(ref, run(probs, us, precision))
        api.set_graphs(True)
        api.set_schedule(0, 8, 1, True)
        same(ref, run(probs, us, precision))
        # a small batch takes the serial schedule, also captured
        same(ref[:3], run(probs[:3], us[:3], precision))
    finally:
        api.set_graphs(True)
        api.set_schedule()


def test_repeated_batch_replays_its_graph(batch):
    probs, us = batch
    api.set_graphs(True)
    first = run(probs, us, "fp32")
    c0 = api.graph_counts()
    again = run(probs, us, "fp32")
    c1 = api.graph_counts()
    assert c1["replays"] == c0["replays"] + 1
    assert c1["captures"] == c0["captures"]
    same(first, again)
    # another batch shape is captured anew
    run(probs[:17], us[:17], "fp32")
    assert api.graph_counts()["captures"] == c1["captures"] + 1


def test_autotune_picks_a_candidate_and_keeps_results(batch):
    probs, us = batch
    ref = run(probs, us, "fp32")
    cfg = api.autotune(probs, precision="fp32", want_path=True, trials=1)
    assert cfg["kpt"] in (0, 2, 4) and cfg["group_div"] in (4, 8, 16)
    assert cfg["chunk"] in (1, 4) and cfg["persistent"] in (0, 1) and cfg["ms"] > 0
    same(ref, run(probs, us, "fp32"))
    api.set_schedule()
