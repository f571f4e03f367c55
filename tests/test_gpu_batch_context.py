"""Batches in flight from one thread (awg_batch_ctx, api.BatchContext): two contexts used in
turn, each batch launched before the previous one is finished, give the results of
awg_run_batch bit for bit (FP32 and FP64 paths, log-likelihoods, forward tables)."""

import numpy as np
import pytest

from argweaver_gb300 import api
from argweaver_gb300.sim import simulate

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_two_contexts_in_turn_equal_run_batch(precision):
    batches = [[simulate(k, L, seed=900 + 10 * b + k, missing=0.005) for k, L in
                ((7, 3000), (15, 2000), (31, 1200), (9, 500))] for b in range(3)]
    rng = np.random.default_rng(5)
    us = [[rng.random(p.seqlen) for p in batch] for batch in batches]
    want = [api.run_batch(b, precision=precision, want_forward=True, want_path=True, uniforms=u)
            for b, u in zip(batches, us)]
    got = []
    with api.BatchContext() as a, api.BatchContext() as b:
        ctxs = [a, b]
        ctxs[0].launch(batches[0], precision=precision, want_forward=True, uniforms=us[0])
        for i in range(1, len(batches)):
            ctxs[i % 2].launch(batches[i], precision=precision, want_forward=True,
                               uniforms=us[i])
            got.append(ctxs[(i - 1) % 2].finish())
        got.append(ctxs[(len(batches) - 1) % 2].finish())
    for w, g in zip(want, got):
        for rw, rg in zip(w, g):
            np.testing.assert_array_equal(rg.path, rw.path)
            np.testing.assert_array_equal(rg.forward, rw.forward)
            assert rg.loglik == rw.loglik


def test_a_context_holds_one_batch():
    p = simulate(7, 300, seed=5)
    with api.BatchContext() as c:
        c.launch([p])
        with pytest.raises(RuntimeError):
            c.launch([p])
        assert len(c.finish()) == 1
        with pytest.raises(RuntimeError):
            c.finish()
