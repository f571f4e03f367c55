"""The generic dense HMM (hmm.cpp:27-85: forward_alg, backward_alg, sample_hmm_posterior)
on the GPU, through the reference's C ABI. Bar: tables within 1e-12 (relative) of the
reference's, paths equal to the reference's after the same srand(seed), on the reference's
own fixtures and on larger random matrices against the oracle."""

import ctypes as C
import os

import numpy as np
import pytest

import pyoracle
from argweaver_gb300 import api, refapi
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

FIXTURES = [("single_k7_s41.npz", False), ("single_k7_s43.npz", False),
            ("densehmm/s37_n160.npz", True), ("densehmm/s5_n64.npz", True)]
_libc = C.CDLL(None)


def _first_column(gold, random):
    emit = gold["dense_emit"]
    return emit[0] - np.log(emit.shape[1]) if random else emit[0].copy()


def _close(a, b):
    fin = np.isfinite(b)
    assert np.array_equal(fin, np.isfinite(a))
    np.testing.assert_array_equal(a[~fin], b[~fin])
    np.testing.assert_allclose(a[fin], b[fin], rtol=1e-12, atol=1e-300)


@pytest.mark.parametrize("name,random", FIXTURES)
def test_dense_tables_match_reference(name, random):
    gold = np.load(os.path.join(GOLDEN, name))
    trans, emit = gold["dense_trans"], gold["dense_emit"]
    fw = np.zeros_like(emit)
    fw[0] = _first_column(gold, random)
    before = api.kernel_launches()
    refapi.forward_alg(trans, emit, fw)
    assert api.kernel_launches() > before
    _close(fw, gold["dense_fw"])
    bw = np.zeros_like(emit)
    refapi.backward_alg(trans, emit, bw)
    _close(bw, gold["dense_bw"])


@pytest.mark.parametrize("name,random", FIXTURES)
def test_dense_path_matches_reference_after_srand(name, random):
    gold = np.load(os.path.join(GOLDEN, name))
    ref = gold["dense_path"]
    path = np.zeros_like(ref)
    path[-1] = ref[-1]
    refapi.srand(int(gold["seed"]))
    _libc.rand()  # the reference's draw of the last column
    refapi.sample_hmm_posterior(gold["dense_trans"], gold["dense_fw"], path)
    np.testing.assert_array_equal(path, ref)


def _random_hmm(S, n, seed, zeros=0.1):
    rng = np.random.default_rng(seed)
    w = 0.05 + rng.random((S, S))
    w[rng.random((S, S)) < zeros] = 0.0
    np.fill_diagonal(w, 1.0)
    with np.errstate(divide="ignore"):
        trans = np.log(w / w.sum(axis=1, keepdims=True))
    emit = np.log(0.01 + rng.random((n, S)))
    return trans, emit


@pytest.mark.parametrize("S,n", [(1, 10), (31, 50), (33, 400), (256, 300), (700, 40)])
def test_dense_hmm_matches_oracle(S, n):
    trans, emit = _random_hmm(S, n, S * 7 + n)
    fw = np.zeros_like(emit)
    fw[0] = emit[0] - np.log(S)
    refapi.forward_alg(trans, emit, fw)
    _close(fw, pyoracle.dense_forward(trans, emit, fw[0]))
    bw = np.zeros_like(emit)
    refapi.backward_alg(trans, emit, bw)
    _close(bw, pyoracle.dense_backward(trans, emit, bw[-1]))
    # paths from the oracle's table, uniforms from libc rand() after the same seed
    ofw = pyoracle.dense_forward(trans, emit, fw[0])
    path = np.zeros(n, dtype=np.int32)
    path[-1] = S // 2
    refapi.srand(S + n)
    refapi.sample_hmm_posterior(trans, ofw, path)
    u = np.concatenate([pyoracle.rand_uniforms(S + n, n - 1), [0.0]])
    np.testing.assert_array_equal(path, pyoracle.dense_sample(trans, ofw, u, S // 2))


def test_dense_hmm_edges():
    trans, emit = _random_hmm(8, 1, 3)
    fw = emit.copy()
    refapi.forward_alg(trans, emit, fw)  # one column: nothing to fill
    np.testing.assert_array_equal(fw, emit)
    with pytest.raises(ValueError):
        refapi.forward_alg(trans[:4, :4], emit, fw)
    lib = api.capi.load()
    lib.forward_alg(0, 8, None, None, None)
    assert "positive" in api.capi.last_error()
