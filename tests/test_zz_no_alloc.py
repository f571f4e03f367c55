"""awg_forward_static: the forward pass with every device buffer in a static device array.

Called through the C ABI and checked against awg_run_batch (the allocating entry point) on
the same problems, two calls in a row, so that the second call runs over scratch the first
one left behind. Tolerances: FP64 forward table and log-likelihood 1e-12 relative; FP32
forward table 1e-6 relative (both paths run the same kernels, so equality is expected).
The file is named to be collected last: it has to pass alone in a fresh process as well as
after every other test has used the batch engine.
"""

import ctypes as C
import os

import numpy as np
import pytest

from argweaver_gb300 import api, capi
from argweaver_gb300.problem import Problem
from argweaver_gb300.sim import simulate
from conftest import GOLDEN, golden_names

pytestmark = pytest.mark.gpu

SCRATCH_BYTES = 64 << 20  # AWG_STATIC_SCRATCH_BYTES


def static_forward(prob, precision):
    """One awg_forward_static call; returns (rc, forward table, loglik)."""
    lib = capi.load()
    b = api._Bound(prob)
    ncell = lib.awg_problem_cells(C.byref(b.c))
    assert ncell > 0, capi.last_error()
    fp32 = precision == "fp32"
    fw = np.full(ncell, np.nan, dtype=np.float32 if fp32 else np.float64)
    ll = np.full(1, np.nan)
    out = capi.AwgOutputs()
    if fp32:
        out.forward32 = fw.ctypes.data
    else:
        out.forward = fw.ctypes.data
    out.loglik = ll.ctypes.data
    rc = lib.awg_forward_static(C.byref(b.c), C.byref(out),
                                capi.AWG_FP32 if fp32 else capi.AWG_FP64, None)
    return rc, fw, float(ll[0])


def check_against_batch(prob, precision):
    ref = api.run_batch([prob], precision=precision)[0]
    rtol = 1e-6 if precision == "fp32" else 1e-12
    for call in range(2):
        rc, fw, ll = static_forward(prob, precision)
        assert rc == 0, f"call {call}: {capi.last_error()}"
        np.testing.assert_allclose(fw, ref.forward, rtol=rtol, atol=0.0)
        assert abs(ll - ref.loglik) <= 1e-12 * abs(ref.loglik)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", golden_names())
def test_static_matches_batch_on_golden(name, precision):
    prob = Problem.load(os.path.join(GOLDEN, name + ".prob"))
    check_against_batch(prob, precision)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_static_matches_batch_on_larger_problem(precision):
    prob = simulate(24, 3000, seed=101, missing=0.005)
    check_against_batch(prob, precision)


def test_static_rejects_problem_beyond_scratch():
    prob = simulate(32, 40000, seed=7)
    cells = api.cells(prob)
    assert cells * 8 > SCRATCH_BYTES  # the FP64 table alone exceeds the array
    rc, fw, _ = static_forward(prob, "fp64")
    assert rc == -5
    msg = capi.last_error()
    assert "static scratch holds %d bytes" % SCRATCH_BYTES in msg
    assert np.isnan(fw).all()  # nothing written
    # the array is still usable after a rejection
    check_against_batch(Problem.load(os.path.join(GOLDEN, "dsmc_k8_s11.prob")), "fp64")


def test_static_rejects_path_and_posterior():
    lib = capi.load()
    prob = Problem.load(os.path.join(GOLDEN, "dsmc_k8_s11.prob"))
    b = api._Bound(prob)
    path = np.zeros(prob.seqlen, dtype=np.int32)
    out = capi.AwgOutputs()
    out.path = path.ctypes.data
    assert lib.awg_forward_static(C.byref(b.c), C.byref(out), capi.AWG_FP64, None) == -1
    assert "path and posterior must be NULL" in capi.last_error()
