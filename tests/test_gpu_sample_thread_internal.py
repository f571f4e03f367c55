"""The internal-branch resampling step on the GPU (sample_arg_thread_internal,
sample_thread.cpp:635-692): forward, traceback and recombinations on the device, the regraft
on the host. Bar: after the same srand(seed), the whole ARG is the reference's."""

import os

import numpy as np
import pytest

from argweaver_gb300 import refapi
from conftest import GOLDEN, load_golden

pytestmark = pytest.mark.gpu

NAMES = sorted(f[:-4] for f in os.listdir(os.path.join(GOLDEN, "samplethreadinternal")) if f.endswith(".npz"))


@pytest.mark.parametrize("name", NAMES)
def test_sample_thread_internal_matches_reference(name):
    prob, _ = load_golden(name)
    ref = np.load(os.path.join(GOLDEN, "samplethreadinternal", name + ".npz"))
    refapi.srand(int(ref["seed"]))
    got, path = refapi.sample_arg_thread_internal(prob)
    assert path.shape == (prob.seqlen,)
    for key in ("ptrees", "ages", "blocklens", "root_child0"):
        np.testing.assert_array_equal(got[key], ref[key], err_msg=key)
    np.testing.assert_array_equal(got["sprs"][1:], ref["sprs"][1:])
    np.testing.assert_array_equal(got["mapping"][1:], ref["mapping"][1:])
