"""The re-threading moves of the MCMC loop on the GPU, each against the reference's own run
after the same srand(seed):

- resample_arg_leaf's move (sample_arg.cpp:66-86): awg_remove_arg_thread, then
  awg_sample_arg_thread for the removed sequence (forward, traceback and recombinations on
  the device, the thread added on the host);
- sample_arg_thread_internal (sample_thread.cpp:635-692): awg_sample_arg_thread_internal on
  the cut fixtures (the device step, the regraft on the host).

The host halves and the order of the draws are pinned on the CPU (test_thread_remove.py,
test_thread_internal_step.py); this file is collected after the other GPU files so that
they all run before it.
"""

import os

import numpy as np
import pytest

from argweaver_gb300 import refapi
from argweaver_gb300.problem import Problem
from conftest import GOLDEN, load_golden

pytestmark = pytest.mark.gpu

RL_NAMES = sorted(f[:-4] for f in os.listdir(os.path.join(GOLDEN, "resampleleaf")) if f.endswith(".npz"))
IN_NAMES = sorted(f[:-4] for f in os.listdir(os.path.join(GOLDEN, "samplethreadinternal")) if f.endswith(".npz"))


def _same_arg(got, ref, root_child0=False):
    keys = ("ptrees", "ages", "blocklens") + (("root_child0",) if root_child0 else ())
    for key in keys:
        np.testing.assert_array_equal(got[key], ref[key], err_msg=key)
    np.testing.assert_array_equal(got["sprs"][1:], ref["sprs"][1:])
    np.testing.assert_array_equal(got["mapping"][1:], ref["mapping"][1:])


@pytest.mark.parametrize("name", RL_NAMES)
def test_leaf_resampling_move_matches_reference(name):
    ref = np.load(os.path.join(GOLDEN, "resampleleaf", name + ".npz"))
    full = Problem.load(os.path.join(GOLDEN, "addthread", name + ".prob"))
    refapi.srand(int(ref["seed"]))
    _same_arg(refapi.resample_arg_leaf(full, int(ref["seqid"])), ref)


@pytest.mark.parametrize("name", IN_NAMES)
def test_sample_thread_internal_matches_reference(name):
    prob, _ = load_golden(name)
    ref = np.load(os.path.join(GOLDEN, "samplethreadinternal", name + ".npz"))
    refapi.srand(int(ref["seed"]))
    got, path = refapi.sample_arg_thread_internal(prob)
    assert path.shape == (prob.seqlen,)
    _same_arg(got, ref, root_child0=True)
