"""Recombination sampling along a thread on the GPU (awg_sample_recombinations, the
reference's sample_recombinations, recomb.cpp:151-235). Bar: the reference's
recombinations exactly (columns, nodes, times) and the same number of draws, given the
draws rand() gives after srand(seed)."""

import ctypes as C
import glob
import os

import numpy as np
import pytest

from argweaver_gb300 import api, refapi
from argweaver_gb300.problem import Problem
from conftest import GOLDEN, load_golden

pytestmark = pytest.mark.gpu

RMAX = 2147483647.0
NAMES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "recomb", "*.npz")))


def case(name):
    rec = np.load(os.path.join(GOLDEN, "recomb", name + ".npz"))
    if name.startswith("extra_"):
        return Problem.load(os.path.join(GOLDEN, "recomb", name + ".prob")), rec["path"], rec
    prob, gold = load_golden(name)
    return prob, gold["path"], rec


@pytest.mark.parametrize("name", NAMES)
def test_recombinations_match_reference(name):
    prob, path, rec = case(name)
    before = api.kernel_launches()
    pos, node, time, used = refapi.sample_recombinations(prob, path, int(rec["seed"]))
    assert api.kernel_launches() > before
    np.testing.assert_array_equal(pos, rec["pos"])
    np.testing.assert_array_equal(node, rec["node"])
    np.testing.assert_array_equal(time, rec["time"])
    # the draw after the last one used is the reference's next rand()
    refapi.srand(int(rec["seed"]))
    libc = C.CDLL(None)
    for _ in range(used):
        libc.rand()
    assert libc.rand() == int(rec["next_rand"])


def test_recombination_errors():
    prob, path, rec = case("extra_k8_T20")
    u = np.full(4, 0.5)
    with pytest.raises(api.GpuError, match="uniforms ran out"):
        api.sample_recombinations(prob, path, u)
    bad = np.array(path, dtype=np.int32)
    bad[rec["pos"][0]] = 10 ** 6
    with pytest.raises(api.GpuError, match="not a state"):
        api.sample_recombinations(prob, bad, np.full(2 * prob.seqlen + 2, 0.5))
