"""Regrafting a cut subtree along its internal thread path (add_arg_thread_path,
thread.cpp:1314-1449) on the host: the whole ARG (trees, SPRs, block lengths, node mappings,
root child order) equals the reference's for the internal fixtures' paths and
recombinations; a cut followed by the regraft along the cut's own thread gives back trees
that cover the region."""

import os

import numpy as np
import pytest

from argweaver_gb300 import refapi
from argweaver_gb300.problem import Problem
from conftest import GOLDEN, load_golden

NAMES = sorted(f[:-4] for f in os.listdir(os.path.join(GOLDEN, "addthreadpath")) if f.endswith(".npz"))


@pytest.mark.parametrize("name", NAMES)
def test_add_thread_path_matches_reference(name):
    prob, gold = load_golden(name)
    rec = np.load(os.path.join(GOLDEN, "recomb", name + ".npz"))
    ref = np.load(os.path.join(GOLDEN, "addthreadpath", name + ".npz"))
    got = refapi.add_arg_thread_path(prob, gold["path"], rec["pos"], rec["node"], rec["time"])
    assert got["ptrees"].shape == ref["ptrees"].shape
    for key in ("ptrees", "ages", "sprs", "blocklens", "root_child0"):
        sl = slice(1, None) if key == "sprs" else slice(None)  # the first tree has no SPR
        np.testing.assert_array_equal(got[key][sl], ref[key][sl], err_msg=key)
    np.testing.assert_array_equal(got["mapping"][1:], ref["mapping"][1:])
    assert got["ptrees"].shape[0] == prob.ntrees + len(rec["pos"])


@pytest.mark.parametrize("name", NAMES)
def test_thread_times_match_reference(name):
    prob, gold = load_golden(name)
    ref = np.load(os.path.join(GOLDEN, "addthreadpath", name + ".npz"))
    got = refapi.get_thread_times(prob, gold["path"])
    if len(ref["thread_times"]):  # every tree has states: the reference's times
        np.testing.assert_array_equal(got, ref["thread_times"])
    else:  # some tree is whole: -1 on its columns, a state time elsewhere
        assert np.all(got >= -1) and np.any(got == -1) and np.all(got < prob.ntimes)


def test_add_thread_path_rejects_bad_input():
    name = NAMES[0]
    prob, gold = load_golden(name)
    rec = np.load(os.path.join(GOLDEN, "recomb", name + ".npz"))
    bad = np.full(len(gold["path"]), 10 ** 6, dtype=np.int32)  # partial trees read the path
    with pytest.raises(ValueError, match="state"):
        refapi.add_arg_thread_path(prob, bad, rec["pos"], rec["node"], rec["time"])
    with pytest.raises(ValueError, match="increase"):
        refapi.add_arg_thread_path(prob, gold["path"], rec["pos"][::-1], rec["node"][::-1],
                                   rec["time"][::-1])
    full = Problem.load(os.path.join(GOLDEN, "addthread", "single_k7_s41.prob"))
    with pytest.raises(ValueError, match="internal"):
        refapi.add_arg_thread_path(full, np.zeros(full.seqlen), [], [], [])
