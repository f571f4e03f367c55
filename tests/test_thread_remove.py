"""Removing a leaf's thread from the ARG (remove_arg_thread, thread.cpp:425-556) on the host:
after each removal the trees, SPRs, merged blocks (remove_null_sprs, local_tree.cpp:409-469),
node mappings, root child order and the leaves' sequence ids equal the reference's, down to
the trunk genealogy; and adding the removed sequence back gives a full ARG again."""

import os

import numpy as np
import pytest

from argweaver_gb300 import capi, refapi
from argweaver_gb300.problem import Problem
from conftest import GOLDEN

NAMES = sorted(f[:-4] for f in os.listdir(os.path.join(GOLDEN, "removethread")) if f.endswith(".npz"))


def grown(name):
    return Problem.load(os.path.join(GOLDEN, "addthread", name + ".prob"))


@pytest.mark.parametrize("name", NAMES)
def test_remove_thread_matches_reference(name):
    ref = np.load(os.path.join(GOLDEN, "removethread", name + ".npz"))
    removed = [int(x) for x in ref["removed"]]
    steps = refapi.remove_arg_thread(grown(name), removed)
    assert len(steps) == len(removed)
    for i, got in enumerate(steps):
        np.testing.assert_array_equal(got["seqids"], ref[f"seqids_{i}"], err_msg=f"step {i}")
        assert got["ptrees"].shape == ref[f"ptrees_{i}"].shape, f"step {i}"
        np.testing.assert_array_equal(got["ptrees"], ref[f"ptrees_{i}"], err_msg=f"step {i}")
        np.testing.assert_array_equal(got["ages"], ref[f"ages_{i}"], err_msg=f"step {i}")
        np.testing.assert_array_equal(got["sprs"], ref[f"sprs_{i}"], err_msg=f"step {i}")
        np.testing.assert_array_equal(got["blocklens"], ref[f"blocklens_{i}"], err_msg=f"step {i}")
        np.testing.assert_array_equal(got["mapping"][1:], ref[f"mapping_{i}"][1:],
                                      err_msg=f"step {i}")
        np.testing.assert_array_equal(got["root_child0"], ref[f"root_child0_{i}"],
                                      err_msg=f"step {i}")


def test_remove_thread_keeps_region_and_shrinks():
    prob = grown("dsmc_k17_missing")
    steps = refapi.remove_arg_thread(prob, [5])
    s = steps[0]
    assert s["ptrees"].shape[1] == prob.nnodes - 2
    assert int(s["blocklens"].sum()) == int(np.sum(prob.blocklens))
    assert sorted(s["seqids"].tolist()) == [i for i in range(prob.nnodes // 2 + 1) if i != 5]
    # no null SPR is left behind a tree (remove_null_sprs)
    assert np.all(s["sprs"][1:, 0] >= 0)


def test_remove_thread_rejects_unknown_sequence():
    prob = grown("single_k7_s41")
    with pytest.raises(ValueError, match="sequence"):
        refapi.remove_arg_thread(prob, [99])
    with pytest.raises(ValueError, match="sequence"):
        refapi.remove_arg_thread(prob, [2, 2])


def test_remove_then_add_restores_leaf_count():
    """A removed sequence threads back in as a new leaf holding its id: a Gibbs step's
    bookkeeping (resample_arg_leaf, sample_arg.cpp:66-86)."""
    lib = capi.load()
    prob = grown("single_k7_s41").normalized()
    trees = refapi._trees_handle(prob)
    try:
        assert lib.awg_remove_arg_thread(trees.handle, 3) == 0
        nn = lib.get_local_trees_nnodes(trees.handle)
        assert nn == prob.nnodes - 2
        _, _, ids = refapi._read_structure(trees)
        assert 3 not in ids.tolist()
        # re-thread it at the oldest state of every column, without recombinations
        nstates = np.zeros(prob.seqlen, dtype=np.int32)
        lib.arghmm_get_nstates(trees.handle, prob.ntimes, False,
                               nstates.ctypes.data_as(capi.c_int_p))
        path = np.zeros(prob.seqlen, dtype=np.int32)
        z = np.zeros(1, dtype=np.int32)
        p = lambda a: a.ctypes.data_as(capi.c_int_p)
        assert lib.awg_add_arg_thread(trees.handle, prob.ntimes, p(path), prob.seqlen, p(z),
                                      p(z), p(z), 0) == 0, capi.last_error()
        _, _, ids = refapi._read_structure(trees)
        assert sorted(ids.tolist()) == list(range((prob.nnodes + 1) // 2))
        assert ids[-1] == 3
    finally:
        trees.close()


RL_NAMES = sorted(f[:-4] for f in os.listdir(os.path.join(GOLDEN, "resampleleaf")) if f.endswith(".npz"))


@pytest.mark.parametrize("name", RL_NAMES)
def test_leaf_resampling_move_matches_reference(name):
    """resample_arg_leaf's move (sample_arg.cpp:66-86) on one handle: the sequence removed
    (awg_remove_arg_thread), re-threaded by the oracle's traceback and recombination sampler
    on the reference's draws after srand(seed), added back (awg_add_arg_thread, which gives the
    new leaf the freed sequence id); the ARG, leaves named by sequence, is the reference's."""
    import pyoracle
    ref = np.load(os.path.join(GOLDEN, "resampleleaf", name + ".npz"))
    full = grown(name).normalized()
    lib = capi.load()
    trees = refapi._trees_handle(full)
    try:
        assert lib.awg_remove_arg_thread(trees.handle, int(ref["seqid"])) == 0
        partial = refapi.as_problem(full, refapi._tree_dict(trees))
        L = partial.seqlen
        draws = pyoracle.rand_uniforms(int(ref["seed"]), 3 * L + 2)[::-1]
        fw, _ = pyoracle.forward(partial)
        path = pyoracle.traceback(partial, fw, draws[:L][::-1].copy())
        pos, node, time, _ = pyoracle.sample_recombinations(partial, path, draws[L:].copy())
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        path, pos, node, time = i32(path), i32(pos), i32(node), i32(time)
        p = lambda a: a.ctypes.data_as(capi.c_int_p)
        assert lib.awg_add_arg_thread(trees.handle, full.ntimes, p(path), L, p(pos), p(node),
                                      p(time), len(pos)) == 0, capi.last_error()
        got = refapi._tree_dict(trees)
    finally:
        trees.close()
    assert sorted(got["seqids"].tolist()) == list(range((full.nnodes + 1) // 2))
    for key in ("ptrees", "ages", "blocklens"):
        np.testing.assert_array_equal(got[key], ref[key], err_msg=key)
    np.testing.assert_array_equal(got["sprs"][1:], ref["sprs"][1:])
    np.testing.assert_array_equal(got["mapping"][1:], ref["mapping"][1:])


def test_sample_arg_thread_rejects_a_leafs_sequence():
    """awg_sample_arg_thread threads only a sequence no leaf holds (checked before any device
    work)."""
    full = grown("single_k7_s41").normalized()
    lib = capi.load()
    trees = refapi._trees_handle(full)
    try:
        seqs, _keep = refapi._char_pp(full.seqs)
        rc = lib.awg_sample_arg_thread(trees.handle, full.times.ctypes.data_as(capi.c_double_p),
                                       full.ntimes, full.popsizes.ctypes.data_as(capi.c_double_p),
                                       full.rho, full.mu, seqs, full.nseqs, full.seqlen, 2)
        assert rc == -1 and "no leaf holds" in capi.last_error()
    finally:
        trees.close()
