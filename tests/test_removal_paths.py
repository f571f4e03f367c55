"""Removal paths and the internal-branch cut on the host (thread.cpp:562-1002,1481-1668):
after srand(seed) the uniform path, its log path count, the forward path from a node, the
path through a node at a position, the leaf path and the path preferring recombinations
equal the reference's draws, and the ARG cut along the uniform path (subtree/main-tree form,
merged trees, mappings, root child order, the removed thread as states of the cut trees)
equals the reference's."""

import os

import numpy as np
import pytest

from argweaver_gb300 import refapi
from argweaver_gb300.problem import Problem
from conftest import GOLDEN

NAMES = sorted(f[:-4] for f in os.listdir(os.path.join(GOLDEN, "removalpaths")) if f.endswith(".npz"))


def grown(name):
    return Problem.load(os.path.join(GOLDEN, "addthread", name + ".prob"))


@pytest.mark.parametrize("name", NAMES)
def test_removal_paths_match_reference(name):
    ref = np.load(os.path.join(GOLDEN, "removalpaths", name + ".npz"))
    prob = grown(name)
    node, pos = int(ref["node"]), int(ref["pos"])
    refapi.srand(int(ref["seed"]))
    upath, lntotal = refapi.sample_arg_removal_path_uniform(prob)
    fpath = refapi.sample_arg_removal_path(prob, node)
    ppath = refapi.sample_arg_removal_path(prob, node, pos)
    lpath = refapi.sample_arg_removal_path(prob, 0, leaf=True)
    rpath = refapi.sample_arg_removal_path_recomb(prob, 0.9)
    paths = ref["paths"]
    np.testing.assert_array_equal(upath, paths[0])
    assert lntotal == float(ref["lntotal"])
    np.testing.assert_array_equal(fpath, paths[1])
    np.testing.assert_array_equal(ppath, paths[2])
    np.testing.assert_array_equal(lpath, paths[3])
    np.testing.assert_array_equal(rpath, paths[4])


@pytest.mark.parametrize("name", NAMES)
def test_cut_matches_reference(name):
    ref = np.load(os.path.join(GOLDEN, "removalpaths", name + ".npz"))
    got = refapi.remove_arg_thread_path(grown(name), ref["paths"][0], original_thread=True)
    np.testing.assert_array_equal(got["original_thread"], ref["original_thread"])
    assert got["ptrees"].shape == ref["ptrees"].shape
    for key in ("ptrees", "ages", "sprs", "blocklens", "root_child0"):
        np.testing.assert_array_equal(got[key], ref[key], err_msg=key)
    np.testing.assert_array_equal(got["mapping"][1:], ref["mapping"][1:])


def test_leaf_path_stays_on_the_leaf():
    prob = grown("dsmc_k10_T16")
    for leaf in range((prob.nnodes + 1) // 2):
        np.testing.assert_array_equal(refapi.sample_arg_removal_path(prob, leaf, leaf=True), leaf)


def test_cut_along_leaf_path_gives_internal_trees():
    """A leaf's path cuts that leaf out of every tree: each root is at maxtime with the leaf
    as its first child, and the region is kept."""
    prob = grown("dsmc_k8_s12")
    path = refapi.sample_arg_removal_path(prob, 4, leaf=True)
    got = refapi.remove_arg_thread_path(prob, path)
    roots = np.argmax(got["ptrees"] == -1, axis=1)
    assert np.all(got["ages"][np.arange(len(roots)), roots] == prob.ntimes + 1)
    assert np.all(got["root_child0"] == 4)
    assert int(got["blocklens"].sum()) == int(np.sum(prob.blocklens))


def test_bad_inputs_raise():
    prob = grown("single_k7_s41")
    with pytest.raises(ValueError, match="pos"):
        refapi.sample_arg_removal_path(prob, 1, pos=prob.start_coord + 10 ** 9)
    with pytest.raises(ValueError, match="range"):
        refapi.sample_arg_removal_path(prob, prob.nnodes)
    with pytest.raises(ValueError, match="range"):
        refapi.remove_arg_thread_path(prob, np.full(prob.ntrees, prob.nnodes))
