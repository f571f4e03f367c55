"""Adding a sampled thread to the ARG (add_arg_thread, thread.cpp:272-422) on the host:
the grown trees, SPRs, block lengths and node mappings equal the reference's for the
recombination fixtures' threads and recombinations."""

import ctypes as C
import glob
import os

import numpy as np
import pytest

from argweaver_gb300 import capi, refapi
from argweaver_gb300.problem import Problem
from conftest import GOLDEN, load_golden

NAMES = sorted(os.path.basename(p)[:-5] for p in glob.glob(os.path.join(GOLDEN, "addthread", "*.prob")))


def case(name):
    rec = np.load(os.path.join(GOLDEN, "recomb", name + ".npz"))
    if name.startswith("extra_"):
        return Problem.load(os.path.join(GOLDEN, "recomb", name + ".prob")), rec["path"], rec
    prob, gold = load_golden(name)
    return prob, gold["path"], rec


def grown(prob, path, pos, node, time):
    """(ptrees, ages, sprs, blocklens, mapping) of the trees after awg_add_arg_thread."""
    lib = capi.load()
    trees = refapi.LocalTrees(prob)
    try:
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        if prob.mapping is not None or prob.root_child0 is not None:
            mp = None if prob.mapping is None else i32(prob.mapping)
            rc0 = None if prob.root_child0 is None else i32(prob.root_child0)
            assert lib.awg_local_trees_set_structure(
                trees.handle, None if mp is None else mp.ctypes.data_as(capi.c_int_p),
                None if rc0 is None else rc0.ctypes.data_as(capi.c_int_p)) == 0
        path, pos, node, time = i32(path), i32(pos), i32(node), i32(time)
        p = lambda a: a.ctypes.data_as(capi.c_int_p)
        rc = lib.awg_add_arg_thread(trees.handle, prob.ntimes, p(path), len(path), p(pos),
                                    p(node), p(time), len(pos))
        if rc != 0:
            raise ValueError(capi.last_error())
        nt = lib.get_local_trees_ntrees(trees.handle)
        nn = lib.get_local_trees_nnodes(trees.handle)
        pt, ag, sp = (np.zeros((nt, k), dtype=np.int32) for k in (nn, nn, 4))
        bl = np.zeros(nt, dtype=np.int32)
        rows = lambda a: (capi.c_int_p * nt)(*[a[i].ctypes.data_as(capi.c_int_p) for i in range(nt)])
        lib.get_local_trees_ptrees(trees.handle, rows(pt), rows(ag), rows(sp), p(bl))
        mp = np.zeros((nt, nn), dtype=np.int32)
        assert lib.awg_local_trees_mapping(trees.handle, p(mp)) == 0
    finally:
        trees.close()
    return pt, ag, sp, bl, mp


@pytest.mark.parametrize("name", NAMES)
def test_add_thread_matches_reference(name):
    prob, path, rec = case(name)
    ref = Problem.load(os.path.join(GOLDEN, "addthread", name + ".prob"))
    pt, ag, sp, bl, mp = grown(prob, path, rec["pos"], rec["node"], rec["time"])
    assert pt.shape == ref.ptrees.shape
    np.testing.assert_array_equal(pt, ref.ptrees)
    np.testing.assert_array_equal(ag, ref.ages)
    np.testing.assert_array_equal(sp[1:], ref.sprs[1:])
    np.testing.assert_array_equal(bl, ref.blocklens)
    np.testing.assert_array_equal(mp[1:], ref.mapping[1:])
    assert pt.shape[0] == prob.ntrees + len(rec["pos"])


def test_add_thread_rejects_bad_input():
    prob, path, rec = case("sim1_c20")
    with pytest.raises(ValueError, match="state"):
        bad = np.array(path, dtype=np.int32)
        bad[0] = 10 ** 6
        grown(prob, bad, rec["pos"], rec["node"], rec["time"])
    with pytest.raises(ValueError, match="increase"):
        grown(prob, path, rec["pos"][::-1], rec["node"][::-1], rec["time"][::-1])


ST_NAMES = sorted(os.path.basename(p)[:-5] for p in glob.glob(os.path.join(GOLDEN, "samplethread", "*.prob")))


@pytest.mark.parametrize("name", ST_NAMES)
def test_threading_step_on_the_host_matches_reference(name):
    # arghmm_sample_thread's steps with the device ones replaced by the oracle (pinned to
    # the reference): the traceback's rand() draws, then the recombination sampler's draws
    # continuing rand(), then the thread added by this library; the grown ARG must be the
    # reference's, so the composite export's draw order and glue are those of the reference
    import pyoracle
    prob, _ = load_golden(name)
    ref = Problem.load(os.path.join(GOLDEN, "samplethread", name + ".prob"))
    seed = int(np.load(os.path.join(GOLDEN, "samplethread", name + ".npz"))["seed"])
    L = prob.seqlen
    libc = C.CDLL(None)
    libc.srand(C.c_uint(seed))
    d = np.array([libc.rand() / 2147483647.0 for _ in range(L + 2 * L + 2)])
    fw, _ = pyoracle.forward(prob)
    path = pyoracle.traceback(prob, fw, d[:L][::-1].copy())
    pos, node, time, used = pyoracle.sample_recombinations(prob, path, d[L:])
    pt, ag, sp, bl, mp = grown(prob, path, pos, node, time)
    np.testing.assert_array_equal(pt, ref.ptrees)
    np.testing.assert_array_equal(ag, ref.ages)
    np.testing.assert_array_equal(sp[1:], ref.sprs[1:])
    np.testing.assert_array_equal(bl, ref.blocklens)
    np.testing.assert_array_equal(mp[1:], ref.mapping[1:])
