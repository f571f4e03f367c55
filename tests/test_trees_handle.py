"""Trees-handle utilities of the reference's C interface (local_tree.cpp:1827-1958):
read_local_trees from an SMC file equals the reference's ingest of the same file (at
compression 1 the blocks keep their lengths), arghmm_copy_trees is independent of its source,
get_local_trees_blocks tiles the region and get_treelens sums branch lengths in node order."""

import ctypes as C
import os

import numpy as np

from argweaver_gb300 import capi, refapi
from argweaver_gb300.problem import Problem
from conftest import GOLDEN

FMT = os.path.join(GOLDEN, "formats")


def _read(path, times):
    lib = capi.load()
    t = np.ascontiguousarray(times, dtype=np.float64)
    h = lib.read_local_trees(path.encode(), t.ctypes.data_as(capi.c_double_p), len(t))
    assert h, capi.last_error()
    return h


def _arrays(h):
    lib = capi.load()
    nt, nn = lib.get_local_trees_ntrees(h), lib.get_local_trees_nnodes(h)
    pt, ag, sp = (np.zeros((nt, k), dtype=np.int32) for k in (nn, nn, 4))
    bl = np.zeros(nt, dtype=np.int32)
    rows = lambda a: (capi.c_int_p * nt)(*[a[i].ctypes.data_as(capi.c_int_p) for i in range(nt)])
    lib.get_local_trees_ptrees(h, rows(pt), rows(ag), rows(sp), bl.ctypes.data_as(capi.c_int_p))
    return pt, ag, sp, bl


def test_read_local_trees_matches_reference_ingest():
    ref = Problem.load(os.path.join(FMT, "k8_c1.prob"))
    lib = capi.load()
    h = _read(os.path.join(FMT, "k8.smc"), ref.times)
    try:
        pt, ag, sp, bl = _arrays(h)
        np.testing.assert_array_equal(pt, ref.ptrees)
        np.testing.assert_array_equal(ag, ref.ages)
        np.testing.assert_array_equal(sp[1:], ref.sprs[1:])
        np.testing.assert_array_equal(bl, ref.blocklens)
        starts = np.zeros(len(bl), dtype=np.int32)
        ends = np.zeros(len(bl), dtype=np.int32)
        lib.get_local_trees_blocks(h, starts.ctypes.data_as(capi.c_int_p),
                                   ends.ctypes.data_as(capi.c_int_p))
        assert starts[0] == ref.start_coord and np.all(starts[1:] == ends[:-1])
        np.testing.assert_array_equal(ends - starts, bl)
        # gzip input reads the same trees
        h2 = _read(os.path.join(FMT, "k16_missing.smc.gz"), ref.times)
        assert lib.get_local_trees_nnodes(h2) == 31
        lib.delete_local_trees(h2)
    finally:
        lib.delete_local_trees(h)


def test_read_local_trees_reports_missing_file():
    lib = capi.load()
    t = np.linspace(0, 1, 20)
    assert not lib.read_local_trees(b"/nonexistent.smc", t.ctypes.data_as(capi.c_double_p), 20)
    assert "cannot read" in capi.last_error()


def test_copy_and_treelens():
    ref = Problem.load(os.path.join(FMT, "k8_c1.prob"))
    lib = capi.load()
    h = _read(os.path.join(FMT, "k8.smc"), ref.times)
    h2 = lib.arghmm_copy_trees(h)
    try:
        lib.delete_local_trees(h)
        h = None
        pt, ag, _, _ = _arrays(h2)  # the copy outlives its source
        np.testing.assert_array_equal(pt, ref.ptrees)
        lens = np.zeros(len(pt), dtype=np.float64)
        lib.get_treelens(h2, ref.times.ctypes.data_as(capi.c_double_p), ref.ntimes,
                         lens.ctypes.data_as(capi.c_double_p))
        for b in range(len(pt)):
            want = 0.0
            for i in range(pt.shape[1]):
                if pt[b, i] != -1:
                    want += ref.times[ag[b, pt[b, i]]] - ref.times[ag[b, i]]
            assert lens[b] == want
    finally:
        if h:
            lib.delete_local_trees(h)
        lib.delete_local_trees(h2)
