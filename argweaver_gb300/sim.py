"""Seeded threading problems from the DSMC generator (csrc/sim.cpp).

``simulate`` returns a :class:`~argweaver_gb300.problem.Problem`; with ``add_thread`` the
ARG has ``nleaves`` leaves and one more sequence to thread (external threading, as
``sample_arg_thread``, src/argweaver/sample_thread.cpp:578), otherwise it is a full ARG
whose sequences match its leaves.
"""

from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from .problem import Problem

_lock = threading.Lock()
_lib = None


class _Params(C.Structure):
    _fields_ = [("nleaves", C.c_int), ("seqlen", C.c_int), ("compress", C.c_int),
                ("ntimes", C.c_int), ("add_thread", C.c_int), ("pad", C.c_int),
                ("maxtime", C.c_double), ("popsize", C.c_double), ("rho", C.c_double),
                ("mu", C.c_double), ("missing", C.c_double), ("seed", C.c_ulonglong)]


class _Result(C.Structure):
    _fields_ = [("ntrees", C.c_int), ("nnodes", C.c_int), ("nseqs", C.c_int),
                ("seqlen", C.c_int), ("ntimes", C.c_int),
                ("ptrees", C.POINTER(C.c_int)), ("ages", C.POINTER(C.c_int)),
                ("sprs", C.POINTER(C.c_int)), ("blocklens", C.POINTER(C.c_int)),
                ("mapping", C.POINTER(C.c_int)), ("seqs", C.POINTER(C.c_char)),
                ("path_node", C.POINTER(C.c_int)), ("path_time", C.POINTER(C.c_int)),
                ("times", C.POINTER(C.c_double)), ("popsizes", C.POINTER(C.c_double)),
                ("rho", C.c_double), ("mu", C.c_double)]


def _load():
    global _lib
    with _lock:
        if _lib is None:
            from . import build
            path = build.SIM_LIB
            if not os.path.exists(path):
                build.build_sim()
            lib = C.CDLL(path)
            lib.awg_sim_run.restype = C.POINTER(_Result)
            lib.awg_sim_run.argtypes = [C.POINTER(_Params)]
            lib.awg_sim_free.restype = None
            lib.awg_sim_free.argtypes = [C.POINTER(_Result)]
            _lib = lib
    return _lib


def simulate(nleaves: int, seqlen: int, seed: int, *, compress: int = 10, ntimes: int = 20,
             maxtime: float = 200e3, popsize: float = 1e4, rho: float = 1.6e-8,
             mu: float = 1.8e-8, missing: float = 0.0, add_thread: bool = True) -> Problem:
    """Simulate one seeded problem in compressed columns (``seqlen`` columns of
    ``compress`` bp; rho and mu per bp)."""
    lib = _load()
    p = _Params(nleaves, seqlen, compress, ntimes, 1 if add_thread else 0, 0, maxtime,
                popsize, rho, mu, missing, seed & 0xFFFFFFFFFFFFFFFF)
    r = lib.awg_sim_run(C.byref(p))
    if not r:
        raise ValueError("invalid simulation parameters")
    try:
        res = r.contents
        nt, nn, ns, L, T = res.ntrees, res.nnodes, res.nseqs, res.seqlen, res.ntimes

        def arr(ptr, count, dt, shape):
            return np.ctypeslib.as_array(ptr, shape=(count,)).astype(dt).reshape(shape)

        prob = Problem(
            times=arr(res.times, T, np.float64, (T,)),
            popsizes=arr(res.popsizes, T, np.float64, (T,)),
            rho=float(res.rho), mu=float(res.mu),
            ptrees=arr(res.ptrees, nt * nn, np.int32, (nt, nn)),
            ages=arr(res.ages, nt * nn, np.int32, (nt, nn)),
            sprs=arr(res.sprs, nt * 4, np.int32, (nt, 4)),
            blocklens=arr(res.blocklens, nt, np.int32, (nt,)),
            seqs=np.frombuffer(C.string_at(res.seqs, ns * L), dtype=np.uint8)
                 .reshape(ns, L).copy(),
            mapping=arr(res.mapping, nt * nn, np.int32, (nt, nn)),
            path_node=arr(res.path_node, L, np.int32, (L,)) if add_thread else None,
            path_time=arr(res.path_time, L, np.int32, (L,)) if add_thread else None,
        )
    finally:
        lib.awg_sim_free(r)
    return prob


def leaf_cut(p: Problem) -> Problem:
    """The internal-branch form of an external threading problem: the threaded haplotype
    becomes leaf k of a (k+1)-leaf tree whose root is the virtual root of a cut
    (age ntimes+1), with child[0] the cut subtree (the single leaf k) and child[1] the main
    tree, the layout remove_arg_thread_path leaves for a removed leaf (thread.cpp:1481,
    states.cpp:109-167). Nodes are renumbered leaves first (main leaves 0..k-1, leaf k, the
    main tree's internal nodes, the virtual root last); SPRs and node maps follow."""
    k = (p.nnodes + 1) // 2            # leaves of the main trees
    n2 = p.nnodes + 2
    T = p.ntimes
    remap = np.arange(p.nnodes + 1, dtype=np.int64)
    remap[k:p.nnodes] = np.arange(k, p.nnodes) + 1
    vroot, leaf = n2 - 1, k

    def rm(v):
        return np.where(v >= 0, remap[np.maximum(v, 0)], -1)

    B = p.ntrees
    ptrees = np.empty((B, n2), dtype=np.int32)
    ages = np.empty((B, n2), dtype=np.int32)
    for b in range(B):
        par = p.ptrees[b]
        newp = rm(par)
        newp[par == -1] = vroot
        ptrees[b, remap[:p.nnodes]] = newp
        ages[b, remap[:p.nnodes]] = p.ages[b]
        ptrees[b, leaf], ages[b, leaf] = vroot, 0
        ptrees[b, vroot], ages[b, vroot] = -1, T + 1
    sprs = p.sprs.copy()
    sprs[:, 0] = rm(sprs[:, 0])
    sprs[:, 2] = rm(sprs[:, 2])
    mapping = None
    if p.mapping is not None:
        mapping = np.empty((B, n2), dtype=np.int32)
        for b in range(B):
            mapping[b, remap[:p.nnodes]] = rm(p.mapping[b])
            mapping[b, leaf], mapping[b, vroot] = leaf, vroot
    return Problem(times=p.times, popsizes=p.popsizes, rho=p.rho, mu=p.mu, ptrees=ptrees,
                   ages=ages, sprs=sprs, blocklens=p.blocklens.copy(), seqs=p.seqs.copy(),
                   internal=True, mapping=mapping,
                   root_child0=np.full(B, leaf, dtype=np.int32))
