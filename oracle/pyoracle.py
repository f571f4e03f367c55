"""ctypes binding of the CPU restatement (awg_oracle.cpp).

Test infrastructure: imported only by tests/, __graft_entry__.smoke() and bench.py's CPU
leg, as the checker the CUDA path is compared against. It never feeds the product path.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
_lib = None


class OracleProblem(C.Structure):
    _fields_ = [("ntrees", C.c_int), ("nnodes", C.c_int), ("ntimes", C.c_int),
                ("nseqs", C.c_int), ("seqlen", C.c_int), ("internal", C.c_int),
                ("start_coord", C.c_int), ("minage", C.c_int),
                ("ptrees", C.c_void_p), ("ages", C.c_void_p), ("sprs", C.c_void_p),
                ("blocklens", C.c_void_p), ("mapping", C.c_void_p),
                ("root_child0", C.c_void_p), ("times", C.c_void_p),
                ("popsizes", C.c_void_p), ("rho", C.c_double), ("mu", C.c_double),
                ("seqs", C.c_void_p), ("infsites_penalty", C.c_double)]


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    return LIB


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        lib = C.CDLL(LIB)
        P = C.POINTER(OracleProblem)
        for name, args in [("oracle_nstates", [P, C.c_void_p]),
                           ("oracle_forward", [P, C.c_void_p, C.c_void_p]),
                           ("oracle_traceback", [P, C.c_void_p, C.c_void_p, C.c_void_p]),
                           ("oracle_traceback_given", [P, C.c_void_p, C.c_void_p, C.c_void_p,
                                                       C.c_void_p]),
                           ("oracle_traceback_last", [P, C.c_void_p, C.c_void_p, C.c_void_p,
                                                      C.c_int, C.c_void_p]),
                           ("oracle_forward_prior", [P, C.c_void_p, C.c_void_p, C.c_void_p]),
                           ("oracle_traceback_split", [P, C.c_void_p, C.c_void_p, C.c_void_p,
                                                       C.c_void_p]),
                           ("oracle_backward", [P, C.c_void_p]),
                           ("oracle_posterior", [P, C.c_void_p, C.c_void_p, C.c_void_p]),
                           ("oracle_block_terms", [P, C.c_void_p, C.c_void_p]),
                           ("oracle_emissions", [P, C.c_void_p]),
                           ("oracle_dense_matrices", [P, C.c_int, C.c_void_p, C.c_void_p]),
                           ("oracle_debug_tables", [P, C.c_void_p, C.c_void_p, C.c_void_p,
                                                    C.c_void_p]),
                           ("oracle_dense_forward", [C.c_int, C.c_int] + [C.c_void_p] * 3),
                           ("oracle_dense_backward", [C.c_int, C.c_int] + [C.c_void_p] * 3),
                           ("oracle_dense_sample", [C.c_int, C.c_int] + [C.c_void_p] * 4),
                           ("oracle_arg_prob", [P, C.c_void_p]),
                           ("oracle_sample_recombinations", [P, C.c_void_p, C.c_void_p, C.c_int,
                                                             C.c_void_p, C.c_void_p, C.c_void_p,
                                                             C.c_int, C.c_void_p])]:
            fn = getattr(lib, name)
            fn.restype = C.c_int
            fn.argtypes = args
        lib.oracle_cells.restype = C.c_longlong
        lib.oracle_cells.argtypes = [P]
        _lib = lib
    return _lib


class Bound:
    """A problem pinned in memory with its C view."""

    def __init__(self, prob):
        self.p = prob.normalized()
        p = self.p
        ptr = lambda a: None if a is None else a.ctypes.data
        self.c = OracleProblem(p.ntrees, p.nnodes, p.ntimes, p.nseqs, p.seqlen,
                               int(p.internal), p.start_coord, 0,
                               ptr(p.ptrees), ptr(p.ages), ptr(p.sprs), ptr(p.blocklens),
                               ptr(p.mapping), ptr(p.root_child0), ptr(p.times),
                               ptr(p.popsizes), p.rho, p.mu, ptr(p.seqs),
                               float(p.infsites_penalty))

    @property
    def ref(self):
        return C.byref(self.c)


def _check(rc, what):
    if rc != 0:
        raise ValueError(f"oracle {what} rejected the problem (code {rc})")


def nstates(prob) -> np.ndarray:
    b = Bound(prob)
    out = np.zeros(prob.seqlen, dtype=np.int32)
    _check(load().oracle_nstates(b.ref, out.ctypes.data), "nstates")
    return out


def offsets(ns: np.ndarray) -> np.ndarray:
    off = np.zeros(ns.shape[0] + 1, dtype=np.int64)
    np.cumsum(np.maximum(ns, 1), out=off[1:])
    return off


def forward(prob, prior=None):
    """Packed forward table and the log-likelihood from the column norms; with ``prior``,
    column 0 holds those values instead of the state priors."""
    b = Bound(prob)
    lib = load()
    ncells = lib.oracle_cells(b.ref)
    if ncells < 0:
        raise ValueError("oracle rejected the problem")
    fw = np.zeros(ncells, dtype=np.float64)
    lnl = C.c_double(0.0)
    pr = None if prior is None else np.ascontiguousarray(prior, dtype=np.float64)
    _check(lib.oracle_forward_prior(b.ref, None if pr is None else pr.ctypes.data,
                                    fw.ctypes.data, C.addressof(lnl)), "forward")
    return fw, lnl.value


def traceback_last(prob, fw: np.ndarray, u: np.ndarray, last_state: int) -> np.ndarray:
    """The reference's scan with the last column's state given (no draw there)."""
    b = Bound(prob)
    fw = np.ascontiguousarray(fw, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    path = np.zeros(prob.seqlen, dtype=np.int32)
    _check(load().oracle_traceback_last(b.ref, fw.ctypes.data, u.ctypes.data, None,
                                        int(last_state), path.ctypes.data), "traceback")
    return path


def traceback(prob, fw: np.ndarray, u: np.ndarray, given=None) -> np.ndarray:
    """The reference's scan (sample_hmm_posterior). With ``given``, column i draws
    conditioned on given[i + 1] instead of the path drawn so far."""
    b = Bound(prob)
    fw = np.ascontiguousarray(fw, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    g = None if given is None else np.ascontiguousarray(given, dtype=np.int32)
    path = np.zeros(prob.seqlen, dtype=np.int32)
    _check(load().oracle_traceback_given(b.ref, fw.ctypes.data, u.ctypes.data,
                                         None if g is None else g.ctypes.data,
                                         path.ctypes.data), "traceback")
    return path


def traceback_split(prob, fw: np.ndarray, u: np.ndarray, given=None) -> np.ndarray:
    """The FP32 path's decomposed draw (same distribution, another uniform-to-state map).
    With ``given``, column i draws conditioned on given[i + 1]."""
    b = Bound(prob)
    fw = np.ascontiguousarray(fw, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    g = None if given is None else np.ascontiguousarray(given, dtype=np.int32)
    path = np.zeros(prob.seqlen, dtype=np.int32)
    _check(load().oracle_traceback_split(b.ref, fw.ctypes.data, u.ctypes.data,
                                         None if g is None else g.ctypes.data,
                                         path.ctypes.data), "split traceback")
    return path


def backward(prob) -> np.ndarray:
    b = Bound(prob)
    lib = load()
    bw = np.zeros(lib.oracle_cells(b.ref), dtype=np.float64)
    _check(lib.oracle_backward(b.ref, bw.ctypes.data), "backward")
    return bw


def posterior(prob, fw: np.ndarray, bw: np.ndarray) -> np.ndarray:
    b = Bound(prob)
    post = np.zeros_like(fw)
    _check(load().oracle_posterior(b.ref, np.ascontiguousarray(fw).ctypes.data,
                                   np.ascontiguousarray(bw).ctypes.data, post.ctypes.data),
           "posterior")
    return post


def block_terms(prob):
    b = Bound(prob)
    T = prob.ntimes
    out = np.zeros((prob.ntrees, 9, T), dtype=np.float64)
    minage = np.zeros(prob.ntrees, dtype=np.int32)
    _check(load().oracle_block_terms(b.ref, out.ctypes.data, minage.ctypes.data), "terms")
    return out, minage


def dense_matrices(prob, b: int, switch: bool = False):
    """Tree b's log transition matrix [S][S] and, with switch (b > 0), the log switch
    matrix [S1][S2] from tree b - 1, states in the reference's get_coal_states order."""
    bd = Bound(prob)
    ns = prob.nstates_per_tree()
    S = int(ns[b])
    trans = np.zeros((S, S))
    sw = np.zeros((int(ns[b - 1]), S)) if switch else None
    _check(load().oracle_dense_matrices(bd.ref, b, trans.ctypes.data,
                                        sw.ctypes.data if switch else None), "dense matrices")
    return (trans, sw) if switch else trans


def emissions(prob) -> np.ndarray:
    b = Bound(prob)
    lib = load()
    out = np.zeros(lib.oracle_cells(b.ref), dtype=np.float64)
    _check(lib.oracle_emissions(b.ref, out.ctypes.data), "emissions")
    return out


def debug_tables(prob):
    """tmatrix, same-branch rows, invariant emissions and prior, GPU table-kernel layout."""
    b = Bound(prob)
    T = prob.ntimes
    S = prob.nstates_per_tree()
    M = 0
    for t in range(prob.ntrees):
        par, age = prob.ptrees[t], prob.ages[t]
    tm = np.zeros(prob.ntrees * (T - 1) * (T - 1))
    # sizes from the host-side state spaces
    Mtot = _total_M(prob)
    gts = np.zeros(max(Mtot, 1))
    inv = np.zeros(int(np.maximum(S, 1).sum()))
    prior = np.zeros(max(int(S[0]), 1))
    _check(load().oracle_debug_tables(b.ref, tm.ctypes.data, gts.ctypes.data, inv.ctypes.data,
                                      prior.ctypes.data), "debug tables")
    return tm.reshape(prob.ntrees, T - 1, T - 1), gts[:Mtot], inv, prior


def _total_M(prob) -> int:
    ns = nstates(prob)
    del ns
    T = prob.ntimes
    tot = 0
    for t in range(prob.ntrees):
        par, age = prob.ptrees[t], prob.ages[t]
        if not prob.internal:
            for v in range(prob.nnodes):
                top = T - 2 if par[v] == -1 else age[par[v]]
                m = max(0, top - age[v] + 1)
                tot += m * m
        else:
            raise NotImplementedError("debug tables: external problems only")
    return tot


def rand_uniforms(seed: int, n: int) -> np.ndarray:
    """The uniforms the reference's traceback draws after srand(seed): rand()/RAND_MAX,
    one per column, last column first (sample_thread.cpp:537, common.h:103-110).
    Returned indexed by column."""
    libc = C.CDLL(None)
    libc.srand(C.c_uint(seed))
    rmax = 2147483647.0  # glibc RAND_MAX
    draws = np.array([libc.rand() / rmax for _ in range(n)], dtype=np.float64)
    return draws[::-1].copy()


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def dense_forward(trans, emit, fw0) -> np.ndarray:
    """The dense forward table (hmm.cpp:27-43) from its first column fw0."""
    trans, emit = _f64(trans), _f64(emit)
    fw = np.zeros_like(emit)
    fw[0] = fw0
    _check(load().oracle_dense_forward(emit.shape[0], emit.shape[1], trans.ctypes.data,
                                       emit.ctypes.data, fw.ctypes.data), "dense forward")
    return fw


def dense_backward(trans, emit, bwlast) -> np.ndarray:
    """The dense backward table (hmm.cpp:48-64) from its last column bwlast."""
    trans, emit = _f64(trans), _f64(emit)
    bw = np.zeros_like(emit)
    bw[-1] = bwlast
    _check(load().oracle_dense_backward(emit.shape[0], emit.shape[1], trans.ctypes.data,
                                        emit.ctypes.data, bw.ctypes.data), "dense backward")
    return bw


def dense_sample(trans, fw, u, last: int) -> np.ndarray:
    """A path drawn by sample_hmm_posterior (hmm.cpp:67-85) with uniforms u by column."""
    trans, fw, u = _f64(trans), _f64(fw), _f64(u)
    path = np.zeros(fw.shape[0], dtype=np.int32)
    path[-1] = last
    _check(load().oracle_dense_sample(fw.shape[0], fw.shape[1], trans.ctypes.data,
                                      fw.ctypes.data, u.ctypes.data, path.ctypes.data),
           "dense sample")
    return path


def arg_prob(prob) -> np.ndarray:
    """(log-likelihood, ARG prior, first-tree prior) of the problem's ARG (total_prob.cpp)."""
    b = Bound(prob)
    out = np.zeros(3)
    _check(load().oracle_arg_prob(b.ref, out.ctypes.data), "ARG probability")
    return out


def sample_recombinations(prob, path, u):
    """(columns, nodes, times, draws used) of sample_recombinations (recomb.cpp:151-235)
    along `path` with the draws `u` in order."""
    b = Bound(prob)
    path = np.ascontiguousarray(path, dtype=np.int32)
    u = np.ascontiguousarray(u, dtype=np.float64)
    L = prob.seqlen
    pos, node, time = (np.zeros(L, dtype=np.int32) for _ in range(3))
    used = np.zeros(1, dtype=np.int32)
    n = load().oracle_sample_recombinations(b.ref, path.ctypes.data, u.ctypes.data, len(u),
                                            pos.ctypes.data, node.ctypes.data, time.ctypes.data,
                                            L, used.ctypes.data)
    if n < 0:
        raise ValueError(f"oracle sample_recombinations failed ({n})")
    return pos[:n].copy(), node[:n].copy(), time[:n].copy(), int(used[0])

