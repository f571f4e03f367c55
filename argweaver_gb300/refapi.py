"""The reference's Python-facing threading-HMM calls, in Python 3, over this library.

Mirrors argweaver/argweaverc.py: ``argweaver_forward_algorithm`` (argweaverc.py:529-572),
``sample_posterior`` (the commented-out wrapper at argweaverc.py:611-649, here live) and
the raw prototypes, taking the same tree arrays the reference's ``get_treeset`` builds
(ptrees, ages, sprs, blocklens). Randomness follows the reference: libc rand(), seeded
with ``srand`` (argweaverc.py:347-354).
"""

from __future__ import annotations

import ctypes as C
from typing import List, Sequence

import numpy as np

from . import capi
from .problem import Problem

_libc = C.CDLL(None)


def srand(seed: int) -> None:
    """Seed libc's rand(), the generator the samplers draw from (common.h:103-110)."""
    _libc.srand(C.c_uint(seed))


def _int_matrix(a: np.ndarray):
    a = np.ascontiguousarray(a, dtype=np.int32)
    rows = (capi.c_int_p * a.shape[0])(*[a[i].ctypes.data_as(capi.c_int_p)
                                        for i in range(a.shape[0])])
    return rows, a


def _char_pp(seqs: np.ndarray):
    seqs = np.ascontiguousarray(seqs, dtype=np.uint8)
    rows = (C.c_char_p * seqs.shape[0])(*[bytes(seqs[i]) for i in range(seqs.shape[0])])
    return C.cast(rows, capi.c_char_pp), rows


class LocalTrees:
    """Handle from arghmm_new_trees (local_tree.cpp:1817); freed on close/delete."""

    def __init__(self, prob: Problem):
        lib = capi.load()
        p = prob.normalized()
        self._pt = _int_matrix(p.ptrees)
        self._ag = _int_matrix(p.ages)
        self._sp = _int_matrix(p.sprs)
        self._bl = p.blocklens
        self.handle = lib.arghmm_new_trees(self._pt[0], self._ag[0], self._sp[0],
                                           p.blocklens.ctypes.data_as(capi.c_int_p),
                                           p.ntrees, p.nnodes, p.start_coord)
        if not self.handle:
            raise ValueError(capi.last_error())
        # node mappings and root child order the parent arrays do not carry (an ARG after
        # surgery, e.g. an internal-branch cut), when the problem has them
        if p.mapping is not None or p.root_child0 is not None:
            mp = None if p.mapping is None else np.ascontiguousarray(p.mapping, dtype=np.int32)
            rc = None if p.root_child0 is None else np.ascontiguousarray(p.root_child0, dtype=np.int32)
            if lib.awg_local_trees_set_structure(
                    self.handle, None if mp is None else mp.ctypes.data_as(capi.c_int_p),
                    None if rc is None else rc.ctypes.data_as(capi.c_int_p)) != 0:
                raise ValueError(capi.last_error())

    def close(self):
        if self.handle:
            capi.load().delete_local_trees(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def get_nstates(trees: LocalTrees, ntimes: int, internal: bool, seqlen: int) -> np.ndarray:
    out = np.zeros(seqlen, dtype=np.int32)
    capi.load().arghmm_get_nstates(trees.handle, ntimes, internal,
                                   out.ctypes.data_as(capi.c_int_p))
    return out


def _rows_to_list(mat, nstates: np.ndarray) -> List[np.ndarray]:
    return [np.ctypeslib.as_array(mat[i], shape=(max(int(n), 1),)).copy()
            for i, n in enumerate(nstates)]


def arghmm_forward_alg(prob: Problem, prior: Sequence[float] = (), slow: bool = False
                       ) -> List[np.ndarray]:
    """Forward table as a list of per-column arrays, like argweaver_forward_algorithm."""
    lib = capi.load()
    p = prob.normalized()
    trees = LocalTrees(p)
    seqs, _keep = _char_pp(p.seqs)
    prior_arr = np.ascontiguousarray(prior, dtype=np.float64)
    fw = lib.arghmm_forward_alg(trees.handle, p.times.ctypes.data_as(capi.c_double_p),
                                p.ntimes, p.popsizes.ctypes.data_as(capi.c_double_p), p.rho,
                                p.mu, seqs, p.nseqs, p.seqlen, len(prior_arr) > 0,
                                prior_arr.ctypes.data_as(capi.c_double_p), p.internal, slow)
    if not fw:
        raise RuntimeError(capi.last_error())
    nstates = get_nstates(trees, p.ntimes, p.internal, p.seqlen)
    probs = _rows_to_list(fw, nstates)
    lib.delete_forward_matrix(fw, p.seqlen)
    trees.close()
    return probs


def _table_call(name: str, prob: Problem) -> List[np.ndarray]:
    lib = capi.load()
    p = prob.normalized()
    trees = LocalTrees(p)
    seqs, _keep = _char_pp(p.seqs)
    mat = getattr(lib, name)(trees.handle, p.times.ctypes.data_as(capi.c_double_p), p.ntimes,
                             p.popsizes.ctypes.data_as(capi.c_double_p), p.rho, p.mu, seqs,
                             p.nseqs, p.seqlen, p.internal)
    if not mat:
        raise RuntimeError(capi.last_error())
    nstates = get_nstates(trees, p.ntimes, p.internal, p.seqlen)
    out = _rows_to_list(mat, nstates)
    lib.delete_forward_matrix(mat, p.seqlen)
    trees.close()
    return out


def arghmm_backward_alg(prob: Problem) -> List[np.ndarray]:
    return _table_call("arghmm_backward_alg", prob)


def arghmm_posterior_marginals(prob: Problem) -> List[np.ndarray]:
    return _table_call("arghmm_posterior_marginals", prob)


def arghmm_sample_posterior(prob: Problem) -> np.ndarray:
    """(node, time) of the sampled thread per column (arghmm_sample_posterior)."""
    lib = capi.load()
    p = prob.normalized()
    pt, _a = _int_matrix(p.ptrees)
    ag, _b = _int_matrix(p.ages)
    sp, _c = _int_matrix(p.sprs)
    seqs, _keep = _char_pp(p.seqs)
    path = lib.arghmm_sample_posterior(pt, ag, sp, p.blocklens.ctypes.data_as(capi.c_int_p),
                                       p.ntrees, p.nnodes,
                                       p.times.ctypes.data_as(capi.c_double_p), p.ntimes,
                                       p.popsizes.ctypes.data_as(capi.c_double_p), p.rho, p.mu,
                                       seqs, p.nseqs, p.seqlen, None)
    if not path:
        raise RuntimeError(capi.last_error())
    out = np.ctypeslib.as_array(path, shape=(2 * p.seqlen,)).reshape(p.seqlen, 2).copy()
    lib.delete_path(path)
    return out


def arghmm_sample_arg_thread_internal(prob: Problem) -> np.ndarray:
    """State index per column of a sampled internal-branch thread."""
    lib = capi.load()
    p = prob.normalized()
    trees = LocalTrees(p)
    seqs, _keep = _char_pp(p.seqs)
    out = np.zeros(p.seqlen, dtype=np.int32)
    lib.arghmm_sample_arg_thread_internal(trees.handle, p.times.ctypes.data_as(capi.c_double_p),
                                          p.ntimes, p.popsizes.ctypes.data_as(capi.c_double_p),
                                          p.rho, p.mu, seqs, p.nseqs, p.seqlen,
                                          out.ctypes.data_as(capi.c_int_p))
    err = capi.last_error()
    trees.close()
    if err:
        raise RuntimeError(err)
    return out


# ----------------------------------------------------------------------------- dense HMM
# forward_alg / backward_alg / sample_hmm_posterior (argweaverc.py:42-56, hmm.cpp:27-85):
# the tables are filled in place, as the reference's c_out matrices are.

def _double_rows(a: np.ndarray, name: str):
    if a.dtype != np.float64 or a.ndim != 2 or not a.flags.c_contiguous:
        raise ValueError(f"{name} must be a C-contiguous 2-D float64 array")
    return (capi.c_double_p * a.shape[0])(*[a[i].ctypes.data_as(capi.c_double_p)
                                           for i in range(a.shape[0])])


def _dense_check(trans: np.ndarray, tab: np.ndarray):
    S = tab.shape[1]
    if trans.shape != (S, S):
        raise ValueError("trans must be nstates x nstates")
    return tab.shape[0], S


def forward_alg(trans: np.ndarray, emit: np.ndarray, fw: np.ndarray) -> np.ndarray:
    """Fill fw[1:] from fw[0] (the caller's) in place; log-space tables, n x nstates."""
    n, S = _dense_check(trans, fw)
    if emit.shape != fw.shape:
        raise ValueError("emit must have the shape of fw")
    capi.load().forward_alg(n, S, _double_rows(trans, "trans"), _double_rows(emit, "emit"),
                            _double_rows(fw, "fw"))
    err = capi.last_error()
    if err:
        raise RuntimeError(err)
    return fw


def backward_alg(trans: np.ndarray, emit: np.ndarray, bw: np.ndarray) -> np.ndarray:
    """Fill bw[:-1] from bw[-1] (the caller's) in place."""
    n, S = _dense_check(trans, bw)
    if emit.shape != bw.shape:
        raise ValueError("emit must have the shape of bw")
    capi.load().backward_alg(n, S, _double_rows(trans, "trans"), _double_rows(emit, "emit"),
                             _double_rows(bw, "bw"))
    err = capi.last_error()
    if err:
        raise RuntimeError(err)
    return bw


def sample_hmm_posterior(trans: np.ndarray, fw: np.ndarray, path: np.ndarray) -> np.ndarray:
    """Fill path[:-1] from path[-1] (the caller's) in place, one rand() per column."""
    n, S = _dense_check(trans, fw)
    if path.dtype != np.int32 or path.shape != (n,) or not path.flags.c_contiguous:
        raise ValueError("path must be a contiguous int32 array of n entries")
    capi.load().sample_hmm_posterior(n, S, _double_rows(trans, "trans"), _double_rows(fw, "fw"),
                                     path.ctypes.data_as(capi.c_int_p))
    err = capi.last_error()
    if err:
        raise RuntimeError(err)
    return path


# ----------------------------------------------------------------------------- ARG probabilities
# arghmm_likelihood / arghmm_prior_prob / arghmm_tree_prior_prob / arghmm_joint_prob
# (argweaverc.py:219-245, total_prob.cpp:315-382), computed on the GPU.

def _site_rows(p: Problem):
    """The problem's sequences as the reference indexes them: by absolute position, the
    trees' first site at start_coord (earlier positions padded with 'N')."""
    seqs = np.ascontiguousarray(p.seqs, dtype=np.uint8)
    if p.start_coord:
        pad = np.full((seqs.shape[0], p.start_coord), ord("N"), dtype=np.uint8)
        seqs = np.concatenate([pad, seqs], axis=1)
    return seqs


def _arg_call(prob: Problem, name: str) -> float:
    lib = capi.load()
    p = prob.normalized()
    trees = LocalTrees(p)
    rows = _site_rows(p)
    seqs, _keep = _char_pp(rows)
    times = p.times.ctypes.data_as(capi.c_double_p)
    pops = p.popsizes.ctypes.data_as(capi.c_double_p)
    try:
        if name == "likelihood":
            v = lib.arghmm_likelihood(trees.handle, times, p.ntimes, p.mu, seqs, p.nseqs,
                                      rows.shape[1])
        elif name == "prior":
            v = lib.arghmm_prior_prob(trees.handle, times, p.ntimes, pops, p.rho)
        elif name == "tree_prior":
            v = lib.arghmm_tree_prior_prob(trees.handle, times, p.ntimes, pops)
        else:
            v = lib.arghmm_joint_prob(trees.handle, times, p.ntimes, pops, p.mu, p.rho, seqs,
                                      p.nseqs, rows.shape[1])
        err = capi.last_error()
    finally:
        trees.close()
    if err:
        raise ValueError(err)
    return float(v)


def arghmm_likelihood(prob: Problem) -> float:
    """log P(sequences | ARG) (calc_arg_likelihood, total_prob.cpp:19-45)."""
    return _arg_call(prob, "likelihood")


def arghmm_prior_prob(prob: Problem) -> float:
    """log P(ARG): recombination spacing and SPRs (calc_arg_prior, total_prob.cpp:262-300)."""
    return _arg_call(prob, "prior")


def arghmm_tree_prior_prob(prob: Problem) -> float:
    """The first tree's coalescent prior (calc_tree_prior, total_prob.cpp:132-165)."""
    return _arg_call(prob, "tree_prior")


def arghmm_joint_prob(prob: Problem) -> float:
    """Likelihood + prior (calc_arg_joint_prob, total_prob.cpp:303-308)."""
    return _arg_call(prob, "joint")


def sample_recombinations(prob: Problem, path: np.ndarray, seed: int):
    """sample_recombinations (recomb.cpp:151-235) along `path` with the draws rand() gives
    after srand(seed), as the reference draws them: (columns, nodes, times, draws used).
    The generator is left as after those draws plus the unused ones (2 per column are
    drawn up front)."""
    from . import api
    srand(seed)
    n = 2 * prob.seqlen + 2
    u = np.array([_libc.rand() / 2147483647.0 for _ in range(n)], dtype=np.float64)
    return api.sample_recombinations(prob, path, u)



# ----------------------------------------------------------------------------- threading step
# arghmm_sample_thread (argweaverc.py:157-161, sample_thread.cpp:1010-1023): the last sequence
# threaded into the ARG (forward, traceback and recombinations on the GPU, the surgery on
# the host).

def _trees_handle(p: Problem) -> "LocalTrees":
    lib = capi.load()
    trees = LocalTrees(p)
    if p.mapping is not None or p.root_child0 is not None:
        mp = None if p.mapping is None else np.ascontiguousarray(p.mapping, dtype=np.int32)
        rc0 = None if p.root_child0 is None else np.ascontiguousarray(p.root_child0, dtype=np.int32)
        rc = lib.awg_local_trees_set_structure(
            trees.handle, None if mp is None else mp.ctypes.data_as(capi.c_int_p),
            None if rc0 is None else rc0.ctypes.data_as(capi.c_int_p))
        if rc != 0:
            trees.close()
            raise ValueError(capi.last_error())
    return trees


def _read_trees(trees: "LocalTrees"):
    lib = capi.load()
    nt = lib.get_local_trees_ntrees(trees.handle)
    nn = lib.get_local_trees_nnodes(trees.handle)
    pt, ag, sp = (np.zeros((nt, k), dtype=np.int32) for k in (nn, nn, 4))
    bl = np.zeros(nt, dtype=np.int32)
    rows = lambda a: (capi.c_int_p * nt)(*[a[i].ctypes.data_as(capi.c_int_p) for i in range(nt)])
    lib.get_local_trees_ptrees(trees.handle, rows(pt), rows(ag), rows(sp),
                               bl.ctypes.data_as(capi.c_int_p))
    mp = np.zeros((nt, nn), dtype=np.int32)
    lib.awg_local_trees_mapping(trees.handle, mp.ctypes.data_as(capi.c_int_p))
    return pt, ag, sp, bl, mp


def _read_structure(trees: "LocalTrees"):
    """Each tree's root child[0] and the leaves' sequence ids of a handle."""
    lib = capi.load()
    nt = lib.get_local_trees_ntrees(trees.handle)
    nn = lib.get_local_trees_nnodes(trees.handle)
    c0, c1 = (np.zeros((nt, nn), dtype=np.int32) for _ in range(2))
    if lib.awg_local_trees_children(trees.handle, c0.ctypes.data_as(capi.c_int_p),
                                    c1.ctypes.data_as(capi.c_int_p)) != 0:
        raise RuntimeError(capi.last_error())
    nleaves = lib.awg_local_trees_seqids(trees.handle, None)
    seqids = np.zeros(max(nleaves, 0), dtype=np.int32)
    lib.awg_local_trees_seqids(trees.handle, seqids.ctypes.data_as(capi.c_int_p))
    return c0, c1, seqids


def remove_arg_thread(prob: Problem, seqids):
    """remove_arg_thread (thread.cpp:425-556) of each listed sequence in turn from the
    problem's full ARG, on the host. Returns, after each removal, a dict of the trees
    (ptrees, ages, sprs, blocklens, mapping in the names get_local_trees_ptrees gives,
    root_child0: each root's first child) and the leaves' sequence ids."""
    lib = capi.load()
    p = prob.normalized()
    if p.internal:
        raise ValueError("remove_arg_thread: full ARGs only")
    trees = _trees_handle(p)
    out = []
    try:
        for sid in seqids:
            if lib.awg_remove_arg_thread(trees.handle, int(sid)) != 0:
                raise ValueError(capi.last_error())
            out.append(_tree_dict(trees))
    finally:
        trees.close()
    return out


def _tree_dict(trees: "LocalTrees") -> dict:
    pt, ag, sp, bl, mp = _read_trees(trees)
    c0, _c1, ids = _read_structure(trees)
    roots = np.argmax(pt == -1, axis=1)
    return dict(ptrees=pt, ages=ag, sprs=sp, blocklens=bl, mapping=mp,
                root_child0=c0[np.arange(len(roots)), roots], seqids=ids)


def _with_trees(prob: Problem, fn):
    p = prob.normalized()
    trees = _trees_handle(p)
    try:
        return fn(capi.load(), trees, p)
    finally:
        trees.close()


def as_problem(prob: Problem, trees: dict, internal: bool = False) -> Problem:
    """A Problem over the trees a surgery call returned (its dict) with prob's model and
    sequences: sequence rows follow the leaves' sequence ids, so leaf i reads row i, and an
    internal problem (a cut ARG) carries each root's first child."""
    ids = np.asarray(trees["seqids"], dtype=np.int64)
    nleaves = (trees["ptrees"].shape[1] + 1) // 2
    rows = list(ids[:nleaves]) + [i for i in range(prob.nseqs) if i not in set(ids[:nleaves].tolist())]
    return Problem(times=prob.times, popsizes=prob.popsizes, rho=prob.rho, mu=prob.mu,
                   ptrees=trees["ptrees"], ages=trees["ages"], sprs=trees["sprs"],
                   blocklens=trees["blocklens"], seqs=np.ascontiguousarray(prob.seqs[rows]),
                   internal=internal, start_coord=prob.start_coord, mapping=trees["mapping"],
                   root_child0=trees["root_child0"])


def get_state_spaces(prob: Problem) -> list:
    """Each tree's external states as an (S, 2) array of (node, time) (get_state_spaces,
    states.cpp:228-251)."""
    def run(lib, trees, p):
        ptr = lib.get_state_spaces(trees.handle, p.ntimes, False)
        if not ptr:
            raise ValueError(capi.last_error())
        try:
            rows = C.cast(ptr, C.POINTER(C.POINTER(C.c_int)))
            ns = np.zeros(p.seqlen, dtype=np.int32)
            lib.arghmm_get_nstates(trees.handle, p.ntimes, False, ns.ctypes.data_as(capi.c_int_p))
            starts = np.concatenate([[0], np.cumsum(p.blocklens)[:-1]])
            return [np.ctypeslib.as_array(rows[b], shape=(int(ns[starts[b]]) * 2,)).reshape(-1, 2).copy()
                    if ns[starts[b]] > 0 else np.zeros((0, 2), np.int32) for b in range(p.ntrees)]
        finally:
            lib.delete_state_spaces(ptr, p.ntrees)
    return _with_trees(prob, run)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64c(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _take_matrix(lib, mat, nrows: int, ncols: int, free: str) -> np.ndarray:
    if not mat:
        raise ValueError(capi.last_error())
    try:
        if nrows == 0 or ncols == 0:
            return np.zeros((nrows, ncols))
        return np.ctypeslib.as_array(mat[0], shape=(nrows * ncols,)).reshape(nrows, ncols).copy()
    finally:
        getattr(lib, free)(mat, nrows)


def new_transition_probs(ptree, ages, states, times, popsizes, rho: float) -> np.ndarray:
    """The log transition matrix within one tree over `states` ((node, time) rows, any
    order), as the reference's new_transition_probs (trans.cpp:1190-1208)."""
    lib = capi.load()
    pt, ag, st = _i32(ptree), _i32(ages), _i32(states).reshape(-1, 2)
    tm, pops = _f64c(times), _f64c(popsizes)
    S = st.shape[0]
    mat = lib.new_transition_probs(len(pt), pt.ctypes.data_as(capi.c_int_p),
                                   ag.ctypes.data_as(capi.c_int_p), 0.0,
                                   st.ctypes.data_as(capi.c_int_p), S, len(tm),
                                   tm.ctypes.data_as(capi.c_double_p), None, None, None, None,
                                   pops.ctypes.data_as(capi.c_double_p), float(rho))
    return _take_matrix(lib, mat, S, S, "delete_transition_probs")


def new_transition_probs_switch(ptree, last_ptree, spr, ages, last_ages, states1, states2,
                                times, popsizes, rho: float) -> np.ndarray:
    """The log switch matrix from last_ptree's states1 to ptree's states2 across `spr`
    (recomb_node, recomb_time, coal_node, coal_time), as the reference's
    new_transition_probs_switch (trans.cpp:1212-1245)."""
    lib = capi.load()
    pt, lpt, ag, lag = _i32(ptree), _i32(last_ptree), _i32(ages), _i32(last_ages)
    s1, s2 = _i32(states1).reshape(-1, 2), _i32(states2).reshape(-1, 2)
    tm, pops = _f64c(times), _f64c(popsizes)
    r = [int(x) for x in spr]
    mat = lib.new_transition_probs_switch(
        pt.ctypes.data_as(capi.c_int_p), lpt.ctypes.data_as(capi.c_int_p), len(pt), r[0], r[1],
        r[2], r[3], ag.ctypes.data_as(capi.c_int_p), lag.ctypes.data_as(capi.c_int_p), 0.0, 0.0,
        s1.ctypes.data_as(capi.c_int_p), s1.shape[0], s2.ctypes.data_as(capi.c_int_p),
        s2.shape[0], len(tm), tm.ctypes.data_as(capi.c_double_p), None, None, None, None,
        pops.ctypes.data_as(capi.c_double_p), float(rho))
    return _take_matrix(lib, mat, s1.shape[0], s2.shape[0], "delete_transition_probs")


def new_emissions(states, ptree, ages, seqs: np.ndarray, times, mu: float) -> np.ndarray:
    """Emissions P(column | state) of the threaded sequence (the last row of seqs) on one
    tree, [columns][states], as the reference's new_emissions (emit.cpp:1288-1301)."""
    lib = capi.load()
    pt, ag, st = _i32(ptree), _i32(ages), _i32(states).reshape(-1, 2)
    tm = _f64c(times)
    sq, _keep = _char_pp(seqs)
    nseqs, seqlen = np.asarray(seqs).shape
    mat = lib.new_emissions(st.ctypes.data_as(capi.c_int_p), st.shape[0],
                            pt.ctypes.data_as(capi.c_int_p), len(pt),
                            ag.ctypes.data_as(capi.c_int_p), sq, nseqs, seqlen,
                            tm.ctypes.data_as(capi.c_double_p), len(tm), float(mu))
    return _take_matrix(lib, mat, seqlen, st.shape[0], "delete_emissions")


def sample_arg_removal_path(prob: Problem, node: int, pos: int | None = None,
                            leaf: bool = False) -> np.ndarray:
    """A removal path (one node per tree) from `node` of the first tree forward
    (sample_arg_removal_path, thread.cpp:793-799), through `node` at coordinate `pos`
    (thread.cpp:772-790), or the leaf path (leaf=True, thread.cpp:672-700); draws from libc
    rand() (seed it with srand)."""
    def run(lib, trees, p):
        path = np.zeros(p.ntrees, dtype=np.int32)
        ptr = path.ctypes.data_as(capi.c_int_p)
        if leaf:
            lib.arghmm_sample_arg_removal_leaf_path(trees.handle, int(node), ptr)
        elif pos is None:
            lib.arghmm_sample_arg_removal_path(trees.handle, int(node), ptr)
        else:
            lib.arghmm_sample_arg_removal_path2(trees.handle, int(node), int(pos), ptr)
        err = capi.last_error()
        if err:
            raise ValueError(err)
        return path
    return _with_trees(prob, run)


def sample_arg_removal_path_recomb(prob: Problem, recomb_preference: float) -> np.ndarray:
    """A removal path preferring recombination-bearing branches
    (sample_arg_removal_path_recomb, thread.cpp:800-912); draws from libc rand()."""
    def run(lib, trees, p):
        path = np.zeros(p.ntrees, dtype=np.int32)
        lib.arghmm_sample_arg_removal_path_recomb(trees.handle, float(recomb_preference),
                                                  path.ctypes.data_as(capi.c_int_p))
        err = capi.last_error()
        if err:
            raise ValueError(err)
        return path
    return _with_trees(prob, run)


def sample_arg_removal_path_uniform(prob: Problem):
    """(path, log number of paths): a removal path drawn uniformly over all of them
    (sample_arg_removal_path_uniform, thread.cpp:963-1002); draws from libc rand()."""
    def run(lib, trees, p):
        path = np.zeros(p.ntrees, dtype=np.int32)
        lnt = lib.awg_sample_arg_removal_path_uniform(trees.handle, path.ctypes.data_as(capi.c_int_p))
        err = capi.last_error()
        if err:
            raise ValueError(err)
        return path, lnt
    return _with_trees(prob, run)


def remove_arg_thread_path(prob: Problem, path, maxtime: int | None = None,
                           original_thread: bool = False) -> dict:
    """The problem's ARG cut along a removal path (remove_arg_thread_path, thread.cpp:1481-1668;
    maxtime defaults to ntimes + 1 as arg-sample passes): the trees in subtree/main-tree form
    as a dict (ptrees, ages, sprs, blocklens, mapping, root_child0, seqids), with
    original_thread=True also the removed thread as state indices of the cut trees
    (arghmm_remove_arg_thread_path2)."""
    def run(lib, trees, p):
        rp = np.ascontiguousarray(path, dtype=np.int32)
        if rp.shape != (p.ntrees,):
            raise ValueError("remove_arg_thread_path: the path needs one node per tree")
        mt = p.ntimes + 1 if maxtime is None else int(maxtime)
        orig = np.zeros(p.seqlen, dtype=np.int32)
        if original_thread:
            lib.arghmm_remove_arg_thread_path2(trees.handle, rp.ctypes.data_as(capi.c_int_p),
                                               mt, orig.ctypes.data_as(capi.c_int_p))
        else:
            lib.arghmm_remove_arg_thread_path(trees.handle, rp.ctypes.data_as(capi.c_int_p), mt)
        err = capi.last_error()
        if err:
            raise ValueError(err)
        out = _tree_dict(trees)
        if original_thread:
            out["original_thread"] = orig
        return out
    return _with_trees(prob, run)


def get_thread_times(prob: Problem, path) -> np.ndarray:
    """The time of each column's internal state along the thread path (arghmm_get_thread_times,
    thread.cpp:1718-1733), indexed by column."""
    def run(lib, trees, p):
        off = p.start_coord  # the reference indexes both arrays by coordinate
        pa = np.zeros(off + p.seqlen, dtype=np.int32)
        pa[off:] = np.asarray(path, dtype=np.int32)
        times = np.zeros(off + p.seqlen, dtype=np.int32)
        lib.arghmm_get_thread_times(trees.handle, p.ntimes, pa.ctypes.data_as(capi.c_int_p),
                                    times.ctypes.data_as(capi.c_int_p))
        err = capi.last_error()
        if err:
            raise ValueError(err)
        return times[off:].copy()
    return _with_trees(prob, run)


def add_arg_thread_path(prob: Problem, path, rec_pos, rec_node, rec_time,
                        minage: int | None = None) -> dict:  # ArgModel minage, 0 by default
    """The internal problem's cut subtree regrafted along its thread path with the path's
    recombinations (add_arg_thread_path, thread.cpp:1314-1449), on the host: the whole ARG
    as a dict (ptrees, ages, sprs, blocklens, mapping, root_child0, seqids)."""
    def run(lib, trees, p):
        if not p.internal:
            raise ValueError("add_arg_thread_path: internal problems only")
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        pa, rp, rn, rt = i32(path), i32(rec_pos), i32(rec_node), i32(rec_time)
        ptr = lambda a: a.ctypes.data_as(capi.c_int_p)
        rc = lib.awg_add_arg_thread_path(trees.handle, p.ntimes,
                                         0 if minage is None else int(minage), ptr(pa),
                                         len(pa), ptr(rp), ptr(rn), ptr(rt), len(rp))
        if rc != 0:
            raise ValueError(capi.last_error())
        return _tree_dict(trees)
    return _with_trees(prob, run)


def resample_arg_leaf(prob: Problem, seqid: int) -> dict:
    """resample_arg_leaf's move (sample_arg.cpp:66-86) on a full ARG: sequence `seqid`
    removed (host) and threaded back in (awg_sample_arg_thread: forward, traceback and
    recombinations on the device with draws from libc rand(), the thread added on the host).
    Returns the ARG as a dict, leaves named by sequence."""
    def run(lib, trees, p):
        if p.internal:
            raise ValueError("resample_arg_leaf: full ARGs only")
        if lib.awg_remove_arg_thread(trees.handle, int(seqid)) != 0:
            raise ValueError(capi.last_error())
        seqs, _keep = _char_pp(p.seqs)
        rc = lib.awg_sample_arg_thread(trees.handle, p.times.ctypes.data_as(capi.c_double_p),
                                       p.ntimes, p.popsizes.ctypes.data_as(capi.c_double_p),
                                       p.rho, p.mu, seqs, p.nseqs, p.seqlen, int(seqid))
        if rc != 0:
            raise RuntimeError(capi.last_error())
        return _tree_dict(trees)
    return _with_trees(prob, run)


def sample_arg_thread_internal(prob: Problem, minage: int = 0):
    """The internal problem's cut subtree re-threaded (sample_arg_thread_internal,
    sample_thread.cpp:635-692): forward, traceback and recombinations on the device with draws
    from libc rand() (seed it with srand), the regraft on the host. Returns (the whole ARG as
    a dict, the thread path)."""
    def run(lib, trees, p):
        if not p.internal:
            raise ValueError("sample_arg_thread_internal: internal problems only")
        seqs, _keep = _char_pp(p.seqs)
        path = np.zeros(p.seqlen, dtype=np.int32)
        rc = lib.awg_sample_arg_thread_internal(
            trees.handle, p.times.ctypes.data_as(capi.c_double_p), p.ntimes,
            p.popsizes.ctypes.data_as(capi.c_double_p), p.rho, p.mu, seqs, p.nseqs, p.seqlen,
            int(minage), path.ctypes.data_as(capi.c_int_p))
        if rc != 0:
            raise RuntimeError(capi.last_error())
        return _tree_dict(trees), path
    return _with_trees(prob, run)


def arghmm_sample_thread(prob: Problem) -> Problem:
    """The problem's ARG with its last sequence threaded in (draws from libc rand(): seed it
    with srand). The result is a full ARG over all the problem's sequences."""
    lib = capi.load()
    p = prob.normalized()
    if p.internal:
        raise ValueError("arghmm_sample_thread: external (threading) problems only")
    trees = _trees_handle(p)
    try:
        seqs, _keep = _char_pp(p.seqs)
        lib.arghmm_sample_thread(trees.handle, p.times.ctypes.data_as(capi.c_double_p),
                                 p.ntimes, p.popsizes.ctypes.data_as(capi.c_double_p), p.rho,
                                 p.mu, seqs, p.nseqs, p.seqlen)
        err = capi.last_error()
        if err:
            raise RuntimeError(err)
        pt, ag, sp, bl, mp = _read_trees(trees)
    finally:
        trees.close()
    return Problem(times=p.times, popsizes=p.popsizes, rho=p.rho, mu=p.mu, ptrees=pt, ages=ag,
                   sprs=sp, blocklens=bl, seqs=p.seqs, start_coord=p.start_coord, mapping=mp)
