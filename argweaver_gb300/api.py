"""NumPy-level host API of the GPU threading HMM.

  forward(problem)                -> packed forward table (FP64) and log-likelihood
  sample_path(problem, uniforms)  -> sampled state index per column
  posterior(problem)              -> posterior marginals (forward-backward)
  run_batch(problems, ...)        -> many problems in one launch sequence

The reference-compatible calls (arghmm_forward_alg and friends) live in
:mod:`argweaver_gb300.refapi`. Tables are packed column after column with max(nstates,1)
entries per column, the rows of the reference's forward table laid end to end.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional, Sequence

import numpy as np

from . import capi
from .problem import Problem


class GpuError(RuntimeError):
    pass


class _Bound:
    """Problem arrays pinned for the duration of a call, with their C view."""

    def __init__(self, prob: Problem):
        self.p = prob.normalized()
        p = self.p
        ptr = lambda a: None if a is None else a.ctypes.data
        self.c = capi.AwgProblem(p.ntrees, p.nnodes, p.ntimes, p.nseqs, p.seqlen,
                                 int(p.internal), p.start_coord, 0, ptr(p.ptrees),
                                 ptr(p.ages), ptr(p.sprs), ptr(p.blocklens), ptr(p.mapping),
                                 ptr(p.root_child0), ptr(p.times), ptr(p.popsizes), p.rho,
                                 p.mu, ptr(p.seqs), float(p.infsites_penalty))


def cells(prob: Problem) -> int:
    lib = capi.load()
    b = _Bound(prob)
    n = lib.awg_problem_cells(C.byref(b.c))
    if n < 0:
        raise ValueError(capi.last_error())
    return int(n)


def offsets(nstates: np.ndarray) -> np.ndarray:
    off = np.zeros(nstates.shape[0] + 1, dtype=np.int64)
    np.cumsum(np.maximum(nstates, 1), out=off[1:])
    return off


@dataclass
class Result:
    forward: Optional[np.ndarray] = None
    posterior: Optional[np.ndarray] = None
    path: Optional[np.ndarray] = None
    loglik: float = float("nan")


def run_batch(problems: Sequence[Problem], *, precision: str = "fp64",
              want_forward: bool = True, want_path: bool = False,
              want_posterior: bool = False,
              uniforms: Optional[Sequence[Optional[np.ndarray]]] = None) -> List[Result]:
    """Run forward (+ traceback, + backward/posterior) for a batch of problems."""
    lib = capi.load()
    fp32 = precision == "fp32"
    if precision not in ("fp32", "fp64"):
        raise ValueError("precision must be 'fp64' or 'fp32'")
    n = len(problems)
    bound = [_Bound(p) for p in problems]
    probs = (capi.AwgProblem * n)(*[b.c for b in bound])
    outs = (capi.AwgOutputs * n)()
    results, keep = [], []
    ncells = np.zeros(n, dtype=np.int64)
    if lib.awg_problems_cells(probs, n, ncells.ctypes.data) != 0:
        raise ValueError(capi.last_error())
    for q, b in enumerate(bound):
        r = Result()
        ncell = int(ncells[q])
        o = outs[q]
        if want_forward:
            r.forward = np.empty(ncell, dtype=np.float32 if fp32 else np.float64)
            if fp32:
                o.forward32 = r.forward.ctypes.data
            else:
                o.forward = r.forward.ctypes.data
        if want_posterior:
            r.posterior = np.empty(ncell, dtype=np.float64)
            o.posterior = r.posterior.ctypes.data
        if want_path:
            r.path = np.empty(b.p.seqlen, dtype=np.int32)
            o.path = r.path.ctypes.data
            if uniforms is not None and uniforms[q] is not None:
                u = np.ascontiguousarray(uniforms[q], dtype=np.float64)
                if u.shape[0] != b.p.seqlen:
                    raise ValueError("uniforms must have one entry per column")
                keep.append(u)
                o.uniforms = u.ctypes.data
        ll = np.zeros(1, dtype=np.float64)
        keep.append(ll)
        o.loglik = ll.ctypes.data
        results.append((r, ll))
    rc = lib.awg_run_batch(probs, outs, n, capi.AWG_FP32 if fp32 else capi.AWG_FP64)
    if rc != 0:
        raise GpuError(f"awg_run_batch failed ({rc}): {capi.last_error()}")
    out = []
    for r, ll in results:
        r.loglik = float(ll[0])
        out.append(r)
    return out


def _bind_batch(problems, precision, want_forward, want_path, want_posterior, uniforms):
    """ctypes views of a batch and its output arrays (kept alive by the returned lists)."""
    fp32 = precision == "fp32"
    if precision not in ("fp32", "fp64"):
        raise ValueError("precision must be 'fp64' or 'fp32'")
    lib = capi.load()
    n = len(problems)
    bound = [_Bound(p) for p in problems]
    probs = (capi.AwgProblem * n)(*[b.c for b in bound])
    outs = (capi.AwgOutputs * n)()
    ncells = np.zeros(n, dtype=np.int64)
    if lib.awg_problems_cells(probs, n, ncells.ctypes.data) != 0:
        raise ValueError(capi.last_error())
    results, keep = [], [bound]
    for q, b in enumerate(bound):
        r = Result()
        o = outs[q]
        if want_forward:
            r.forward = np.empty(int(ncells[q]), dtype=np.float32 if fp32 else np.float64)
            if fp32:
                o.forward32 = r.forward.ctypes.data
            else:
                o.forward = r.forward.ctypes.data
        if want_posterior:
            r.posterior = np.empty(int(ncells[q]), dtype=np.float64)
            o.posterior = r.posterior.ctypes.data
        if want_path:
            r.path = np.empty(b.p.seqlen, dtype=np.int32)
            o.path = r.path.ctypes.data
            if uniforms is not None and uniforms[q] is not None:
                u = np.ascontiguousarray(uniforms[q], dtype=np.float64)
                keep.append(u)
                o.uniforms = u.ctypes.data
        ll = np.zeros(1, dtype=np.float64)
        keep.append(ll)
        o.loglik = ll.ctypes.data
        results.append((r, ll))
    return probs, outs, results, keep


class BatchContext:
    """Batches in flight from one thread (awg_batch_ctx): launch() plans, uploads and queues
    a batch and returns; finish() waits for it and returns its results. Two contexts used in
    turn overlap one batch's host work (binding, planning, upload) with the other's kernels;
    a context holds one batch at a time."""

    def __init__(self):
        self._lib = capi.load()
        self._h = self._lib.awg_batch_ctx_create()
        if not self._h:
            raise GpuError(capi.last_error())
        self._pending = None

    def launch(self, problems: Sequence[Problem], *, precision: str = "fp32",
               want_forward: bool = False, want_path: bool = True, want_posterior: bool = False,
               uniforms: Optional[Sequence[Optional[np.ndarray]]] = None) -> None:
        if self._pending is not None:
            raise RuntimeError("finish() the context's last batch before launching another")
        probs, outs, results, keep = _bind_batch(problems, precision, want_forward, want_path,
                                                 want_posterior, uniforms)
        prec = capi.AWG_FP32 if precision == "fp32" else capi.AWG_FP64
        rc = self._lib.awg_batch_launch(self._h, probs, outs, len(problems), prec)
        if rc != 0:
            raise GpuError(f"awg_batch_launch failed ({rc}): {capi.last_error()}")
        self._pending = (probs, outs, results, keep)

    def finish(self) -> List[Result]:
        if self._pending is None:
            raise RuntimeError("no batch in flight")
        _, _, results, _ = self._pending
        self._pending = None
        rc = self._lib.awg_batch_finish(self._h)
        if rc != 0:
            raise GpuError(f"awg_batch_finish failed ({rc}): {capi.last_error()}")
        out = []
        for r, ll in results:
            r.loglik = float(ll[0])
            out.append(r)
        return out

    def close(self) -> None:
        if self._h:
            self._lib.awg_batch_ctx_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(problems: Sequence[Problem], *, precision: str = "fp32", want_path: bool = True,
             trials: int = 2) -> dict:
    """Time the candidate schedules on this batch and keep the fastest for its shape class
    (awg_autotune); returns the chosen knobs and the best compute time (ms)."""
    lib = capi.load()
    probs, outs, _, keep = _bind_batch(problems, precision, False, want_path, False, None)
    buf = C.create_string_buffer(256)
    rc = lib.awg_autotune(probs, outs, len(problems),
                          capi.AWG_FP32 if precision == "fp32" else capi.AWG_FP64, trials, buf, 256)
    del keep
    if rc != 0:
        raise GpuError(f"awg_autotune failed ({rc}): {capi.last_error()}")
    out = {}
    for kv in buf.value.decode().split():
        k, v = kv.split("=")
        out[k] = float(v) if k == "ms" else int(v)
    return out


def release_memory() -> None:
    """Free the engine's device arena and staging (awg_release_memory)."""
    capi.load().awg_release_memory()


def set_graphs(on: bool) -> None:
    capi.load().awg_set_graphs(int(bool(on)))


def set_schedule(kpt: int = 0, group_div: int = 8, chunk: int = 1, persistent: bool = True) -> None:
    """Default schedule knobs (awg_set_schedule); forgets the autotuner's choices."""
    capi.load().awg_set_schedule(int(kpt), int(group_div), int(chunk), int(bool(persistent)))


def graph_counts() -> dict:
    lib = capi.load()
    return {"replays": int(lib.awg_graph_replays()), "captures": int(lib.awg_graph_captures())}


def forward(prob: Problem, precision: str = "fp64"):
    r = run_batch([prob], precision=precision)[0]
    return r.forward, r.loglik


def sample_path(prob: Problem, uniforms: Optional[np.ndarray] = None,
                precision: str = "fp64") -> np.ndarray:
    r = run_batch([prob], precision=precision, want_forward=False, want_path=True,
                  uniforms=[uniforms])[0]
    return r.path


def sample_path_conditioned(prob: Problem, prior: Optional[np.ndarray] = None,
                            last_state: int = -1,
                            uniforms: Optional[np.ndarray] = None) -> np.ndarray:
    """FP64 forward + traceback with a given first column (``prior``) and/or a given last
    state (awg_sample_path_conditioned); uniforms as for sample_path (u[L-1] unused when the
    last state is given; None draws libc rand() as the reference does)."""
    lib = capi.load()
    b = _Bound(prob)
    path = np.empty(b.p.seqlen, dtype=np.int32)
    pr = None if prior is None else np.ascontiguousarray(prior, dtype=np.float64)
    u = None if uniforms is None else np.ascontiguousarray(uniforms, dtype=np.float64)
    rc = lib.awg_sample_path_conditioned(
        C.byref(b.c), None if pr is None else pr.ctypes.data_as(capi.c_double_p),
        int(last_state), None if u is None else u.ctypes.data_as(capi.c_double_p),
        path.ctypes.data_as(capi.c_int_p), None)
    if rc != 0:
        raise GpuError(f"awg_sample_path_conditioned failed ({rc}): {capi.last_error()}")
    return path


def posterior(prob: Problem, precision: str = "fp64") -> np.ndarray:
    return run_batch([prob], precision=precision, want_forward=False,
                     want_posterior=True)[0].posterior


def sample_recombinations(prob: Problem, path: np.ndarray, uniforms: np.ndarray,
                          cap: Optional[int] = None):
    """Recombinations along a sampled thread path (sample_recombinations,
    recomb.cpp:151-235), on the GPU: (columns, nodes (-1: the thread's branch of an external
    problem), times, uniforms used). The uniforms are consumed in order, one per draw
    (at most 2 per column)."""
    lib = capi.load()
    b = _Bound(prob)
    path = np.ascontiguousarray(path, dtype=np.int32)
    u = np.ascontiguousarray(uniforms, dtype=np.float64)
    if path.shape != (b.p.seqlen,):
        raise ValueError("path must hold one state per column")
    cap = b.p.seqlen if cap is None else int(cap)
    pos, node, time = (np.zeros(max(cap, 1), dtype=np.int32) for _ in range(3))
    used = C.c_int(0)
    n = lib.awg_sample_recombinations(C.byref(b.c), path.ctypes.data_as(capi.c_int_p),
                                      u.ctypes.data_as(capi.c_double_p), len(u),
                                      pos.ctypes.data_as(capi.c_int_p),
                                      node.ctypes.data_as(capi.c_int_p),
                                      time.ctypes.data_as(capi.c_int_p), cap, C.byref(used))
    if n < 0:
        raise GpuError(capi.last_error())
    return pos[:n].copy(), node[:n].copy(), time[:n].copy(), used.value


def kernel_launches() -> int:
    return int(capi.load().awg_kernel_launches())


def set_timing(mode) -> None:
    """0/False: off; 1/True: device times of the overlapped schedule (compute total);
    2: kernels one phase after another, each phase timed."""
    capi.load().awg_set_timing(int(mode))


def last_timings() -> dict:
    out = np.zeros(8, dtype=np.float64)
    capi.load().awg_last_timings(out.ctypes.data_as(capi.c_double_p))
    keys = ["h2d", "tables", "emit", "forward", "traceback", "backward", "d2h", "compute"]
    return {k: float(v) for k, v in zip(keys, out)}
