"""arg-sample's input formats through the library's host code (formats.cpp): sites files
and SMC local trees, read and compressed as arg-sample reads them (arg-sample.cpp:996-1155),
and written in the reference's layouts.

    names, seqs = read_sites("data.sites.gz", compress=10)
    prob, names = read_arg("data.sites.gz", "out.100.smc.gz", compress=10)
    refapi.arghmm_likelihood(prob)
"""

from __future__ import annotations

import ctypes as C
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import capi
from .problem import Problem, time_points


def _err() -> str:
    msg = capi.load().awg_formats_last_error()
    return msg.decode() if msg else ""


def _load(sites_path: str, smc_path: Optional[str], compress: int, times: np.ndarray):
    lib = capi.load()
    t = np.ascontiguousarray(times, dtype=np.float64)
    h = lib.awg_read_arg_input(sites_path.encode(), smc_path.encode() if smc_path else None,
                               int(compress), t.ctypes.data_as(capi.c_double_p), len(t))
    if not h:
        raise ValueError(_err())
    try:
        dims = [C.c_int() for _ in range(5)]
        lib.awg_arg_input_dims(h, *[C.byref(d) for d in dims])
        nseqs, seqlen, ntrees, nnodes, start = (d.value for d in dims)
        names = [lib.awg_arg_input_name(h, i).decode() for i in range(nseqs)]
        seqs = np.zeros((nseqs, seqlen), dtype=np.uint8)
        ptrees = np.zeros((ntrees, nnodes), dtype=np.int32)
        ages = np.zeros((ntrees, nnodes), dtype=np.int32)
        sprs = np.zeros((ntrees, 4), dtype=np.int32)
        blocklens = np.zeros(ntrees, dtype=np.int32)
        lib.awg_arg_input_copy(h, seqs.ctypes.data, ptrees.ctypes.data, ages.ctypes.data,
                               sprs.ctypes.data, blocklens.ctypes.data)
    finally:
        lib.awg_free_arg_input(h)
    return names, seqs, start, ptrees, ages, sprs, blocklens


def read_sites(path: str, compress: int = 1) -> Tuple[List[str], np.ndarray]:
    """Sequence names and the compressed alignment (uint8 [nseqs, columns]; non-variant
    columns 'A', as make_sequences_from_sites fills them)."""
    names, seqs, *_ = _load(path, None, compress, np.zeros(2))
    return names, seqs


def read_arg(sites_path: str, smc_path: str, compress: int = 1, *,
             times: Optional[np.ndarray] = None, ntimes: int = 20, maxtime: float = 200e3,
             popsize: float = 1e4, rho: float = 1.5e-8, mu: float = 2.5e-8
             ) -> Tuple[Problem, List[str]]:
    """The ARG of an SMC file over the sites file's compressed alignment, as a Problem (rho
    and mu per base scaled by `compress`, as arg-sample does, arg-sample.cpp:428-436), and
    the sequence names. Sequences beyond the SMC's leaves stay in the problem: with one
    more sequence than leaves it is the threading problem of the last one."""
    if times is None:
        times = time_points(ntimes, maxtime)
    times = np.ascontiguousarray(times, dtype=np.float64)
    names, seqs, start, ptrees, ages, sprs, blocklens = _load(sites_path, smc_path, compress,
                                                              times)
    prob = Problem(times=times, popsizes=np.full(len(times), float(popsize)),
                   rho=rho * compress, mu=mu * compress, ptrees=ptrees, ages=ages, sprs=sprs,
                   blocklens=blocklens, seqs=seqs, start_coord=start)
    return prob, names


def _names_pp(names: Sequence[str]):
    arr = (C.c_char_p * len(names))(*[n.encode() for n in names])
    return C.cast(arr, capi.c_char_pp), arr


def write_sites(path: str, names: Sequence[str], seqs: np.ndarray, chrom: str = "chr",
                start_coord: int = 0) -> None:
    """A sites file of the columns whose bases differ (write_sites, sequences.cpp:133-157);
    ".gz" paths are compressed."""
    seqs = np.ascontiguousarray(seqs, dtype=np.uint8)
    pp, _keep = _names_pp(names)
    if capi.load().awg_write_sites(path.encode(), pp, seqs.shape[0], chrom.encode(),
                                   int(start_coord), seqs.shape[1], seqs.ctypes.data) != 0:
        raise ValueError(_err())


def write_smc(path: str, prob: Problem, names: Sequence[str], chrom: str = "chr") -> None:
    """The problem's local trees as an SMC file (write_local_trees,
    local_tree.cpp:1286-1362); trees numbered by the default node mapping."""
    p = prob.normalized()
    if p.internal:
        raise ValueError("write_smc: external (full) trees only")
    pp, _keep = _names_pp(names)
    pt = np.ascontiguousarray(p.ptrees, dtype=np.int32)
    ag = np.ascontiguousarray(p.ages, dtype=np.int32)
    sp = np.ascontiguousarray(p.sprs, dtype=np.int32)
    bl = np.ascontiguousarray(p.blocklens, dtype=np.int32)
    t = np.ascontiguousarray(p.times, dtype=np.float64)
    if capi.load().awg_write_smc(path.encode(), pp, chrom.encode(), int(p.start_coord),
                                 pt.ctypes.data, ag.ctypes.data, sp.ctypes.data, bl.ctypes.data,
                                 p.ntrees, p.nnodes, t.ctypes.data_as(capi.c_double_p),
                                 len(t)) != 0:
        raise ValueError(_err())
