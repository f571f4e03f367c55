"""One threading problem: an ARG (local trees + SPRs), its sequences and the model.

The arrays are exactly what the reference's C API takes to build a ``LocalTrees``
(``arghmm_new_trees``, src/argweaver/local_tree.cpp:1817, and the constructor at
local_tree.cpp:321): per tree a parent array and age indices (leaves first), the SPR to
the left of each tree ``(recomb_node, recomb_time, coal_node, coal_time)`` and the block
lengths. ``mapping`` optionally carries ``LocalTreeSpr::mapping`` (local_tree.h:493);
when absent it is the reference's ``make_node_mapping`` (local_tree.h:767).
``root_child0`` optionally names ``child[0]`` of each tree's root: for internal-branch
trees that is the cut subtree (states.cpp:121), which parent arrays alone (children in
index order, local_tree.h:216-229) cannot always express.

Sequences are rows of bytes: the tree's leaves in leaf order, followed (external
threading) by the sequence being threaded, as ``ArgHmmMatrixIter`` expects with
``new_chrom = nleaves`` (matrices.h:225-227).

File format "AWGPROB1" (little endian) is shared with the fixture harness under oracle/.
"""

from __future__ import annotations

import dataclasses
import struct
from typing import Optional

import numpy as np

MAGIC = b"AWGPROB1"


@dataclasses.dataclass
class Problem:
    times: np.ndarray          # f64 [ntimes]
    popsizes: np.ndarray       # f64 [ntimes]
    rho: float                 # per column
    mu: float                  # per column
    ptrees: np.ndarray         # i32 [ntrees, nnodes]
    ages: np.ndarray           # i32 [ntrees, nnodes]
    sprs: np.ndarray           # i32 [ntrees, 4]
    blocklens: np.ndarray      # i32 [ntrees]
    seqs: np.ndarray           # u8  [nseqs, seqlen]
    internal: bool = False
    start_coord: int = 0
    mapping: Optional[np.ndarray] = None   # i32 [ntrees, nnodes]
    root_child0: Optional[np.ndarray] = None  # i32 [ntrees]
    path_node: Optional[np.ndarray] = None  # true thread (simulated inputs only)
    path_time: Optional[np.ndarray] = None
    # ArgModel::infsites_penalty (model.h:53): emissions of states that break the
    # infinite-sites model are multiplied by it (emit.cpp:847-862); 1 (or 0): off
    infsites_penalty: float = 1.0

    @property
    def ntimes(self) -> int:
        return int(self.times.shape[0])

    @property
    def ntrees(self) -> int:
        return int(self.ptrees.shape[0])

    @property
    def nnodes(self) -> int:
        return int(self.ptrees.shape[1])

    @property
    def nseqs(self) -> int:
        return int(self.seqs.shape[0])

    @property
    def seqlen(self) -> int:
        return int(self.seqs.shape[1])

    @property
    def nleaves(self) -> int:
        return (self.nnodes + 1) // 2

    def normalized(self) -> "Problem":
        """Contiguous arrays of the dtypes the C ABI takes."""
        f = lambda a, dt: np.ascontiguousarray(a, dtype=dt)
        return dataclasses.replace(
            self,
            times=f(self.times, np.float64), popsizes=f(self.popsizes, np.float64),
            ptrees=f(self.ptrees, np.int32), ages=f(self.ages, np.int32),
            sprs=f(self.sprs, np.int32), blocklens=f(self.blocklens, np.int32),
            seqs=f(self.seqs, np.uint8),
            mapping=None if self.mapping is None else f(self.mapping, np.int32),
            root_child0=None if self.root_child0 is None else f(self.root_child0, np.int32))

    def nstates_per_tree(self) -> np.ndarray:
        """State-space size of each local tree (states.cpp:77-100 and :170-199)."""
        T = self.ntimes
        out = np.zeros(self.ntrees, dtype=np.int64)
        for b in range(self.ntrees):
            par = self.ptrees[b]
            age = self.ages[b]
            if not self.internal:
                root = int(np.nonzero(par == -1)[0][0])
                nonroot = par != -1
                s = int(np.sum(age[par[nonroot]] - age[nonroot] + 1))
                s += max(0, T - 1 - int(age[root]))
            else:
                root = int(np.nonzero(par == -1)[0][0])
                if age[root] < T:
                    out[b] = 0
                    continue
                kids = np.nonzero(par == root)[0]
                sub = (int(self.root_child0[b]) if self.root_child0 is not None
                       else _first_child(par, root))
                minage = int(age[sub])
                ignore = _subtree_mask(par, sub)
                ignore[root] = True
                s = 0
                for i in range(self.nnodes):
                    if ignore[i]:
                        continue
                    t0 = max(int(age[i]), minage)
                    top = T - 2 if par[i] == root else int(age[par[i]])
                    s += max(0, top - t0 + 1)
                del kids
            out[b] = s
        return out

    def nstates_per_column(self) -> np.ndarray:
        return np.repeat(self.nstates_per_tree(), self.blocklens.astype(np.int64))

    def cells(self) -> int:
        """State-cells of this problem: sum over columns of max(nstates, 1)."""
        s = np.maximum(self.nstates_per_tree(), 1)
        return int(np.sum(s * self.blocklens.astype(np.int64)))

    # -- file I/O --------------------------------------------------------------
    def save(self, path: str) -> None:
        p = self.normalized()
        has_map = p.mapping is not None
        has_rc0 = p.root_child0 is not None
        with open(path, "wb") as f:
            f.write(MAGIC)
            f.write(struct.pack("<8i", p.ntrees, p.nnodes, p.ntimes, p.nseqs, p.seqlen,
                                int(p.internal), p.start_coord,
                                (1 if has_map else 0) | (2 if has_rc0 else 0)))
            f.write(struct.pack("<2d", p.rho, p.mu))
            for a in (p.times, p.popsizes, p.ptrees, p.ages, p.sprs, p.blocklens, p.seqs):
                f.write(a.tobytes())
            if has_map:
                f.write(p.mapping.tobytes())
            if has_rc0:
                f.write(p.root_child0.tobytes())

    @staticmethod
    def load(path: str) -> "Problem":
        with open(path, "rb") as f:
            data = f.read()
        if data[:8] != MAGIC:
            raise ValueError(f"{path}: not an AWGPROB1 file")
        ntrees, nnodes, ntimes, nseqs, seqlen, internal, start, flags = \
            struct.unpack_from("<8i", data, 8)
        rho, mu = struct.unpack_from("<2d", data, 40)
        off = 56

        def take(dt, count, shape):
            nonlocal off
            a = np.frombuffer(data, dtype=dt, count=count, offset=off).reshape(shape)
            off += a.nbytes
            return a.copy()

        times = take(np.float64, ntimes, (ntimes,))
        popsizes = take(np.float64, ntimes, (ntimes,))
        ptrees = take(np.int32, ntrees * nnodes, (ntrees, nnodes))
        ages = take(np.int32, ntrees * nnodes, (ntrees, nnodes))
        sprs = take(np.int32, ntrees * 4, (ntrees, 4))
        blocklens = take(np.int32, ntrees, (ntrees,))
        seqs = take(np.uint8, nseqs * seqlen, (nseqs, seqlen))
        mapping = take(np.int32, ntrees * nnodes, (ntrees, nnodes)) if flags & 1 else None
        rc0 = take(np.int32, ntrees, (ntrees,)) if flags & 2 else None
        return Problem(times=times, popsizes=popsizes, rho=rho, mu=mu, ptrees=ptrees,
                       ages=ages, sprs=sprs, blocklens=blocklens, seqs=seqs,
                       internal=bool(internal), start_coord=start, mapping=mapping,
                       root_child0=rc0)


def _first_child(par: np.ndarray, node: int) -> int:
    """child[0] as the reference's set_ptree assigns it: the lowest-index child."""
    kids = np.nonzero(par == node)[0]
    return int(kids[0])


def _subtree_mask(par: np.ndarray, top: int) -> np.ndarray:
    n = par.shape[0]
    mask = np.zeros(n, dtype=bool)
    for v in range(n):
        u = v
        while u != -1:
            if u == top:
                mask[v] = True
                break
            u = int(par[u])
    return mask


def time_points(ntimes: int, maxtime: float, delta: float = 0.01) -> np.ndarray:
    """Log-spaced time points (get_time_points, src/argweaver/model.h:21-32)."""
    i = np.arange(ntimes, dtype=np.float64)
    return (np.exp(i / (ntimes - 1) * np.log(1.0 + delta * maxtime)) - 1.0) / delta
