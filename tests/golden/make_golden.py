"""Generate the golden fixtures in tests/golden/ from the compiled reference.

Run where the reference checkout exists ($AWG_REFERENCE, default: a sibling of this
repository named "reference"):

    python tests/golden/make_golden.py            # all fixtures
    python tests/golden/make_golden.py infsites   # only the infinite-sites ones
    python tests/golden/make_golden.py dense      # only the dense-HMM ones
    python tests/golden/make_golden.py helpers    # the dense transition / emission helpers
    python tests/golden/make_golden.py argprob    # only the ARG-probability ones
    python tests/golden/make_golden.py formats    # only the sites / SMC ones
    python tests/golden/make_golden.py recomb     # only the recombination-sampling ones
    python tests/golden/make_golden.py addthread  # only the thread-addition ones
    python tests/golden/make_golden.py samplethread  # only the full threading step
    python tests/golden/make_golden.py removethread  # leaf-thread removals
    python tests/golden/make_golden.py removalpaths  # removal paths and the cut
    python tests/golden/make_golden.py addthreadpath  # the internal-branch regraft
    python tests/golden/make_golden.py samplethreadinternal  # the internal re-threading step
    python tests/golden/make_golden.py resampleleaf  # the leaf re-threading move
    python tests/golden/make_golden.py large      # config-scale shapes (k = 48, k = 50 cut)

It builds the reference from its own sources (oracle/Makefile target ``ref``), writes
each problem as an AWGPROB1 file and runs the reference's threading HMM on it through
oracle/ref_harness.cpp. Each ``<name>.npz`` then holds, from the reference:

  nstates      int32 [L]    states per column (arghmm_get_nstates, states.cpp:209)
  colsum       f64   [L]    sum of each forward column
  colwsum      f64   [L]    sum of fw[i][k] * w_k, w_k = 1 + ((k * 2654435761) % 1000) / 1000
  rows         int32 [R]    sampled columns (every 32nd and the last)
  rowvals      f64   [..]   those forward columns, packed
  seed         int          srand seed of the traceback
  uniforms     f64   [L]    rand()/RAND_MAX the traceback drew, indexed by column
  path         int32 [L]    sampled state path (stochastic_traceback, sample_thread.cpp:522)
  infsites_penalty  f64     (infsites_* fixtures) the model's infsites_penalty they ran with
and for single-tree problems the reference's dense log-space backward (hmm.cpp:48) with
the log transition matrix (calc_transition_probs, trans.cpp:136) and log emissions it ran on:
  dense_bw     f64   [L, S]
  dense_trans  f64   [S, S]
  dense_emit   f64   [L, S]
  dense_fw     f64   [L, S]   the reference's dense forward_alg (first column: dense_emit[0])
  dense_path   int32 [L]      a path drawn from it after srand(seed) (sample_hmm_posterior)

``densehmm/s<S>_n<n>.npz`` hold the same dense_* arrays (and seed) for the generic HMM of
hmm.cpp run on random S-state matrices with zero entries (harness command densernd); their
first forward column is dense_emit[0] - log(S), the last backward column zero.

Sources of the problems: examples/sim1 (the reference's bundled data, converted by
the harness the way arg-sample reads it), the seeded DSMC generator of this project
(argweaver_gb300/csrc/sim.cpp), and internal-branch cuts made by the reference's own
removal-path code (remove_arg_thread_path) on simulated full ARGs.
"""

from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from argweaver_gb300.problem import Problem  # noqa: E402
from argweaver_gb300.sim import simulate  # noqa: E402
import pyoracle  # noqa: E402

REF = os.environ.get("AWG_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))
HARNESS = os.path.join(ROOT, "oracle", "_ref", "ref_harness")


def weights(n: int) -> np.ndarray:
    k = np.arange(n, dtype=np.int64)
    return 1.0 + ((k * 2654435761) % 1000) / 1000.0


def read_ref(path: str):
    d = open(path, "rb").read()
    assert d[:8] == b"AWGREF01"
    L = int(np.frombuffer(d, np.int32, 1, 8)[0])
    ncells = int(np.frombuffer(d, np.int64, 1, 16)[0])
    off = 24
    ns = np.frombuffer(d, np.int32, L, off).copy(); off += 4 * L
    fw = np.frombuffer(d, np.float64, ncells, off).copy(); off += 8 * ncells
    path = np.frombuffer(d, np.int32, L, off).copy()
    return ns, fw, path


def read_dense(path: str):
    d = open(path, "rb").read()
    assert d[:8] == b"AWGDNS03"
    L, S = (int(x) for x in np.frombuffer(d, np.int32, 2, 8))
    off = 16
    bw = np.frombuffer(d, np.float64, L * S, off).reshape(L, S).copy(); off += 8 * L * S
    trans = np.frombuffer(d, np.float64, S * S, off).reshape(S, S).copy(); off += 8 * S * S
    emit = np.frombuffer(d, np.float64, L * S, off).reshape(L, S).copy(); off += 8 * L * S
    fw = np.frombuffer(d, np.float64, L * S, off).reshape(L, S).copy(); off += 8 * L * S
    path = np.frombuffer(d, np.int32, L, off).copy()
    return bw, trans, emit, fw, path


def summarize(ns, fw):
    off = pyoracle.offsets(ns)
    L = ns.shape[0]
    colsum = np.zeros(L)
    colwsum = np.zeros(L)
    for i in range(L):
        col = fw[off[i]:off[i + 1]]
        colsum[i] = col.sum()
        colwsum[i] = (col * weights(col.shape[0])).sum()
    rows = np.unique(np.concatenate([np.arange(0, L, 32), [L - 1]])).astype(np.int32)
    rowvals = np.concatenate([fw[off[i]:off[i + 1]] for i in rows])
    return colsum, colwsum, rows, rowvals


def run(*args):
    subprocess.run([HARNESS] + [str(a) for a in args], check=True)


def make(name: str, prob_path: str, seed: int, tmp: str, dense: bool = False,
         penalty: float = 1.0):
    prob = Problem.load(prob_path)
    out = os.path.join(tmp, name + ".ref")
    if penalty < 1.0:
        run("forward", prob_path, out, seed, repr(penalty))
    else:
        run("forward", prob_path, out, seed)
    ns, fw, path = read_ref(out)
    colsum, colwsum, rows, rowvals = summarize(ns, fw)
    extra = {}
    if dense:
        dout = os.path.join(tmp, name + ".dense")
        run("dense", prob_path, dout, seed)
        (extra["dense_bw"], extra["dense_trans"], extra["dense_emit"], extra["dense_fw"],
         extra["dense_path"]) = read_dense(dout)
    if penalty < 1.0:
        extra["infsites_penalty"] = penalty
    u = pyoracle.rand_uniforms(seed, prob.seqlen)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), nstates=ns, colsum=colsum,
                        colwsum=colwsum, rows=rows, rowvals=rowvals, seed=seed,
                        uniforms=u, path=path, **extra)
    dst = os.path.join(HERE, name + ".prob")
    if os.path.abspath(prob_path) != dst:
        prob.save(dst)
    print(f"{name}: L={prob.seqlen} trees={prob.ntrees} cells={fw.size} "
          f"internal={prob.internal}")


def first_tree(prob: Problem) -> Problem:
    """The problem restricted to its first local tree (single-block HMM)."""
    L = int(prob.blocklens[0])
    return Problem(times=prob.times, popsizes=prob.popsizes, rho=prob.rho, mu=prob.mu,
                   ptrees=prob.ptrees[:1].copy(), ages=prob.ages[:1].copy(),
                   sprs=prob.sprs[:1].copy(), blocklens=prob.blocklens[:1].copy(),
                   seqs=prob.seqs[:, :L].copy(), internal=prob.internal)


def dense(tmp):
    """Single-tree problems with the reference's dense HMM (hmm.cpp): backward, forward and
    a sampled path."""
    for seed in (41, 43):
        prob = first_tree(simulate(6, 400, seed))
        p = os.path.join(tmp, "p.prob"); prob.save(p)
        make(f"single_k7_s{seed}", p, seed, tmp, dense=True)


def helpers(tmp):
    """The reference's dense helper exports (new_transition_probs, new_emissions,
    new_transition_probs_switch) on simulated external ARGs with default node mappings:
    tree 0's log transition matrix and emissions, and the log switch matrices into the next
    trees, states in get_coal_states order; and whether the reference's brute-force
    self-checks (arghmm_assert_transmat, _switch, arghmm_assert_emit: trans.cpp:856-1032,
    emit.cpp:1222-1248) pass on the same trees (self_checks, 1 each)."""
    out_dir = os.path.join(HERE, "helpers")
    os.makedirs(out_dir, exist_ok=True)
    cases = [("k8_s11", simulate(7, 1500, 11), 12),
             ("k10_T32", simulate(9, 1500, 31, ntimes=32), 8),
             ("k17_missing", simulate(16, 1000, 21, missing=0.02), 8)]
    for name, prob, maxb in cases:
        pp = os.path.join(tmp, "h.prob")
        prob.save(pp)
        ob = os.path.join(tmp, "h.bin")
        run("helpers", pp, ob, maxb)
        d = open(ob, "rb").read()
        assert d[:8] == b"AWGHLP01"
        S0, L0, nsw = np.frombuffer(d, np.int32, 3, 8)
        o = 20
        trans = np.frombuffer(d, np.float64, S0 * S0, o).reshape(S0, S0); o += 8 * S0 * S0
        emit = np.frombuffer(d, np.float64, L0 * S0, o).reshape(L0, S0); o += 8 * L0 * S0
        sizes, mats = [], []
        for _ in range(nsw):
            S1, S2 = np.frombuffer(d, np.int32, 2, o); o += 8
            mats.append(np.frombuffer(d, np.float64, S1 * S2, o)); o += 8 * S1 * S2
            sizes.append((S1, S2))
        checks = np.frombuffer(d, np.int32, nsw + 2, o); o += 4 * (nsw + 2)
        assert o == len(d)
        prob.save(os.path.join(out_dir, name + ".prob"))
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), trans=trans, emit=emit,
                            switch_sizes=np.array(sizes, np.int32).reshape(-1, 2),
                            switch=np.concatenate(mats) if mats else np.zeros(0),
                            self_checks=checks)
        print(name, S0, L0, sizes, checks)


def densernd(tmp):
    """The dense HMM (hmm.cpp) on random matrices with zero entries: S = 37 (a warp and a
    few states) and S = 5 (fewer states than a warp)."""
    for S, n, seed in ((37, 160, 7), (5, 64, 9)):
        out = os.path.join(tmp, "d.bin")
        run("densernd", S, n, seed, out)
        bw, trans, emit, fw, path = read_dense(out)
        os.makedirs(os.path.join(HERE, "densehmm"), exist_ok=True)
        np.savez_compressed(os.path.join(HERE, "densehmm", f"s{S}_n{n}.npz"), seed=seed,
                            dense_bw=bw, dense_trans=trans, dense_emit=emit, dense_fw=fw,
                            dense_path=path)


def argprob(tmp):
    """The ARG's probabilities (total_prob.cpp) from the reference's C exports, on full ARGs
    (one sequence per leaf), one with missing calls and whole columns masked at tree starts
    (the reference reuses a tree's first invariant site's likelihood for every invariant
    site, an all-'N' one included), and a threading problem (one sequence more than
    leaves)."""
    out_dir = os.path.join(HERE, "argprob")
    os.makedirs(out_dir, exist_ok=True)
    cases = []
    cases.append(("full_k10", simulate(10, 1500, 205, add_thread=False)))
    cases.append(("full_k24_T16", simulate(24, 4000, 31, add_thread=False, ntimes=16)))
    p = simulate(12, 3000, 77, add_thread=False, missing=0.02)
    starts = np.concatenate([[0], np.cumsum(p.blocklens)[:-1]])
    seqs = p.seqs.copy()
    seqs[:, starts[::2]] = ord("N")
    p.seqs = seqs
    cases.append(("full_k12_masked", p))
    cases.append(("thread_k8", simulate(7, 2000, 12)))
    for name, prob in cases:
        pp = os.path.join(out_dir, name + ".prob")
        prob.save(pp)
        ob = os.path.join(tmp, "ap.bin")
        run("argprob", pp, ob)
        v = np.fromfile(ob, dtype=np.float64)
        np.savez(os.path.join(out_dir, name + ".npz"), likelihood=v[0], prior=v[1],
                 tree_prior=v[2], joint=v[3])
        print(name, v)


def formats(tmp):
    """Sites and SMC files written by this library from seeded full ARGs (1 bp per column),
    read back by the reference the way arg-sample reads them (harness `ingest`), at
    compression 1 and 10 (1 and 4 where missing calls make most columns variant: the
    reference refuses 10 there); one pair gzip-compressed."""
    from argweaver_gb300 import formats as fm
    out_dir = os.path.join(HERE, "formats")
    os.makedirs(out_dir, exist_ok=True)
    for name, k, L, seed, missing, gz, comp in (("k8", 8, 30000, 61, 0.0, False, (1, 10)),
                                                ("k16_missing", 16, 8000, 62, 0.01, True, (1, 4))):
        prob = simulate(k, L, seed, compress=1, add_thread=False, missing=missing)
        names = [f"n{i}" for i in range(prob.nseqs)]
        ext = ".gz" if gz else ""
        sites = os.path.join(out_dir, name + ".sites" + ext)
        smc = os.path.join(out_dir, name + ".smc" + ext)
        fm.write_sites(sites, names, prob.seqs)
        fm.write_smc(smc, prob, names)
        for c in comp:
            pc = os.path.join(out_dir, f"{name}_c{c}.prob")
            run("ingest", sites, smc, c, pc)
            # the reference's probabilities of the ARG it read
            ob = os.path.join(tmp, "ap.bin")
            run("argprob", pc, ob)
            v = np.fromfile(ob, dtype=np.float64)
            np.savez(os.path.join(out_dir, f"{name}_c{c}.npz"), likelihood=v[0], prior=v[1],
                     tree_prior=v[2], joint=v[3])
            print(name, c, v)


def recomb(tmp):
    """sample_recombinations (recomb.cpp:151-235) along each fixture's sampled path, after
    srand(seed + 7000): the recombination positions, nodes and times, and the rand() value
    that follows (which pins how many draws the sampler consumed)."""
    out_dir = os.path.join(HERE, "recomb")
    os.makedirs(out_dir, exist_ok=True)
    for f in sorted(os.listdir(HERE)):
        if not f.endswith(".npz"):
            continue
        name = f[:-4]
        gold = np.load(os.path.join(HERE, f))
        if "path" not in gold.files:
            continue
        pp = os.path.join(HERE, name + ".prob")
        path_file = os.path.join(tmp, "path.bin")
        np.ascontiguousarray(gold["path"], dtype=np.int32).tofile(path_file)
        seed = int(gold["seed"]) + 7000
        ob = os.path.join(tmp, "rec.bin")
        run("recomb", pp, path_file, seed, ob)
        d = open(ob, "rb").read()
        assert d[:8] == b"AWGREC01"
        n, nxt = (int(x) for x in np.frombuffer(d, np.int32, 2, 8))
        rec = np.frombuffer(d, np.int32, 3 * n, 16).reshape(n, 3)
        np.savez(os.path.join(out_dir, name + ".npz"), seed=seed, pos=rec[:, 0].copy(),
                 node=rec[:, 1].copy(), time=rec[:, 2].copy(), next_rand=nxt)
        print(name, n)
    # larger external problems, paths drawn by the oracle's traceback (pinned to the
    # reference's) after srand(seed): many more state changes
    for k, L, seed, T, missing, rho in ((12, 10000, 73, 32, 0.01, 1.6e-7),
                                        (8, 15000, 74, 20, 0.0, 5e-7)):
        name = f"extra_k{k}_T{T}"
        prob = simulate(k, L, seed, ntimes=T, missing=missing, rho=rho)
        pp = os.path.join(out_dir, name + ".prob")
        prob.save(pp)
        fw, _ = pyoracle.forward(prob)
        path = pyoracle.traceback(prob, fw, pyoracle.rand_uniforms(seed, prob.seqlen))
        path_file = os.path.join(tmp, "path.bin")
        np.ascontiguousarray(path, dtype=np.int32).tofile(path_file)
        rseed = seed + 7000
        ob = os.path.join(tmp, "rec.bin")
        run("recomb", pp, path_file, rseed, ob)
        d = open(ob, "rb").read()
        n, nxt = (int(x) for x in np.frombuffer(d, np.int32, 2, 8))
        rec = np.frombuffer(d, np.int32, 3 * n, 16).reshape(n, 3)
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), seed=rseed,
                            path=path.astype(np.int32), pos=rec[:, 0].copy(),
                            node=rec[:, 1].copy(), time=rec[:, 2].copy(), next_rand=nxt)
        print(name, n)


def addthread(tmp):
    """add_arg_thread (thread.cpp:272-422): the recombination fixtures' threads and
    recombinations added to their problems' trees by the reference; the grown ARG."""
    out_dir = os.path.join(HERE, "addthread")
    os.makedirs(out_dir, exist_ok=True)
    rdir = os.path.join(HERE, "recomb")
    for f in sorted(os.listdir(rdir)):
        if not f.endswith(".npz"):
            continue
        name = f[:-4]
        rec = np.load(os.path.join(rdir, f))
        if name.startswith("extra_"):
            if name != "extra_k8_T20":
                continue
            pp = os.path.join(rdir, name + ".prob")
            path = rec["path"]
        else:
            pp = os.path.join(HERE, name + ".prob")
            path = np.load(os.path.join(HERE, name + ".npz"))["path"]
        if Problem.load(pp).internal:
            continue
        path_file = os.path.join(tmp, "path.bin")
        np.ascontiguousarray(path, dtype=np.int32).tofile(path_file)
        rec_file = os.path.join(tmp, "rec.bin")
        np.ascontiguousarray(np.stack([rec["pos"], rec["node"], rec["time"]], axis=1),
                             dtype=np.int32).tofile(rec_file)
        run("addthread", pp, path_file, rec_file, os.path.join(out_dir, name + ".prob"))
        print(name, len(rec["pos"]))


def addthreadpath(tmp):
    """add_arg_thread_path (thread.cpp:1314-1449): the internal fixtures' thread paths and
    recombinations regrafted into their cut ARGs by the reference; the whole ARG."""
    out_dir = os.path.join(HERE, "addthreadpath")
    os.makedirs(out_dir, exist_ok=True)
    rdir = os.path.join(HERE, "recomb")
    for f in sorted(os.listdir(rdir)):
        if not f.endswith(".npz") or f.startswith("extra_"):
            continue
        name = f[:-4]
        pp = os.path.join(HERE, name + ".prob")
        if not Problem.load(pp).internal:
            continue
        rec = np.load(os.path.join(rdir, f))
        path = np.load(os.path.join(HERE, name + ".npz"))["path"]
        path_file = os.path.join(tmp, "path.bin")
        np.ascontiguousarray(path, dtype=np.int32).tofile(path_file)
        rec_file = os.path.join(tmp, "rec.bin")
        np.ascontiguousarray(np.stack([rec["pos"], rec["node"], rec["time"]], axis=1),
                             dtype=np.int32).tofile(rec_file)
        out = os.path.join(tmp, name + ".prob")
        run("addthreadpath", pp, path_file, rec_file, out)
        q = Problem.load(out)
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), ptrees=q.ptrees, ages=q.ages,
                            sprs=q.sprs, blocklens=q.blocklens, mapping=q.mapping,
                            root_child0=q.root_child0,
                            thread_times=np.fromfile(out + ".times", dtype=np.int32)
                            if os.path.exists(out + ".times") else np.zeros(0, np.int32))
        print(name, len(rec["pos"]), q.ntrees)


def samplethreadinternal(tmp):
    """sample_arg_thread_internal (sample_thread.cpp:635-692) after srand(seed + 9100) on the
    internal fixtures: the whole ARG with the cut subtree re-threaded, as the reference does."""
    out_dir = os.path.join(HERE, "samplethreadinternal")
    os.makedirs(out_dir, exist_ok=True)
    for name in ("cut_k10_s3", "cut_k10_s8", "cut_k10_s17", "cut_k10_s24", "infsites_cut_k10_s5"):
        pp = os.path.join(HERE, name + ".prob")
        seed = int(np.load(os.path.join(HERE, name + ".npz"))["seed"]) + 9100
        out = os.path.join(tmp, name + ".prob")
        run("samplethreadinternal", pp, seed, out)
        q = Problem.load(out)
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), seed=seed, ptrees=q.ptrees,
                            ages=q.ages, sprs=q.sprs, blocklens=q.blocklens, mapping=q.mapping,
                            root_child0=q.root_child0)
        print(name, q.ntrees)


def resampleleaf(tmp):
    """resample_arg_leaf's move (sample_arg.cpp:66-86) after srand(seed) on grown ARGs: a
    sequence removed and threaded back in; the ARG with leaves named by sequence."""
    out_dir = os.path.join(HERE, "resampleleaf")
    os.makedirs(out_dir, exist_ok=True)
    for name, seqid, seed in (("dsmc_k8_s11", 2, 401), ("dsmc_k10_T16", 0, 402),
                              ("single_k7_s41", 6, 403), ("sim1_c20", 4, 404)):
        pp = os.path.join(HERE, "addthread", name + ".prob")
        out = os.path.join(tmp, name + ".prob")
        run("resampleleaf", pp, seqid, seed, out)
        q = Problem.load(out)
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), seqid=seqid, seed=seed,
                            ptrees=q.ptrees, ages=q.ages, sprs=q.sprs, blocklens=q.blocklens,
                            mapping=q.mapping)
        print(name, q.ntrees)


def samplethread(tmp):
    """arghmm_sample_thread (sample_thread.cpp:1010-1023) after srand(seed + 9000) on the
    external fixtures: the ARG with the last sequence threaded in, as the reference grows it."""
    out_dir = os.path.join(HERE, "samplethread")
    os.makedirs(out_dir, exist_ok=True)
    for name in ("dsmc_k8_s11", "dsmc_k8_s12", "dsmc_k10_T16", "dsmc_k17_missing", "sim1_c20",
                 "single_k7_s41"):
        pp = os.path.join(HERE, name + ".prob")
        seed = int(np.load(os.path.join(HERE, name + ".npz"))["seed"]) + 9000
        run("samplethread", pp, seed, os.path.join(out_dir, name + ".prob"))
        np.savez(os.path.join(out_dir, name + ".npz"), seed=seed)
        print(name, Problem.load(os.path.join(out_dir, name + ".prob")).ntrees)


# sequences removed in turn from the grown ARGs (removal orders: the last leaf, middle
# leaves, the first; one run down to the trunk genealogy)
REMOVALS = {
    "dsmc_k8_s11": [3, 0, 7, 5, 1, 6, 2],
    "dsmc_k10_T16": [9, 4],
    "dsmc_k17_missing": [0, 16, 8, 3],
    "sim1_c20": [2, 5],
    "single_k7_s41": [6, 0, 1],
}


def removethread(tmp):
    """remove_arg_thread (thread.cpp:425-556) on the ARGs add_arg_thread grew: after each
    removal, the trees in the names get_local_trees_ptrees gives (leaf names when the
    sequence ids are no permutation of the leaves), mappings, root children and sequence ids."""
    out_dir = os.path.join(HERE, "removethread")
    os.makedirs(out_dir, exist_ok=True)
    for name, ids in REMOVALS.items():
        pp = os.path.join(HERE, "addthread", name + ".prob")
        prefix = os.path.join(tmp, name)
        run("removethread", pp, prefix, *ids)
        arrays = {"removed": np.asarray(ids, dtype=np.int32)}
        for i in range(len(ids)):
            q = Problem.load(f"{prefix}.{i}.prob")
            arrays[f"ptrees_{i}"] = q.ptrees
            arrays[f"ages_{i}"] = q.ages
            arrays[f"sprs_{i}"] = q.sprs
            arrays[f"blocklens_{i}"] = q.blocklens
            arrays[f"mapping_{i}"] = q.mapping
            arrays[f"root_child0_{i}"] = q.root_child0
            arrays[f"seqids_{i}"] = np.fromfile(f"{prefix}.{i}.seqids", dtype=np.int32)
        np.savez_compressed(os.path.join(out_dir, name + ".npz"), **arrays)
        print(name, [int(arrays[f"ptrees_{i}"].shape[0]) for i in range(len(ids))])


# (fixture, seed, node, position as a fraction of the region) for the removal-path fixtures
REMOVAL_PATHS = [
    ("dsmc_k8_s11", 301, 3, 0.5),
    ("dsmc_k8_s12", 302, 11, 0.03),
    ("dsmc_k10_T16", 303, 12, 0.45),
    ("dsmc_k17_missing", 304, 20, 0.75),
    ("sim1_c20", 305, 9, 0.6),
    ("single_k7_s41", 306, 2, 0.0),
    ("extra_k8_T20", 307, 5, 0.9),
]


def removalpaths(tmp):
    """Removal paths through the grown ARGs after srand(seed) (uniform, forward from a node,
    through a node at a position, the leaf path of leaf 0; thread.cpp:672-1002) and the ARG
    cut along the uniform path (remove_arg_thread_path, thread.cpp:1481-1668)."""
    out_dir = os.path.join(HERE, "removalpaths")
    os.makedirs(out_dir, exist_ok=True)
    for name, seed, node, frac in REMOVAL_PATHS:
        pp = os.path.join(HERE, "addthread", name + ".prob")
        prob = Problem.load(pp)
        off = int(frac * int(np.sum(prob.blocklens)))
        prefix = os.path.join(tmp, name)
        run("removalpaths", pp, seed, node, prob.start_coord + off, prefix)
        paths = np.fromfile(prefix + ".paths", dtype=np.int32).reshape(5, prob.ntrees)
        cut = Problem.load(prefix + ".cut.prob")
        np.savez_compressed(
            os.path.join(out_dir, name + ".npz"), seed=seed, node=node,
            pos=prob.start_coord + off, paths=paths,
            lntotal=np.fromfile(prefix + ".lntotal", dtype=np.float64)[0],
            original_thread=np.fromfile(prefix + ".orig", dtype=np.int32),
            ptrees=cut.ptrees, ages=cut.ages, sprs=cut.sprs, blocklens=cut.blocklens,
            mapping=cut.mapping, root_child0=cut.root_child0)
        print(name, prob.ntrees, "->", cut.ntrees)


def infsites(tmp):
    """The infinite-sites penalty (ArgModel::infsites_penalty, emit.cpp:847-862; arg-sample
    --infsites uses 1e-100): external, with missing calls, and an internal-branch cut."""
    prob = simulate(7, 3000, 13)
    p = os.path.join(tmp, "p.prob"); prob.save(p)
    make("infsites_k8_s13", p, 113, tmp, penalty=1e-3)
    prob = simulate(16, 1500, 22, missing=0.02)
    p = os.path.join(tmp, "p.prob"); prob.save(p)
    make("infsites_k17_missing", p, 122, tmp, penalty=1e-100)
    full = simulate(10, 1500, 205, add_thread=False)
    pf = os.path.join(tmp, "full.prob"); full.save(pf)
    pc = os.path.join(tmp, "cut.prob")
    run("cut", pf, 5, pc)
    make("infsites_cut_k10_s5", pc, 505, tmp, penalty=1e-3)


def cut_leaves(prob: Problem) -> int:
    """Most leaves under the cut subtree (each root's child[0]) over the trees of a cut."""
    best = 0
    for b in range(prob.ntrees):
        par = prob.ptrees[b]
        top = int(prob.root_child0[b])
        nleaves = (prob.nnodes + 1) // 2
        n = 0
        for v in range(nleaves):
            x = v
            while x != -1 and x != top:
                x = par[x]
            n += x == top
        best = max(best, n)
    return best


def large(tmp):
    """Shapes at the configurations' scale, pinned by the reference itself: an external
    problem at k = 48 (config 1's upper range, 0.5% missing calls) and internal-branch cuts
    of k = 50 ARGs along the reference's uniform removal path (config 3's shape), the first
    whose cut subtree holds 3 to 12 leaves and leaves at least 100 states per column."""
    prob = simulate(47, 3000, 41, missing=0.005)
    p = os.path.join(tmp, "p.prob"); prob.save(p)
    make("large_k48_s41", p, 141, tmp)
    made = 0
    for seed in range(1, 40):
        full = simulate(50, 3000, 250 + seed, add_thread=False, missing=0.01)
        pf = os.path.join(tmp, "full.prob"); full.save(pf)
        pc = os.path.join(tmp, "cut.prob")
        run("cut", pf, seed, pc)
        cut = Problem.load(pc)
        n = cut_leaves(cut)
        if n < 3 or n > 12 or cut.cells() < 100 * cut.seqlen:
            continue
        make(f"large_cut_k50_s{seed}", pc, 600 + seed, tmp)
        print(f"  cut subtree: up to {n} leaves")
        made += 1
        if made == 1:
            break


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={REF}"],
                   check=True)
    pyoracle.build()
    if sys.argv[1:] == ["large"]:
        with tempfile.TemporaryDirectory() as tmp:
            large(tmp)
        return
    if sys.argv[1:] == ["infsites"]:
        with tempfile.TemporaryDirectory() as tmp:
            infsites(tmp)
        return
    if sys.argv[1:] == ["resampleleaf"]:
        with tempfile.TemporaryDirectory() as tmp:
            resampleleaf(tmp)
        return
    if sys.argv[1:] == ["samplethreadinternal"]:
        with tempfile.TemporaryDirectory() as tmp:
            samplethreadinternal(tmp)
        return
    if sys.argv[1:] == ["addthreadpath"]:
        with tempfile.TemporaryDirectory() as tmp:
            addthreadpath(tmp)
        return
    if sys.argv[1:] == ["removalpaths"]:
        with tempfile.TemporaryDirectory() as tmp:
            removalpaths(tmp)
        return
    if sys.argv[1:] == ["removethread"]:
        with tempfile.TemporaryDirectory() as tmp:
            removethread(tmp)
        return
    if sys.argv[1:] == ["samplethread"]:
        with tempfile.TemporaryDirectory() as tmp:
            samplethread(tmp)
        return
    if sys.argv[1:] == ["addthread"]:
        with tempfile.TemporaryDirectory() as tmp:
            addthread(tmp)
        return
    if sys.argv[1:] == ["recomb"]:
        with tempfile.TemporaryDirectory() as tmp:
            recomb(tmp)
        return
    if sys.argv[1:] == ["formats"]:
        with tempfile.TemporaryDirectory() as tmp:
            formats(tmp)
        return
    if sys.argv[1:] == ["argprob"]:
        with tempfile.TemporaryDirectory() as tmp:
            argprob(tmp)
        return
    if sys.argv[1:] == ["helpers"]:
        with tempfile.TemporaryDirectory() as tmp:
            helpers(tmp)
        return
    if sys.argv[1:] == ["dense"]:
        with tempfile.TemporaryDirectory() as tmp:
            dense(tmp)
            densernd(tmp)
        return
    with tempfile.TemporaryDirectory() as tmp:
        infsites(tmp)
        # the reference's bundled example, re-threading its last sequence (k=8, 100 kb)
        p = os.path.join(HERE, "sim1_c20.prob")
        run("sim1", os.path.join(REF, "examples/sim1/sim1.sites"),
            os.path.join(REF, "examples/sim1/sim1.sample/out.100.smc.gz"), 20, p)
        make("sim1_c20", p, 7, tmp)

        # config-0 shape (k=8: 7 leaves + 1 threaded), shortened
        for seed in (11, 12):
            prob = simulate(7, 4000, seed)
            p = os.path.join(tmp, "p.prob"); prob.save(p)
            make(f"dsmc_k8_s{seed}", p, 100 + seed, tmp)

        # missing data and a larger tree
        prob = simulate(16, 2000, 21, missing=0.02)
        p = os.path.join(tmp, "p.prob"); prob.save(p)
        make("dsmc_k17_missing", p, 121, tmp)

        # ntimes 16 and 32
        for T, seed in ((16, 31), (32, 32)):
            prob = simulate(9, 1500, seed, ntimes=T)
            p = os.path.join(tmp, "p.prob"); prob.save(p)
            make(f"dsmc_k10_T{T}", p, 100 + seed, tmp)

        # internal-branch cuts by the reference's uniform removal path
        for seed in (3, 8, 17, 24):
            full = simulate(10, 2000, 200 + seed, add_thread=False)
            pf = os.path.join(tmp, "full.prob"); full.save(pf)
            pc = os.path.join(tmp, "cut.prob")
            run("cut", pf, seed, pc)
            make(f"cut_k10_s{seed}", pc, 500 + seed, tmp)

        large(tmp)
        dense(tmp)
        densernd(tmp)
        argprob(tmp)
        helpers(tmp)
        formats(tmp)
        recomb(tmp)
        addthread(tmp)
        samplethread(tmp)
        removethread(tmp)
        removalpaths(tmp)
        addthreadpath(tmp)
        samplethreadinternal(tmp)
        resampleleaf(tmp)


if __name__ == "__main__":
    main()
