#!/usr/bin/env python3
"""Benchmark: batched threading HMM, forward + stochastic traceback, state-cells/s.

Workload (the headline configuration): 256 independent threading problems, each a seeded
DSMC ARG with k ~ U{8..64} haplotypes (k-1 in the ARG, one re-threaded), L ~ U[100 kb,
1 Mb] at 10 bp per column, ntimes=20, N=1e4, r=1.6e-8, mu=1.8e-8, 0.5% missing calls.
One step = forward + traceback of the whole batch in FP32 (log scales in FP64).

  value     cells / device time of the step's kernels (upload done, downloads not begun)
  e2e       cells / wall time of K steps through the public API with host buffers, two
            batch contexts in turn (each step: bind, plan, host->device copy of the inputs,
            kernels, device->host copy of the paths; the next step's host work overlaps
            the current step's kernels); `sync_call` beside it: one awg_run_batch call per
            step, waited for, with p50/p99 of its latency
  roofline  the forward kernel: 4 B of FP32 table written per cell over its time (phases
            timed one after another), against the measured HBM copy bandwidth
  fp64_plain  the drop-in FP64 path, one problem per reference C-ABI call
  cpu_baseline  the CPU port of the reference's algorithm (oracle/) on the host cores,
            one problem per thread, on a bounded sample of the same problems

Flags: --gpus N --steps K --warmup W [--impl reference] [--instances n] [--seed s]
Multi-GPU: replicas (each rank threads its own 256 problems; weak scaling).
"""

from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "HMM state-cells/s fwd+traceback, batched FP32 vs plain FP64 @<=1e-5 err; p50/p99"
FWD_DRAM_BYTES_PER_CELL = 7.26  # forward kernel, ncu capture summarised in profiles/
UNIT = "state-cells/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--instances", type=int, default=256)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--cpu-sample-seconds", type=float, default=15.0)
    ap.add_argument("--configs", type=int, default=1,
                    help="also measure the single-instance, large-instance, internal-batch "
                         "and serving configurations (0: skip)")
    ap.add_argument("--max-columns", type=int, default=0,
                    help="cap each problem's length (small cases for profiling)")
    ap.add_argument("--one-instance", default="",
                    help="K,L: run one seeded problem (K haplotypes, L columns, ntimes 20, 0.5%% "
                         "missing) once, FP32 forward + traceback, print its cell count and "
                         "exit (a single launch of each kernel, for ncu captures)")
    return ap.parse_args()


def one_instance(spec: str, seed: int):
    from argweaver_gb300 import api
    from argweaver_gb300.sim import simulate

    k, L = (int(x) for x in spec.split(","))
    p = simulate(k - 1, L, seed, compress=10, ntimes=20, maxtime=200e3, popsize=1e4,
                 rho=1.6e-8, mu=1.8e-8, missing=0.005)
    api.run_batch([p], precision="fp32", want_forward=False, want_path=True)
    print(json.dumps({"one_instance": {"k": k, "columns": L, "seed": seed,
                                       "cells": int(p.cells()), "trees": int(p.ntrees),
                                       "max_states": int(p.nstates_per_tree().max())}}))


def make_workload(n: int, seed: int, rank: int = 0, max_columns: int = 0):
    from argweaver_gb300.sim import simulate

    rng = np.random.default_rng(seed + 7919 * rank)
    ks = rng.integers(8, 65, size=n)                # haplotypes incl. the re-threaded one
    bps = rng.uniform(1e5, 1e6, size=n)
    seeds = rng.integers(1, 2**62, size=n)
    specs = [(int(k) - 1, int(bp // 10), int(s)) for k, bp, s in zip(ks, bps, seeds)]
    if max_columns:
        specs = [(k, min(L, max_columns), s) for k, L, s in specs]

    def one(spec):
        nl, L, s = spec
        return simulate(nl, L, s, compress=10, ntimes=20, maxtime=200e3, popsize=1e4,
                        rho=1.6e-8, mu=1.8e-8, missing=0.005)

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        return list(ex.map(one, specs))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                 f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm = [float(r[0]) for r in self.rows if r and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) > 1 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4)
                          if len(r) > 2 + i and r[2 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(sm)}


def cpu_reference(problems, seconds: float, threads: int):
    """Time the oracle's forward+traceback (the reference's algorithm, ported to C) on
    problems, one per thread, until about `seconds` of wall time; returns cells/s."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle

    pyoracle.load()
    done_cells = [0]
    lock = threading.Lock()
    order = sorted(range(len(problems)), key=lambda i: problems[i].cells())
    t0 = time.perf_counter()
    deadline = t0 + seconds

    def work(i):
        if time.perf_counter() > deadline:
            return
        p = problems[i]
        fw, _ = pyoracle.forward(p)
        u = np.random.default_rng(i).random(p.seqlen)
        pyoracle.traceback(p, fw, u)
        with lock:
            done_cells[0] += fw.size

    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(work, order))
    dt = time.perf_counter() - t0
    return done_cells[0] / dt, done_cells[0], dt


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def _sim_pool(specs):
    """Problems simulated in parallel from (nleaves, columns, seed, ntimes, missing) specs."""
    from argweaver_gb300.sim import simulate

    def one(spec):
        nl, L, sd, T, miss = spec
        return simulate(nl, L, sd, compress=10, ntimes=T, maxtime=200e3, popsize=1e4,
                        rho=1.6e-8, mu=1.8e-8, missing=miss)

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        return list(ex.map(one, specs))


def _prefix(p, columns):
    """The problem cut to its first `columns` columns (whole trees, the last one shortened)."""
    from argweaver_gb300.problem import Problem

    ends = np.cumsum(p.blocklens)
    B = int(np.searchsorted(ends, columns) + 1)
    bl = p.blocklens[:B].copy()
    bl[-1] -= int(ends[B - 1] - columns) if ends[B - 1] > columns else 0
    L = int(bl.sum())
    return Problem(times=p.times, popsizes=p.popsizes, rho=p.rho, mu=p.mu,
                   ptrees=p.ptrees[:B].copy(), ages=p.ages[:B].copy(), sprs=p.sprs[:B].copy(),
                   blocklens=bl, seqs=p.seqs[:, :L].copy(), internal=p.internal,
                   mapping=None if p.mapping is None else p.mapping[:B].copy(),
                   root_child0=None if p.root_child0 is None else p.root_child0[:B].copy())


def config_runs(seed: int):
    """The other configurations of the benchmark spec, each measured once with a bounded workload:
    c0 the plain FP64 single instance, c2 one large instance in FP32 and FP64, c3 the
    internal-branch batch under the autotuned schedule and graph replay, c4 the serving
    loop under Poisson arrivals."""
    from argweaver_gb300 import api

    out = {}
    rng = np.random.default_rng(seed + 17)

    def guarded(name, fn):
        try:
            out[name] = fn()
        except Exception as e:  # one configuration failing leaves the others' results
            out[name] = {"error": f"{type(e).__name__}: {e}"}
        api.release_memory()

    guarded("c0_plain_fp64_single", lambda: _c0(rng))
    guarded("c2_large_single", lambda: _c2(rng))
    guarded("c3_internal_batch", lambda: _c3(rng))
    guarded("c4_serving", lambda: _c4(rng))
    return out


def _c0(rng):
    from argweaver_gb300 import refapi

    # ---- c0: k = 8 (7 leaves + the threaded haplotype), 100 kb = 10,000 columns, FP64
    p0 = _sim_pool([(7, 10000, int(rng.integers(1, 2**62)), 20, 0.0)])[0]
    refapi.arghmm_sample_posterior(p0)
    lat = []
    for _ in range(20):
        t0 = time.perf_counter()
        refapi.arghmm_sample_posterior(p0)
        lat.append(1e3 * (time.perf_counter() - t0))
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    t0 = time.perf_counter()
    fw, _ = pyoracle.forward(p0)
    pyoracle.traceback(p0, fw, np.random.default_rng(1).random(p0.seqlen))
    cpu_ms = 1e3 * (time.perf_counter() - t0)
    from argweaver_gb300 import api
    api.set_timing(2)
    api.run_batch([p0], precision="fp64", want_forward=False, want_path=True)
    phases = api.last_timings()
    api.set_timing(0)
    return {
        "phase_ms": phases,
        "workload": "k=8 (7 + 1 threaded), 10,000 columns, ntimes=20, FP64, one "
                    "arghmm_sample_posterior call (reference C ABI)",
        "cells": int(p0.cells()), "p50_ms": float(np.percentile(lat, 50)),
        "p99_ms": float(np.percentile(lat, 99)),
        "cells_per_s": p0.cells() / (np.median(lat) / 1e3),
        "cpu_port_1core_ms": cpu_ms}


def _c2(rng):
    from argweaver_gb300 import api

    # ---- c2: k = 100, 10 Mb = 1e6 columns, FP32 and FP64 forward + traceback
    p2 = _sim_pool([(99, 1000000, int(rng.integers(1, 2**62)), 20, 0.0)])[0]
    c2 = {"workload": "k=100 (99 + 1 threaded), 1e6 columns (10 Mb at 10 bp), ntimes=20",
          "cells": int(p2.cells()), "trees": int(p2.ntrees),
          "max_states": int(p2.nstates_per_tree().max())}
    u2 = np.random.default_rng(2).random(p2.seqlen)
    for prec in ("fp32", "fp64"):
        api.set_timing(1)
        api.run_batch([p2], precision=prec, want_forward=False, want_path=True, uniforms=[u2])
        t0 = time.perf_counter()
        api.run_batch([p2], precision=prec, want_forward=False, want_path=True, uniforms=[u2])
        wall = time.perf_counter() - t0
        dev = api.last_timings()["compute"] / 1e3
        api.set_timing(0)
        c2[prec] = {"value": p2.cells() / dev, "e2e": p2.cells() / wall,
                    "ms": 1e3 * dev, "e2e_ms": 1e3 * wall}
    c2["fp32_speedup_over_fp64"] = c2["fp32"]["value"] / c2["fp64"]["value"]
    q2 = _prefix(p2, 50000)
    a = api.run_batch([q2], precision="fp32", want_forward=False, want_posterior=True)[0]
    b = api.run_batch([q2], precision="fp64", want_forward=False, want_posterior=True)[0]
    c2["fp32_vs_fp64_posterior_max_abs_err"] = float(np.max(np.abs(a.posterior - b.posterior)))
    c2["error_sample"] = "the instance's first 50,000 columns"
    return c2


def _cut_one(spec):
    """One config-3 instance: a seeded k = 50 ARG cut along a uniform removal path drawn
    after srand(seed) (arg-sample's subtree cut), as an internal-branch problem. Runs in a
    worker process: the removal path draws from libc rand(), which is process-wide."""
    from argweaver_gb300 import refapi
    from argweaver_gb300.sim import simulate

    nleaves, L, seed, miss = spec
    full = simulate(nleaves, L, seed, compress=10, ntimes=20, maxtime=200e3, popsize=1e4,
                    rho=1.6e-8, mu=1.8e-8, missing=miss, add_thread=False)
    refapi.srand(seed % 2**31)
    path, _ = refapi.sample_arg_removal_path_uniform(full)
    return refapi.as_problem(full, refapi.remove_arg_thread_path(full, path), internal=True)


def _c3(rng):
    import multiprocessing as mp

    from argweaver_gb300 import api

    # ---- c3: 128 internal-branch instances, k = 50, 2 Mb = 2e5 columns, missing ~U[0,2%],
    # each a random subtree cut along a uniform removal path (built off the clock, in
    # worker processes started with spawn)
    specs = [(50, 200000, int(rng.integers(1, 2**62)), float(rng.uniform(0, 0.02)))
             for _ in range(128)]
    with cf.ProcessPoolExecutor(max_workers=min(16, os.cpu_count() or 4),
                                mp_context=mp.get_context("spawn")) as ex:
        p3 = list(ex.map(_cut_one, specs))
    cells3 = sum(p.cells() for p in p3)
    u3 = [np.random.default_rng(300 + i).random(p.seqlen) for i, p in enumerate(p3)]
    sched3 = api.autotune(p3, precision="fp32", want_path=True, trials=1)
    api.set_timing(1)
    for _ in range(2):
        api.run_batch(p3, precision="fp32", want_forward=False, want_path=True, uniforms=u3)
    g0 = api.graph_counts()
    dev3, wall3 = [], []
    for _ in range(3):
        t0 = time.perf_counter()
        api.run_batch(p3, precision="fp32", want_forward=False, want_path=True, uniforms=u3)
        wall3.append(time.perf_counter() - t0)
        dev3.append(api.last_timings()["compute"] / 1e3)
    api.set_timing(0)
    return {
        "workload": "128 internal-branch threading problems, k=50, 2e5 columns (2 Mb), "
                    "ntimes=20, missing ~U[0,2%], FP32 forward + traceback; each a seeded ARG "
                    "cut along a uniform removal path (the subtree changes along the genome)",
        "states_per_column_mean": cells3 / sum(p.seqlen for p in p3),
        "cells_per_step": int(cells3), "value": cells3 / float(np.mean(dev3)),
        "e2e": cells3 / float(np.mean(wall3)), "ms_per_step": 1e3 * float(np.mean(dev3)),
        "schedule": sched3,
        "graph_replays": api.graph_counts()["replays"] - g0["replays"]}


def _serve_once(pool, rate, duration, rng, max_inflight=24, max_batch=32, length_ratio=1.25):
    """Poisson arrivals at `rate` requests/s for `duration` s, requests drawn from `pool`
    with fresh uniforms, FP32, through the serving loop; the server's statistics. Batches
    group requests within 1.25x of the oldest's length (the library's default is 2x): at 10
    and 40 requests/s it cut the p50 latency by 28% and 41% for 11% less throughput at 40."""
    from argweaver_gb300.server import Server

    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * duration * 1.5) + 8))
    arrivals = arrivals[arrivals < duration]
    picks = rng.integers(0, len(pool), size=arrivals.size)
    unis = [np.random.default_rng(1000 + q).random(pool[j].seqlen) for q, j in enumerate(picks)]
    with Server(device_bytes=96 << 30, max_inflight=max_inflight, max_batch=max_batch,
                length_ratio=length_ratio) as srv, \
            cf.ThreadPoolExecutor(max_workers=8) as clients:
        t_start = time.perf_counter()
        futs = []
        for q, (t_arr, j) in enumerate(zip(arrivals, picks)):
            delay = t_start + t_arr - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            futs.append(clients.submit(srv.submit, pool[j], precision="fp32", uniforms=unis[q]))
        for f in futs:
            srv.wait(f.result())
        st = srv.stats()
    return st, arrivals.size, sum(pool[j].cells() for j in picks)


def _c4(rng):
    from argweaver_gb300 import api, refapi

    # ---- c4: serving. Requests drawn from config 4's distribution (k log-U[8,200],
    # 50 kb - 5 Mb log-uniform, ntimes in {16, 20, 32}), pre-simulated (off the clock), a
    # pool of distinct ARGs reused with fresh uniforms; Poisson arrivals, swept over rates
    npool = 160
    specs = []
    for _ in range(npool):
        k = int(np.exp(rng.uniform(np.log(8), np.log(200))))
        L = int(np.exp(rng.uniform(np.log(5e3), np.log(5e5))))
        T = int(rng.choice([16, 20, 32]))
        specs.append((k - 1, L, int(rng.integers(1, 2**62)), T, 0.005))
    pool = _sim_pool(specs)
    mean_cells = float(np.mean([p.cells() for p in pool]))
    # a request's own time: a sample of the pool run alone (one problem per batch)
    alone = {}
    for j in rng.permutation(npool)[:24]:
        api.run_batch([pool[j]], precision="fp32", want_forward=False, want_path=True)
        t0 = time.perf_counter()
        api.run_batch([pool[j]], precision="fp32", want_forward=False, want_path=True)
        alone[int(j)] = 1e3 * (time.perf_counter() - t0)
    api.release_memory()
    sweep = []
    for rate in (10.0, 20.0, 40.0, 80.0, 160.0):
        st, n, offered_cells = _serve_once(pool, rate, 8.0, rng)
        row = {"rate": rate, "requests": int(st["completed"]), "failed": int(st["failed"]),
               "throughput": st["cells"] / st["span_s"] if st["span_s"] > 0 else None,
               "offered": offered_cells / 8.0,
               "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
               "queue_p50_ms": st["queue_p50_ms"], "queue_p99_ms": st["queue_p99_ms"],
               "service_p50_ms": st["service_p50_ms"], "service_p99_ms": st["service_p99_ms"],
               "batches_in_flight_max": int(st["inflight_max"])}
        sweep.append(row)
        if st["p99_ms"] > 30000:  # past saturation: the queue grows without bound
            break
    # saturation: the highest rate whose throughput still follows the offered load (80% of
    # it: the measured span runs past the 8 s of arrivals by the last requests' own time, up
    # to a few seconds for the largest, so even an idle server shows less than the offered)
    sat = None
    for row in sweep:
        if row["throughput"] and row["throughput"] >= 0.8 * row["offered"]:
            sat = row
    # the plain FP64 per-request path: one arghmm_sample_posterior call per request, no
    # batching, on requests drawn from the same pool (bounded to ~6 s)
    lat64, c64, t64 = [], 0, 0.0
    for j in rng.permutation(npool):
        t0 = time.perf_counter()
        refapi.arghmm_sample_posterior(pool[j])
        dt = time.perf_counter() - t0
        lat64.append(1e3 * dt)
        c64 += pool[j].cells()
        t64 += dt
        if t64 > 6.0:
            break
    return {
        "workload": f"Poisson arrivals swept over rates (8 s each) of requests drawn from {npool} "
                    "pre-simulated ARGs: k log-U[8,200], 5e3-5e5 columns log-uniform, ntimes "
                    "in {16,20,32}, FP32 forward + traceback per request, batches of requests "
                    "within 1.25x of their oldest's length; the configured 2000 requests/s "
                    "would offer about 1e11 cells/s, above one GPU's capacity",
        "unit": UNIT, "mean_cells_per_request": mean_cells,
        "sweep": sweep,
        "saturation": sat,
        "alone_ms": {"p50": float(np.percentile(list(alone.values()), 50)),
                     "p99": float(np.percentile(list(alone.values()), 99)),
                     "sample": f"{len(alone)} requests of the pool, each run alone"},
        "fp64_plain_per_request": {"requests": len(lat64),
                                   "p50_ms": float(np.percentile(lat64, 50)),
                                   "p99_ms": float(np.percentile(lat64, 99)),
                                   "throughput": c64 / t64,
                                   "sample": "requests of the same pool, one "
                                             "arghmm_sample_posterior call each, ~6 s"}}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    threads = os.cpu_count() or 1

    if args.one_instance:
        one_instance(args.one_instance, args.seed)
        return

    if args.impl == "reference":
        if rank != 0:
            return
        problems = make_workload(args.instances, args.seed, 0, args.max_columns)
        for _ in range(args.warmup):
            cpu_reference(problems, min(2.0, args.cpu_sample_seconds), threads)
        vals = []
        cells_total, t_total = 0, 0.0
        for _ in range(args.steps):
            v, c, dt = cpu_reference(problems, args.cpu_sample_seconds, threads)
            vals.append(v)
            cells_total += c
            t_total += dt
        v = cells_total / t_total
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded DSMC ARGs)",
            "config": {"workload": "batched threading, 256 problems, k~U{8..64}, "
                                   "L~U[1e4,1e5] columns, ntimes=20, 0.5% missing",
                       "sample": "problems in ascending size until the time budget"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "cpu_model": cpu_model(),
                             "sample": f"{args.cpu_sample_seconds:.0f} s per step of the same "
                                       "problems, smallest first, one per thread"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        }))
        return

    import torch

    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    from argweaver_gb300 import api

    problems = make_workload(args.instances, args.seed, rank, args.max_columns)
    cells = sum(p.cells() for p in problems)
    h2d = sum(p.ptrees.nbytes + p.ages.nbytes + p.sprs.nbytes + p.blocklens.nbytes +
              p.seqs.nbytes for p in problems)
    d2h = sum(4 * p.seqlen + 8 for p in problems)
    rng = np.random.default_rng(args.seed)
    uniforms = [rng.random(p.seqlen) for p in problems]

    def step():
        return api.run_batch(problems, precision="fp32", want_forward=False, want_path=True,
                             uniforms=uniforms)

    # the autotuner's schedule for this batch (outside the timed region): forward CTA size,
    # instance groups, work-queue unit length, persistent per-tree kernels
    schedule = api.autotune(problems, precision="fp32", want_path=True, trials=1)
    api.set_timing(1)
    for _ in range(max(args.warmup, 3)):
        step()
    graphs0 = api.graph_counts()
    launches0 = api.kernel_launches()
    sampler = ClockSampler()
    sampler.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    dev_ms, wall = [], []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step()
        wall.append(time.perf_counter() - t0)
        dev_ms.append(api.last_timings()["compute"])
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    launches = api.kernel_launches() - launches0
    graphs1 = api.graph_counts()

    # e2e: the public API as a caller with a stream of batches uses it: two batch contexts
    # in turn (awg_batch_launch / awg_batch_finish), every step binding, planning and
    # uploading its inputs from host buffers and downloading its paths inside the timed
    # region, the next step's host work overlapping the current step's kernels
    pipe = [api.BatchContext(), api.BatchContext()]

    def launch(c):
        c.launch(problems, precision="fp32", want_path=True, uniforms=uniforms)

    for c in pipe:  # warm-up: arenas grown, each context's graph captured
        launch(c)
        c.finish()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    launch(pipe[0])
    for i in range(1, args.steps):
        launch(pipe[i % 2])
        pipe[(i - 1) % 2].finish()
    pipe[(args.steps - 1) % 2].finish()
    torch.cuda.synchronize()
    pipe_s = time.perf_counter() - t0
    if world > 1:
        torch.distributed.barrier()
    for c in pipe:
        c.close()

    dev_s = sum(dev_ms) / 1e3
    wall_s = sum(wall)
    if world > 1:
        t = torch.tensor([dev_s, wall_s, pipe_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        dev_s, wall_s, pipe_s = float(t[0]), float(t[1]), float(t[2])
    value = world * cells * args.steps / dev_s
    e2e = world * cells * args.steps / pipe_s

    # per-kernel times: the same step with its kernels run one phase after another
    api.set_timing(2)
    phases = []
    for _ in range(2):
        step()
        phases.append(api.last_timings())
    api.set_timing(0)
    phase_ms = {k: float(np.mean([t[k] for t in phases])) for k in phases[0]}

    # the plain FP64 path: one problem per call through the reference's C ABI
    # (arghmm_sample_posterior: forward + traceback), on a size-stratified sample (every
    # 16th problem by cell count), bounded to ~10 s
    from argweaver_gb300 import refapi
    by_size = sorted(problems, key=lambda p: p.cells())
    stratified = by_size[8::16]
    plain_cells, plain_t, plain_n = 0, 0.0, 0
    for p in stratified:
        t0 = time.perf_counter()
        refapi.arghmm_sample_posterior(p)
        plain_t += time.perf_counter() - t0
        plain_cells += p.cells()
        plain_n += 1
        if plain_t > 10.0:
            break
    plain = plain_cells / plain_t

    # the same batch in FP64 on the same GPU (forward + traceback, one batched step)
    api.set_timing(1)
    api.run_batch(problems, precision="fp64", want_forward=False, want_path=True, uniforms=uniforms)
    t0 = time.perf_counter()
    api.run_batch(problems, precision="fp64", want_forward=False, want_path=True, uniforms=uniforms)
    fp64_wall = time.perf_counter() - t0
    fp64_dev = api.last_timings()["compute"] / 1e3
    api.set_timing(0)

    # error report outside the timed region, over every problem of the batch: FP32 against
    # FP64 posterior marginals (forward-backward), in batches of 16 problems
    POST_FLOOR = 1e-3
    max_abs, max_rel, n_floor = 0.0, 0.0, 0
    for j in range(0, len(problems), 16):
        chunk = problems[j:j + 16]
        ra = api.run_batch(chunk, precision="fp32", want_forward=False, want_posterior=True)
        rb = api.run_batch(chunk, precision="fp64", want_forward=False, want_posterior=True)
        for a, b in zip(ra, rb):
            e = np.abs(a.posterior - b.posterior)
            big = b.posterior >= POST_FLOOR
            max_abs = max(max_abs, float(e.max()))
            if big.any():
                max_rel = max(max_rel, float(np.max(e[big] / b.posterior[big])))
            n_floor += int(big.sum())

    if rank != 0:
        return
    configs = None
    if args.configs:
        try:
            configs = config_runs(args.seed)
        except Exception as e:  # the headline line is printed regardless
            configs = {"error": f"{type(e).__name__}: {e}"}
    hbm, src = peaks()
    # dominant kernel: the forward pass, 4 B of FP32 table written per cell
    achieved = cells * 4 / (phase_ms["forward"] / 1e3) / 1e9
    cpu_v, cpu_cells, cpu_dt = cpu_reference(problems, args.cpu_sample_seconds, os.cpu_count() or 1)
    cpu1_v, cpu1_cells, cpu1_dt = cpu_reference(problems, min(5.0, args.cpu_sample_seconds), 1)
    per_inst = sorted(p.cells() for p in problems)
    lat = np.array(wall) * 1e3
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dev_s / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded DSMC ARGs, simulated in-process)",
        "config": {"workload": f"batched threading, {args.instances} problems, k~U{{8..64}}, "
                               "L~U[1e4,1e5] columns (10 bp), ntimes=20, 0.5% missing, "
                               "FP32 forward + traceback, log scales in FP64",
                   "cells_per_step": cells, "instances": args.instances,
                   "cells_per_instance_p50": per_inst[len(per_inst) // 2],
                   "l2": "inputs and tables larger than L2 (129 MB)",
                   "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * pipe_s / args.steps,
                "mode": "two batch contexts in turn (api.BatchContext: awg_batch_launch / "
                        "awg_batch_finish), host work of step i+1 overlapping the kernels "
                        "of step i",
                "sync_call": {"value": world * cells * args.steps / wall_s,
                              "ms_per_step": 1e3 * wall_s / args.steps,
                              "p50_ms": float(np.percentile(lat, 50)),
                              "p99_ms": float(np.percentile(lat, 99)),
                              "mode": "one awg_run_batch call per step, each waiting for "
                                      "the last"}},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm,
                     # DRAM bytes of the forward launches: ncu dram__bytes_read.sum +
                     # dram__bytes_write.sum of one k = 64, 100,000-column launch
                     # (--one-instance 64,100000), 7.26 B per state-cell, scaled to this
                     # step's cells (profiles/forward_traffic_k64_1e5.md)
                     "traffic": FWD_DRAM_BYTES_PER_CELL * cells, "peak_source": src,
                     "kernel": "forward (k_forward_reg), 4 B of FP32 table written per cell, "
                               "timed alone (phases run one after another)"},
        "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                         "cpu_model": cpu_model(),
                         "sample": f"{cpu_cells} cells in {cpu_dt:.1f} s: the same problems, "
                                   "smallest first, one per thread",
                         "value_1core": cpu1_v,
                         "sample_1core": f"{cpu1_cells} cells in {cpu1_dt:.1f} s on one "
                                         "thread, smallest problems first"},
        "fp64_plain": {"value": plain, "unit": UNIT, "speedup_of_value": value / plain,
                       "sample": f"{plain_n} problems, every 16th by cell count, one "
                                 "arghmm_sample_posterior call each (FP64, forward + "
                                 "traceback)"},
        "fp64_batched": {"value": cells / fp64_dev, "e2e": cells / fp64_wall, "unit": UNIT,
                         "ms": 1e3 * fp64_dev, "e2e_ms": 1e3 * fp64_wall,
                         "fp32_speedup": value / (cells / fp64_dev),
                         "workload": "the same 256 problems and uniforms, FP64 forward + "
                                     "traceback, one batched step"},
        "fp32_vs_fp64_posterior_max_rel_err": max_rel,
        "fp32_vs_fp64_posterior_max_abs_err": max_abs,
        "error_floor": POST_FLOOR,
        "error_sample": f"all {len(problems)} problems of the batch, full length; relative "
                        f"error over the {n_floor} cells whose FP64 marginal is >= "
                        f"{POST_FLOOR:g}, absolute error over every cell",
        "gpu_launches": launches,
        "schedule": dict(schedule, graph_replays_in_timed_steps=graphs1["replays"] - graphs0["replays"],
                         note="autotuned once before the timed steps; each step replays the "
                              "captured CUDA graph of its kernels"),
        "clocks": clocks,
        "phase_ms": phase_ms,
        "longest_instance_columns": max(p.seqlen for p in problems),
    }
    if configs is not None:
        line["other_configs"] = configs
    print(json.dumps(line))


if __name__ == "__main__":
    main()
