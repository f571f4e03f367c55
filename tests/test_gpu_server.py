"""The serving loop (GPU only): continuous batching, admission by device memory, resident
requests. Bar: every result served in the mix equals the same problem run alone through
awg_run_batch, bit for bit (FP32 and FP64: the kernels' sums have an order fixed by the
problem), and requests that arrive while others run overlap with them on the GPU.
"""

import threading
import time

import numpy as np
import pytest

from argweaver_gb300 import api
from argweaver_gb300.server import Server
from argweaver_gb300.sim import simulate

pytestmark = pytest.mark.gpu


def mixed_problems(n, seed):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        k = int(np.exp(rng.uniform(np.log(8), np.log(60))))
        L = int(np.exp(rng.uniform(np.log(300), np.log(6000))))
        T = int(rng.choice([16, 20, 32]))
        p = simulate(k, L, seed=seed * 1000 + i, ntimes=T, missing=0.005)
        out.append((p, np.random.default_rng(seed + i).random(p.seqlen)))
    return out


def alone(p, u, precision):
    return api.run_batch([p], precision=precision, want_forward=True, want_path=True,
                         uniforms=[u])[0]


def test_results_in_the_mix_equal_results_alone():
    items = mixed_problems(24, 7)
    precisions = ["fp32" if i % 3 else "fp64" for i in range(len(items))]
    with Server(device_bytes=4 << 30, max_inflight=3, max_batch=6) as srv:
        tickets = [None] * len(items)

        def producer(idx):
            for i in idx:
                p, u = items[i]
                tickets[i] = srv.submit(p, precision=precisions[i], want_forward=True, uniforms=u)
                time.sleep(0.002 * (i % 4))  # arrivals spread while earlier batches run

        threads = [threading.Thread(target=producer, args=(range(j, len(items), 3),))
                   for j in range(3)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        results = [srv.wait(t, timeout=120) for t in tickets]
        st = srv.stats()
    assert st["completed"] == len(items) and st["failed"] == 0
    assert st["inflight_max"] >= 2  # batches overlapped on the GPU
    assert st["p99_ms"] >= st["p50_ms"] > 0
    for (p, u), prec, r in zip(items, precisions, results):
        ref = alone(p, u, prec)
        np.testing.assert_array_equal(r.forward, ref.forward)
        np.testing.assert_array_equal(r.path, ref.path)
        assert r.loglik == ref.loglik


def test_admission_by_device_memory():
    items = mixed_problems(6, 11)
    # a pool that holds a few requests at a time; one request too large for it fails alone
    pool = 64 << 20
    big = simulate(64, 40000, seed=3)
    with Server(device_bytes=pool, max_inflight=4, max_batch=8) as srv:
        ts = [srv.submit(p, uniforms=u) for p, u in items]
        tb = srv.submit(big)
        for t, (p, u) in zip(ts, items):
            r = srv.wait(t, timeout=120)
            np.testing.assert_array_equal(r.path, alone(p, u, "fp32").path)
        with pytest.raises(Exception, match="pool holds"):
            srv.wait(tb, timeout=120)
        st = srv.stats()
    assert st["completed"] == len(items) and st["failed"] == 1


def test_resident_request_resamples_from_its_forward_table():
    p = simulate(20, 3000, seed=21, missing=0.005)
    u1 = np.random.default_rng(1).random(p.seqlen)
    u2 = np.random.default_rng(2).random(p.seqlen)
    with Server(device_bytes=1 << 30, max_inflight=2, max_batch=4) as srv:
        t = srv.submit(p, uniforms=u1, resident=True)
        r = srv.wait(t, timeout=120)
        np.testing.assert_array_equal(r.path, alone(p, u1, "fp32").path)
        # other requests keep flowing while the resident one holds its data
        q = simulate(10, 800, seed=22)
        uq = np.random.default_rng(3).random(q.seqlen)
        rq = srv.wait(srv.submit(q, uniforms=uq), timeout=120)
        np.testing.assert_array_equal(rq.path, alone(q, uq, "fp32").path)
        path2 = srv.resample(t, u2)
        np.testing.assert_array_equal(path2, alone(p, u2, "fp32").path)
        srv.release(t)
        with pytest.raises(Exception):
            srv.resample(t, u2)
