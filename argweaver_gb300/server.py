"""Serving loop over the C ABI (awg_server_*): continuous batching of threading requests.

    srv = Server(device_bytes=16 << 30, max_inflight=4, max_batch=32)
    t = srv.submit(problem, precision="fp32", uniforms=u)      # from any thread
    r = srv.wait(t)                                            # Result: path, loglik, ...
    srv.stats()                                                # p50 / p99 latency, cells/s

Requests queue FIFO; a worker thread in the library forms batches from the queue head as
device memory and batch slots free up and keeps several on the GPU at once, so requests
that arrive while others run overlap with them. A resident request keeps its forward table
on the device for new path draws (resample) until released.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from . import capi
from .api import GpuError, Result, _Bound
from .problem import Problem


@dataclass
class Ticket:
    id: int
    result: Result
    loglik: np.ndarray = field(repr=False)


class Server:
    def __init__(self, device_bytes: int = 8 << 30, max_inflight: int = 4, max_batch: int = 32,
                 length_ratio: float = 2.0):
        self._lib = capi.load()
        opt = capi.AwgServerOptions(int(device_bytes), int(max_inflight), int(max_batch),
                                    float(length_ratio))
        self._h = self._lib.awg_server_create(C.byref(opt))
        if not self._h:
            raise GpuError(self._err())

    def _err(self) -> str:
        msg = self._lib.awg_server_last_error()
        return msg.decode() if msg else ""

    def submit(self, prob: Problem, *, precision: str = "fp32", want_path: bool = True,
               want_forward: bool = False, want_posterior: bool = False,
               uniforms: Optional[np.ndarray] = None, resident: bool = False) -> Ticket:
        """Queue one problem; the result arrays are filled in place when it completes."""
        fp32 = precision == "fp32"
        b = _Bound(prob)
        ncell = self._lib.awg_problem_cells(C.byref(b.c))
        if ncell < 0:
            raise ValueError(capi.last_error())
        r = Result()
        out = capi.AwgOutputs()
        if want_forward:
            r.forward = np.empty(ncell, dtype=np.float32 if fp32 else np.float64)
            if fp32:
                out.forward32 = r.forward.ctypes.data
            else:
                out.forward = r.forward.ctypes.data
        if want_posterior:
            r.posterior = np.empty(ncell, dtype=np.float64)
            out.posterior = r.posterior.ctypes.data
        if want_path:
            r.path = np.empty(b.p.seqlen, dtype=np.int32)
            out.path = r.path.ctypes.data
        u = None
        if uniforms is not None:
            u = np.ascontiguousarray(uniforms, dtype=np.float64)
            if u.shape[0] != b.p.seqlen:
                raise ValueError("uniforms must have one entry per column")
            out.uniforms = u.ctypes.data  # copied by the server
        ll = np.full(1, np.nan)
        out.loglik = ll.ctypes.data
        rid = self._lib.awg_server_submit(self._h, C.byref(b.c), C.byref(out),
                                          capi.AWG_FP32 if fp32 else capi.AWG_FP64, int(resident))
        if rid < 0:
            raise GpuError(self._err())
        return Ticket(int(rid), r, ll)

    def wait(self, t: Ticket, timeout: Optional[float] = None) -> Optional[Result]:
        """The request's Result once done (None if still pending after timeout seconds)."""
        ms = -1 if timeout is None else int(1e3 * timeout)
        rc = self._lib.awg_server_wait(self._h, t.id, ms)
        if rc < 0:
            raise GpuError(f"request {t.id} failed ({rc}): {self._err()}")
        if rc == 0:
            return None
        t.result.loglik = float(t.loglik[0])
        return t.result

    def times(self, t: Ticket) -> tuple:
        """(submitted, admitted to a batch, completed), seconds on a steady clock."""
        out = np.zeros(3)
        self._lib.awg_server_request_times(self._h, t.id, out.ctypes.data_as(capi.c_double_p))
        return tuple(float(x) for x in out)

    def forget(self, t: Ticket) -> None:
        self._lib.awg_server_forget(self._h, t.id)

    def resample(self, t: Ticket, uniforms: Optional[np.ndarray] = None) -> np.ndarray:
        """A new path of a completed resident request (traceback only)."""
        path = np.empty_like(t.result.path)
        u = None if uniforms is None else np.ascontiguousarray(uniforms, dtype=np.float64)
        rc = self._lib.awg_server_resample(self._h, t.id, None if u is None else u.ctypes.data,
                                           path.ctypes.data)
        if rc != 0:
            raise GpuError(self._err())
        return path

    def release(self, t: Ticket) -> None:
        if self._lib.awg_server_release(self._h, t.id) != 0:
            raise GpuError("release: not a completed resident request")

    def stats(self) -> dict:
        st = capi.AwgServerStats()
        self._lib.awg_server_stats_get(self._h, C.byref(st))
        return {k: getattr(st, k) for k, _ in st._fields_}

    def close(self) -> None:
        if self._h:
            self._lib.awg_server_destroy(self._h)
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
