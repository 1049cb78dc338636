"""Serving loop: continuous batching of sort requests (C ABI ``rsbd8g_server_*``).

``Server(budget_bytes, max_inflight)`` owns a device-memory budget and a dispatcher thread in the
library; ``submit`` queues a request (device input/output tensors) and returns its id at once;
``wait`` / ``drain`` block; ``info`` gives per-request times (submit, launch, device done) from
which latency percentiles are computed; ``stats`` the counters (batches, most requests coalesced
into one launch, most batches in flight at once).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import api


class RequestInfo(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("reserved", ctypes.c_uint32), ("count", ctypes.c_uint64),
                ("submit_s", ctypes.c_double), ("start_s", ctypes.c_double), ("done_s", ctypes.c_double)]


class ServerCounters(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("submitted", "completed", "keys_completed", "batches",
                                               "max_coalesced", "max_inflight_batches", "pending",
                                               "arena_used", "budget")]


def _lib():
    L = api.lib()
    if not getattr(L, "_srv_sigs", False):
        VP, S = ctypes.c_void_p, ctypes.c_size_t
        L.rsbd8g_server_create.argtypes = [S, ctypes.c_uint32, ctypes.POINTER(VP)]
        L.rsbd8g_server_submit.argtypes = [VP, ctypes.POINTER(api.Desc), S, VP, VP, ctypes.POINTER(ctypes.c_uint64)]
        L.rsbd8g_server_wait.argtypes = [VP, ctypes.c_uint64, ctypes.c_double, ctypes.POINTER(RequestInfo)]
        L.rsbd8g_server_drain.argtypes = [VP, ctypes.c_double]
        L.rsbd8g_server_stats.argtypes = [VP, ctypes.POINTER(ServerCounters)]
        L.rsbd8g_server_destroy.argtypes = [VP]
        for f in ("rsbd8g_server_create", "rsbd8g_server_submit", "rsbd8g_server_wait", "rsbd8g_server_drain",
                  "rsbd8g_server_stats", "rsbd8g_server_destroy"):
            getattr(L, f).restype = ctypes.c_int
        L._srv_sigs = True
    return L


class Server:
    def __init__(self, budget_bytes: int, max_inflight: int = 4):
        self._h = ctypes.c_void_p()
        api._check(_lib().rsbd8g_server_create(budget_bytes, max_inflight, ctypes.byref(self._h)),
                   "rsbd8g_server_create")
        self._keep = {}   # request id -> tensors kept alive until the request is done

    def submit(self, input, output, direction="ascfwdorder", mode="native", key_dtype=None) -> int:
        """Queue one sort of `input` into `output`.  The server's streams are not ordered after the
        caller's, so work still queued on the current stream (which may write the input, or have
        used the arrays' memory before) is waited for on the host first."""
        import torch
        if hasattr(input, "device"):
            cur = torch.cuda.current_stream(input.device)
            if not cur.query():
                cur.synchronize()
        d = api.make_desc(key_dtype if key_dtype is not None else input.dtype, direction, mode)
        rid = ctypes.c_uint64()
        api._check(_lib().rsbd8g_server_submit(self._h, ctypes.byref(d), api._count(input, None, d), api._ptr(input),
                                               api._ptr(output), ctypes.byref(rid)), "rsbd8g_server_submit")
        self._keep[rid.value] = (input, output)
        return rid.value

    def wait(self, rid: int, timeout_s: float = 60.0) -> RequestInfo:
        info = RequestInfo()
        st = _lib().rsbd8g_server_wait(self._h, rid, timeout_s, ctypes.byref(info))
        if st != api.ERR_TIMEOUT:
            self._keep.pop(rid, None)
        api._check(st, f"request {rid}")
        return info

    def info(self, rid: int) -> RequestInfo:
        return self.wait(rid, 0.0)

    def drain(self, timeout_s: float = 600.0) -> None:
        api._check(_lib().rsbd8g_server_drain(self._h, timeout_s), "rsbd8g_server_drain")

    def stats(self) -> dict:
        c = ServerCounters()
        api._check(_lib().rsbd8g_server_stats(self._h, ctypes.byref(c)), "rsbd8g_server_stats")
        return {n: getattr(c, n) for n, _ in ServerCounters._fields_}

    def close(self) -> None:
        if self._h:
            _lib().rsbd8g_server_destroy(self._h)
            self._h = ctypes.c_void_p()
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def latency_summary(infos) -> dict:
    """p50 / p99 / max of (device done - submit) over completed requests, in milliseconds."""
    lat = np.array([(i.done_s - i.submit_s) * 1e3 for i in infos])
    if lat.size == 0:
        return {"p50_ms": None, "p99_ms": None, "max_ms": None}
    return {"p50_ms": round(float(np.percentile(lat, 50)), 3), "p99_ms": round(float(np.percentile(lat, 99)), 3),
            "max_ms": round(float(lat.max()), 3), "requests": int(lat.size)}
