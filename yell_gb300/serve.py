"""Python handle on the library's serving loop (yell_server_* in
include/yell_gb300.h): continuous batching of polymul requests of mixed
size with HBM-budget admission and latency statistics."""
from __future__ import annotations

import ctypes
import threading

import numpy as np

from . import _capi
from ._capi import call, load

YELL_REQ_HOST, YELL_REQ_DEVICE, YELL_REQ_DISCARD_OUTPUT = 0, 1, 2
YELL_REQ_NTT_FORWARD, YELL_REQ_NTT_BACKWARD = 4, 8
_OPS = {"polymul": 0, "forward": YELL_REQ_NTT_FORWARD, "backward": YELL_REQ_NTT_BACKWARD}


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_inflight", ctypes.c_uint32),
                ("max_batch", ctypes.c_uint32), ("inject_alloc_failures", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class Request(ctypes.Structure):
    _fields_ = [("a", ctypes.c_void_p), ("b", ctypes.c_void_p), ("c", ctypes.c_void_p),
                ("log_n", ctypes.c_uint32), ("L", ctypes.c_uint32), ("cm0", ctypes.c_uint32),
                ("flags", ctypes.c_uint32)]


class RequestResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("queue_us", ctypes.c_double),
                ("latency_us", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in ("submitted", "completed", "rejected", "cancelled",
                                                "failed", "batches", "queued", "hbm_budget",
                                                "hbm_in_use", "hbm_peak")] + \
               [(n, ctypes.c_double) for n in ("p50_us", "p99_us", "mean_us", "max_us", "limb_ntts",
                                                "limb_ntts_per_s", "requests_per_s", "window_s")]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


_SIGS = {
    "yell_server_create": (ctypes.c_int, [ctypes.POINTER(ServerConfig), ctypes.POINTER(ctypes.c_void_p)]),
    "yell_server_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "yell_server_submit": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Request),
                                          ctypes.POINTER(ctypes.c_uint64)]),
    "yell_server_wait": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double,
                                        ctypes.POINTER(RequestResult)]),
    "yell_server_cancel": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
    "yell_server_pause": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "yell_server_get_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(Stats)]),
    "yell_server_load_test": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Request), ctypes.c_uint32,
                                             ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                             ctypes.POINTER(Stats)]),
}
_bound = False


def _bind():
    global _bound
    if not _bound:
        lib = load()
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _bound = True
    return load()


def _addr(x) -> int:
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    return x.data_ptr()  # torch tensor


class Server:
    """Continuous-batching polymul server on the current CUDA device."""

    def __init__(self, hbm_budget_bytes: int = 0, max_inflight: int = 4, max_batch: int = 1024,
                 inject_alloc_failures: int = 0):
        lib = _bind()
        cfg = ServerConfig(hbm_budget_bytes, max_inflight, max_batch, inject_alloc_failures, 0)
        h = ctypes.c_void_p()
        _capi.check(lib.yell_server_create(ctypes.byref(cfg), ctypes.byref(h)), "yell_server_create")
        self._h = h
        self._keep = {}
        self._lock = threading.Lock()

    def submit(self, a, b, c, log_n: int, L: int, cm0: int = 0, device: bool = False,
               op: str = "polymul") -> int:
        """a, b, c: (L, N) uint64 numpy arrays (host) or 64-bit CUDA tensors (device=True).
        op: "polymul" (c = a * b), "forward" or "backward" (c = NTT of a; b unused, may be None).
        Host buffers must stay alive until wait() returns; the handle keeps them."""
        flags = (YELL_REQ_DEVICE if device else YELL_REQ_HOST) | _OPS[op]
        req = Request(_addr(a), _addr(b) if b is not None else None, _addr(c), log_n, L, cm0, flags)
        rid = ctypes.c_uint64()
        _capi.check(load().yell_server_submit(self._h, ctypes.byref(req), ctypes.byref(rid)),
                    "yell_server_submit")
        with self._lock:
            self._keep[rid.value] = (a, b, c)
        return rid.value

    def _submit_flags(self, a, b, c, log_n: int, L: int, cm0: int, flags: int) -> int:
        """Submission with raw request flags (tests of the validation)."""
        req = Request(_addr(a), _addr(b) if b is not None else None, _addr(c), log_n, L, cm0, flags)
        rid = ctypes.c_uint64()
        _capi.check(load().yell_server_submit(self._h, ctypes.byref(req), ctypes.byref(rid)),
                    "yell_server_submit")
        return rid.value

    def wait(self, rid: int, timeout: float = 30.0) -> dict:
        res = RequestResult()
        st = load().yell_server_wait(self._h, rid, timeout, ctypes.byref(res))
        if st != _capi.YELL_ERR_TIMEOUT:
            with self._lock:
                self._keep.pop(rid, None)
        _capi.check(st, "yell_server_wait")
        return {"status": res.status, "queue_us": res.queue_us, "latency_us": res.latency_us}

    def cancel(self, rid: int) -> None:
        call("yell_server_cancel", self._h, rid)

    def pause(self, paused: bool = True) -> None:
        call("yell_server_pause", self._h, 1 if paused else 0)

    def stats(self, reset: bool = False) -> dict:
        s = Stats()
        call("yell_server_get_stats", self._h, 1 if reset else 0, ctypes.byref(s))
        return s.as_dict()

    def load_test(self, templates, offered_rps: float, duration_s: float, seed: int = 5) -> dict:
        """templates: list of (a, b, log_n, L, cm0) with device-resident CUDA tensors."""
        arr = (Request * len(templates))()
        for i, (a, b, log_n, L, cm0) in enumerate(templates):
            arr[i] = Request(_addr(a), _addr(b), None, log_n, L, cm0,
                             YELL_REQ_DEVICE | YELL_REQ_DISCARD_OUTPUT)
        s = Stats()
        call("yell_server_load_test", self._h, arr, len(templates), offered_rps, duration_s, seed,
             ctypes.byref(s))
        return s.as_dict()

    def close(self) -> None:
        if self._h:
            call("yell_server_destroy", self._h)
            self._h = None
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
