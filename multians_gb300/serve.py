"""Serving loop through the C ABI (mans_server_*): continuous batching of
decode requests with resident tables and device-memory admission.

    srv = Server(budget_bytes=16 << 30)
    tid = srv.add_table(dec_table)              # L uint32 words, stays resident
    srv.submit([request(units, n_units, out, n_out, tid, first_state, first_bit, tag=7)])
    for c in srv.poll(wait_us=1000): ...        # Completion(tag, status, ...)
    srv.close()

`units` / `out` are page-locked host tensors (torch ``pin_memory=True``) or,
with ``device_io=True``, CUDA tensors owned by the caller.  They must stay
alive until the request's completion has been polled.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

from ._lib import MansError, check, lib

REQ_DEVICE_IO = 0x1
REQ_SOURCE_ORDER = 0x2
REQ_CONTAINER = 0x4
REQ_NO_CAPTURE = 0x8
SMALL_OFF = 0xFFFFFFFF   # ServerCfg.small_bytes: no small-request stream


class ServerCfg(ctypes.Structure):
    _fields_ = [("budget_bytes", ctypes.c_uint64), ("max_inflight", ctypes.c_uint32),
                ("max_batch", ctypes.c_uint32), ("small_bytes", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class RequestC(ctypes.Structure):
    _fields_ = [("units", ctypes.c_void_p), ("n_units", ctypes.c_uint64),
                ("out", ctypes.c_void_p), ("n_out", ctypes.c_uint64),
                ("table", ctypes.c_uint32), ("first_state", ctypes.c_uint32),
                ("first_bit", ctypes.c_uint32), ("flags", ctypes.c_uint32),
                ("tag", ctypes.c_uint64), ("arrival_ns", ctypes.c_uint64)]


class CompletionC(ctypes.Structure):
    _fields_ = [("tag", ctypes.c_uint64), ("status", ctypes.c_int32),
                ("dev_status", ctypes.c_uint32), ("arrival_ns", ctypes.c_uint64),
                ("admit_ns", ctypes.c_uint64), ("done_ns", ctypes.c_uint64),
                ("batch", ctypes.c_uint64)]


class StatsC(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "submitted", "completed", "failed", "batches", "kernel_launches", "streams_redone",
        "bytes_in", "bytes_out", "range_bytes", "range_peak", "range_in_use",
        "admission_waits", "largest_batch")]


@dataclass
class Completion:
    tag: int
    status: int
    dev_status: int
    arrival_ns: int
    admit_ns: int
    done_ns: int
    batch: int

    @property
    def latency_ns(self) -> int:
        return self.done_ns - self.arrival_ns


def _sig():
    L = lib()
    vp, u32, u64, sz = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_size_t
    L.mans_server_create.argtypes = [ctypes.POINTER(ServerCfg), ctypes.POINTER(vp)]
    L.mans_server_add_table.argtypes = [vp, ctypes.POINTER(u32), u32, ctypes.POINTER(u32)]
    L.mans_server_submit.argtypes = [vp, ctypes.POINTER(RequestC), sz]
    L.mans_server_poll.argtypes = [vp, ctypes.POINTER(CompletionC), sz, ctypes.POINTER(sz), u32]
    L.mans_server_stats_get.argtypes = [vp, ctypes.POINTER(StatsC)]
    L.mans_server_destroy.argtypes = [vp]
    for f in ("create", "add_table", "submit", "poll", "stats_get", "destroy"):
        getattr(L, "mans_server_" + f).restype = ctypes.c_int
    L.mans_server_now_ns.argtypes = []
    L.mans_server_now_ns.restype = u64
    return L


def now_ns() -> int:
    """The server's clock (CLOCK_MONOTONIC ns), for arrival stamps."""
    return int(_sig().mans_server_now_ns())


def _buf_addr(t, nbytes: int, device_io: bool, what: str) -> int:
    """Address of a request buffer: a raw address is taken as is; a tensor
    must be contiguous, on the side `device_io` names and at least `nbytes`
    long (the worker copies and decodes by address)."""
    if isinstance(t, int):
        return t
    if t.is_cuda != device_io:
        raise ValueError(f"{what}: a {'CUDA' if device_io else 'host'} tensor is needed "
                         f"with device_io={device_io}")
    if not t.is_contiguous():
        raise ValueError(f"{what}: expected a contiguous tensor")
    have = t.numel() * t.element_size()
    if have < nbytes:
        raise ValueError(f"{what}: {have} bytes, the request needs {nbytes}")
    return t.data_ptr()


def request(units, n_units, out, n_out, table, first_state, first_bit, tag=0,
            arrival_ns=0, device_io=False, source_order=False, capture=True) -> RequestC:
    """A request from tensors (or raw addresses)."""
    up = _buf_addr(units, 4 * int(n_units), device_io, "units")
    op = _buf_addr(out, int(n_out), device_io, "out")
    flags = ((REQ_DEVICE_IO if device_io else 0) | (REQ_SOURCE_ORDER if source_order else 0) |
             (0 if capture else REQ_NO_CAPTURE))
    return RequestC(up, int(n_units), op, int(n_out), int(table), int(first_state),
                    int(first_bit), flags, int(tag), int(arrival_ns))


def request_container(container, out, tag=0, arrival_ns=0, source_order=False) -> RequestC:
    """A request whose stream, table and parameters come from a host
    container (multians_gb300.container); `out` holds at least its symbols."""
    nbytes = container.numel() * container.element_size()
    cp = _buf_addr(container, nbytes, False, "container")
    n_out = out.numel() * out.element_size()
    op = _buf_addr(out, n_out, False, "out")
    flags = REQ_CONTAINER | (REQ_SOURCE_ORDER if source_order else 0)
    return RequestC(cp, int(nbytes), op, int(n_out), 0, 0, 0, flags, int(tag), int(arrival_ns))


class Server:
    """mans_server_create's settings: device range (0 = 16 GiB), batches in
    flight (0 = 2), requests per launch (0 = 4096) and the small-request
    threshold in decoded bytes (0 = 1 MiB; SMALL_OFF: no separate slot for
    small requests)."""

    def __init__(self, budget_bytes: int = 0, max_inflight: int = 0, max_batch: int = 0,
                 small_bytes: int = 0):
        self._L = _sig()
        cfg = ServerCfg(int(budget_bytes), int(max_inflight), int(max_batch), int(small_bytes))
        h = ctypes.c_void_p(0)
        check(self._L.mans_server_create(ctypes.byref(cfg), ctypes.byref(h)), "mans_server_create")
        self._h = h
        self._buf = (CompletionC * 4096)()

    def add_table(self, table) -> int:
        import numpy as np
        t = np.ascontiguousarray(table, dtype=np.uint32)
        tid = ctypes.c_uint32(0)
        check(self._L.mans_server_add_table(self._h, t.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                            t.size, ctypes.byref(tid)), "mans_server_add_table")
        return int(tid.value)

    def submit(self, reqs) -> None:
        reqs = list(reqs)
        if not reqs:
            return
        arr = (RequestC * len(reqs))(*reqs)
        check(self._L.mans_server_submit(self._h, arr, len(reqs)), "mans_server_submit")

    def submit_array(self, arr, start: int, count: int) -> None:
        """Submits arr[start:start+count] of a prebuilt (RequestC * n) array
        without building Python objects per request."""
        if count <= 0:
            return
        ptr = ctypes.cast(ctypes.byref(arr, start * ctypes.sizeof(RequestC)),
                          ctypes.POINTER(RequestC))
        check(self._L.mans_server_submit(self._h, ptr, count), "mans_server_submit")

    def poll_raw(self, wait_us: int = 0):
        """Completions as the raw ctypes buffer and a count (valid until the
        next poll)."""
        n = ctypes.c_size_t(0)
        check(self._L.mans_server_poll(self._h, self._buf, len(self._buf), ctypes.byref(n),
                                       int(wait_us)), "mans_server_poll")
        return self._buf, int(n.value)

    def poll(self, wait_us: int = 0) -> list[Completion]:
        n = ctypes.c_size_t(0)
        check(self._L.mans_server_poll(self._h, self._buf, len(self._buf), ctypes.byref(n),
                                       int(wait_us)), "mans_server_poll")
        return [Completion(c.tag, c.status, c.dev_status, c.arrival_ns, c.admit_ns, c.done_ns,
                           c.batch) for c in self._buf[:n.value]]

    def wait(self, count: int, timeout_s: float = 60.0) -> list[Completion]:
        """Polls until `count` completions arrived (raises on timeout)."""
        import time
        out: list[Completion] = []
        t_end = time.monotonic() + timeout_s
        while len(out) < count:
            if time.monotonic() > t_end:
                raise MansError(7, f"server: {len(out)} of {count} completions before timeout")
            out += self.poll(wait_us=2000)
        return out

    def stats(self) -> dict:
        s = StatsC()
        check(self._L.mans_server_stats_get(self._h, ctypes.byref(s)), "mans_server_stats_get")
        return {f: int(getattr(s, f)) for f, _ in StatsC._fields_}

    def close(self) -> None:
        if self._h:
            self._L.mans_server_destroy(self._h)
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
