"""Batched decode of many independent streams through the C ABI
(mans_batch_*): one launch of each kernel covers the whole batch, optionally
replayed as a CUDA graph."""
from __future__ import annotations

import ctypes

from ._lib import Cfg, check, lib


class StreamDesc(ctypes.Structure):
    _fields_ = [("d_units", ctypes.c_void_p), ("n_units", ctypes.c_uint64),
                ("d_out", ctypes.c_void_p), ("n_out", ctypes.c_uint64),
                ("d_table", ctypes.c_void_p), ("L", ctypes.c_uint32),
                ("first_state", ctypes.c_uint32), ("first_bit", ctypes.c_uint32),
                ("flags", ctypes.c_uint32)]


def _sig():
    L = lib()
    vp, u32 = ctypes.c_void_p, ctypes.c_uint32
    L.mans_batch_workspace_size.argtypes = [ctypes.POINTER(StreamDesc), u32, ctypes.POINTER(Cfg),
                                            ctypes.POINTER(ctypes.c_size_t)]
    L.mans_batch_workspace_size.restype = ctypes.c_int
    L.mans_batch_create.argtypes = [ctypes.POINTER(StreamDesc), u32, ctypes.POINTER(Cfg), vp,
                                    ctypes.c_size_t, ctypes.POINTER(vp)]
    L.mans_batch_create.restype = ctypes.c_int
    L.mans_batch_decode.argtypes = [vp, vp]
    L.mans_batch_decode.restype = ctypes.c_int
    L.mans_batch_graph_decode.argtypes = [vp, vp]
    L.mans_batch_graph_decode.restype = ctypes.c_int
    L.mans_batch_status.argtypes = [vp, vp, ctypes.POINTER(u32), ctypes.POINTER(u32)]
    L.mans_batch_status.restype = ctypes.c_int
    L.mans_batch_fixup.argtypes = [vp, vp, ctypes.POINTER(u32)]
    L.mans_batch_fixup.restype = ctypes.c_int
    L.mans_decode_batch.argtypes = [ctypes.POINTER(StreamDesc), u32, ctypes.POINTER(Cfg), vp,
                                    ctypes.c_size_t, vp, ctypes.POINTER(u32), ctypes.POINTER(u32)]
    L.mans_decode_batch.restype = ctypes.c_int
    L.mans_batch_destroy.argtypes = [vp]
    L.mans_batch_destroy.restype = ctypes.c_int
    L.mans_decode_loop.argtypes = [ctypes.POINTER(StreamDesc), u32, ctypes.POINTER(Cfg),
                                   ctypes.POINTER(vp), ctypes.POINTER(ctypes.c_size_t), vp,
                                   ctypes.POINTER(vp)]
    L.mans_decode_loop.restype = ctypes.c_int
    return L


def _addr(t, nbytes: int, what: str):
    """Device address of a CUDA tensor of at least `nbytes` bytes (None
    passes through: descriptors used only for sizing carry no buffers)."""
    if t is None:
        return None
    from .decoder import _dev_ptr
    return _dev_ptr(t, nbytes, what).value


def desc(units, n_units, out, n_out, table, L, first_state, first_bit,
         source_order: bool = False, capture: bool = True) -> StreamDesc:
    """A stream descriptor from CUDA tensors (units/table int32 or uint32
    views); ``source_order`` writes the output in source order, ``capture``
    False keeps the stream out of symbol capture.  Tensors shorter than the
    sizes given are refused (the batch kernels see only addresses)."""
    from ._lib import DECODE_NO_CAPTURE, DECODE_SOURCE_ORDER
    flags = (DECODE_SOURCE_ORDER if source_order else 0) | (0 if capture else DECODE_NO_CAPTURE)
    return StreamDesc(_addr(units, 4 * int(n_units), "units"), int(n_units),
                      _addr(out, int(n_out), "out"), int(n_out),
                      _addr(table, 4 * int(L), "table"), int(L),
                      int(first_state), int(first_bit), flags)


class Batch:
    """A planned batch; decode() enqueues it, graph_decode() replays it as a
    CUDA graph, status() returns (or-status, per-stream statuses)."""

    def __init__(self, descs, hint: dict | None = None, workspace=None):
        self._L = _sig()
        self.n = len(descs)
        arr = (StreamDesc * self.n)(*descs)
        self._descs = arr
        h = Cfg(**hint) if hint else None
        handle = ctypes.c_void_p(0)
        ws_ptr = ctypes.c_void_p(workspace.data_ptr()) if workspace is not None else None
        ws_bytes = workspace.numel() if workspace is not None else 0
        check(self._L.mans_batch_create(arr, self.n, ctypes.byref(h) if h else None, ws_ptr,
                                        ws_bytes, ctypes.byref(handle)), "mans_batch_create")
        self.handle = handle

    @staticmethod
    def workspace_size(descs, hint: dict | None = None) -> int:
        L = _sig()
        arr = (StreamDesc * len(descs))(*descs)
        h = Cfg(**hint) if hint else None
        out = ctypes.c_size_t(0)
        check(L.mans_batch_workspace_size(arr, len(descs), ctypes.byref(h) if h else None,
                                          ctypes.byref(out)), "mans_batch_workspace_size")
        return int(out.value)

    def decode(self, stream) -> None:
        check(self._L.mans_batch_decode(self.handle, ctypes.c_void_p(stream.cuda_stream)),
              "mans_batch_decode")

    def graph_decode(self, stream) -> None:
        check(self._L.mans_batch_graph_decode(self.handle, ctypes.c_void_p(stream.cuda_stream)),
              "mans_batch_graph_decode")

    def status(self, stream):
        acc = ctypes.c_uint32(0)
        per = (ctypes.c_uint32 * self.n)()
        check(self._L.mans_batch_status(self.handle, ctypes.c_void_p(stream.cuda_stream),
                                        ctypes.byref(acc), per), "mans_batch_status")
        return int(acc.value), [int(x) for x in per]

    def fixup(self, stream) -> int:
        """Re-decodes the streams whose sync walks overflowed; returns how many."""
        n = ctypes.c_uint32(0)
        check(self._L.mans_batch_fixup(self.handle, ctypes.c_void_p(stream.cuda_stream),
                                       ctypes.byref(n)), "mans_batch_fixup")
        return int(n.value)

    def close(self) -> None:
        if self.handle:
            self._L.mans_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def decode_batch(descs, hint: dict | None = None, workspace=None, stream=None):
    """One synchronous call for a batch (mans_decode_batch): returns the OR
    of the device status bits and each stream's."""
    L = _sig()
    n = len(descs)
    arr = (StreamDesc * n)(*descs)
    h = Cfg(**hint) if hint else None
    acc = ctypes.c_uint32(0)
    per = (ctypes.c_uint32 * n)()
    ws_ptr = ctypes.c_void_p(workspace.data_ptr()) if workspace is not None else None
    ws_bytes = workspace.numel() if workspace is not None else 0
    st = ctypes.c_void_p(stream.cuda_stream) if stream is not None else None
    check(L.mans_decode_batch(arr, n, ctypes.byref(h) if h else None, ws_ptr, ws_bytes, st,
                              ctypes.byref(acc), per), "mans_decode_batch")
    return int(acc.value), [int(x) for x in per]


class Loop:
    """A loop of plain decodes over many streams, launched from C
    (mans_decode_loop): each stream with its cached plan and its own
    workspace, one after another on one CUDA stream."""

    def __init__(self, descs, plans, auxes):
        from .decoder import _dev_ptr
        self._L = _sig()
        self.n = len(descs)
        self._descs = (StreamDesc * self.n)(*descs)
        self._plans = (Cfg * self.n)(*[Cfg(**p) for p in plans])
        self._aux = (ctypes.c_void_p * self.n)(*[_dev_ptr(a).value for a in auxes])
        self._bytes = (ctypes.c_size_t * self.n)(*[a.numel() for a in auxes])
        self._keep = auxes

    def run(self, stream, events=None) -> int:
        """Enqueues the loop; ``events`` (torch.cuda.Event, one per stream,
        already created) are recorded after each stream's decode.  Returns
        the number of kernels launched."""
        ev = None
        if events is not None:
            ev = (ctypes.c_void_p * self.n)(*[e.cuda_event for e in events])
        check(self._L.mans_decode_loop(self._descs, self.n, self._plans, self._aux, self._bytes,
                                       ctypes.c_void_p(stream.cuda_stream), ev),
              "mans_decode_loop")
        return int(lib().mans_last_launch_count())
