"""Stream container (mans_container_*): header + decoder table + units in
one buffer, for storage, the wire, and served requests
(MANS_REQ_CONTAINER)."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from ._lib import check, lib

_u32p = ctypes.POINTER(ctypes.c_uint32)


class InfoC(ctypes.Structure):
    _fields_ = [("n_symbols", ctypes.c_uint64), ("n_units", ctypes.c_uint64),
                ("L", ctypes.c_uint32), ("first_state", ctypes.c_uint32),
                ("first_bit", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("table_offset", ctypes.c_uint64), ("units_offset", ctypes.c_uint64)]


@dataclass
class Info:
    n_symbols: int
    n_units: int
    L: int
    first_state: int
    first_bit: int
    table_offset: int
    units_offset: int


def _sig():
    L = lib()
    L.mans_container_size.argtypes = [ctypes.c_uint64, ctypes.c_uint32]
    L.mans_container_size.restype = ctypes.c_size_t
    L.mans_container_write.argtypes = [ctypes.c_void_p, ctypes.c_size_t, _u32p, ctypes.c_uint64,
                                       ctypes.c_uint64, _u32p, ctypes.c_uint32, ctypes.c_uint32,
                                       ctypes.c_uint32, ctypes.POINTER(ctypes.c_size_t)]
    L.mans_container_write.restype = ctypes.c_int
    L.mans_container_parse.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(InfoC)]
    L.mans_container_parse.restype = ctypes.c_int
    return L


def pack(units, n_units: int, n_symbols: int, table, first_state: int, first_bit: int,
         out=None) -> np.ndarray:
    """A container (uint8 array, or written into `out`, e.g. pinned memory)."""
    u = np.ascontiguousarray(units, dtype=np.uint32)
    t = np.ascontiguousarray(table, dtype=np.uint32)
    if not 0 <= n_units <= u.size:
        raise ValueError(f"n_units {n_units} outside the {u.size} units given")
    lb = _sig()
    size = int(lb.mans_container_size(n_units, t.size))
    buf = np.empty(size, dtype=np.uint8) if out is None else out
    written = ctypes.c_size_t(0)
    ptr, cap = _span(buf)
    check(lb.mans_container_write(ptr, cap, u.ctypes.data_as(_u32p), n_units, n_symbols,
                                  t.ctypes.data_as(_u32p), t.size, first_state, first_bit,
                                  ctypes.byref(written)), "mans_container_write")
    return buf


def pack_encoded(st, out=None) -> np.ndarray:
    """A container from a host.Encoded (or oracle) stream."""
    return pack(st.units, st.n_units, st.n, st.table, st.first_state, st.first_bit, out=out)


def _span(buf) -> tuple[int, int]:
    """Address and size in bytes of a contiguous numpy array or host tensor."""
    if isinstance(buf, np.ndarray):
        if not buf.flags.c_contiguous:
            raise ValueError("container buffer must be contiguous")
        return buf.ctypes.data, buf.nbytes
    if not buf.is_contiguous() or buf.is_cuda:
        raise ValueError("container buffer must be a contiguous host tensor")
    return buf.data_ptr(), buf.numel() * buf.element_size()


def parse(buf) -> Info:
    ptr, size = _span(buf)
    info = InfoC()
    check(_sig().mans_container_parse(ptr, size, ctypes.byref(info)), "mans_container_parse")
    return Info(int(info.n_symbols), int(info.n_units), int(info.L), int(info.first_state),
                int(info.first_bit), int(info.table_offset), int(info.units_offset))
