"""ctypes loader of libmultians_gb300.so and the C ABI signatures
(include/multians_gb300.h)."""
from __future__ import annotations

import ctypes
import enum
import os

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libmultians_gb300.so")

DEV_BAD_TABLE = 0x1
DEV_SYNC_OVERFLOW = 0x2
DEV_DEGENERATE = 0x4
DEV_COUNT_MISMATCH = 0x8
DEV_SCAN_TIMEOUT = 0x10


class Status(enum.IntEnum):
    OK = 0
    ERR_ARG = 1
    ERR_CUDA = 2
    ERR_AUX_SMALL = 3
    ERR_TABLE = 4
    ERR_SYNC = 5
    ERR_NOMEM = 6
    ERR_BUSY = 7
    ERR_NOT_FOUND = 8


class MansError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        try:
            name = Status(code).name
        except ValueError:
            name = f"status {code}"
        super().__init__(f"{what}: {name}" if what else name)
        self.code = code


DECODE_SOURCE_ORDER = 0x1
DECODE_NO_CAPTURE = 0x2
DECODE_CAPTURE = 0x4
DECODE_START_OFFSET = 0x10
DECODE_SEEDS = 0x20
DECODE_NO_SEEDS = 0x40
PLAN_MODEL = 0x8


class TuneEntry(ctypes.Structure):
    _fields_ = [("L", ctypes.c_uint32), ("bits_per_symbol", ctypes.c_float),
                ("large", ctypes.c_uint32), ("block_units", ctypes.c_uint32),
                ("meet_mult", ctypes.c_float), ("capture", ctypes.c_uint32),
                ("gbps", ctypes.c_float), ("model_gbps", ctypes.c_float)]

    def as_dict(self):
        return {f: (round(float(getattr(self, f)), 4) if t is ctypes.c_float
                    else int(getattr(self, f))) for f, t in self._fields_}


class SyncStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "regions", "blocks", "walks", "open_walks", "walk_units", "walk_max_units",
        "walk_blocks", "metadata_bytes", "fallback_warps")] + [
        ("unmerged", ctypes.c_uint32), ("seeded_walks", ctypes.c_uint32)]


class Cfg(ctypes.Structure):
    _fields_ = [("block_units", ctypes.c_uint32), ("region_blocks", ctypes.c_uint32),
                ("walk_slots", ctypes.c_uint32), ("threads", ctypes.c_uint32),
                ("flags", ctypes.c_uint32), ("capture_bytes", ctypes.c_uint32)]

    def as_dict(self):
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


_vp = ctypes.c_void_p
_sz = ctypes.c_size_t
_u32 = ctypes.c_uint32
_u32p = ctypes.POINTER(ctypes.c_uint32)

# (name, restype, argtypes) of every exported entry point
SIGNATURES = {
    "mans_version": (ctypes.c_char_p, []),
    "mans_last_launch_count": (_u32, []),
    "mans_plan": (ctypes.c_int, [_sz, _sz, _u32, ctypes.POINTER(Cfg), ctypes.POINTER(Cfg)]),
    "mans_aux_size": (_sz, [_sz, ctypes.POINTER(Cfg)]),
    "mans_aux_size_max": (_sz, [_sz]),
    "mans_aux_size_max_any": (_sz, [_sz]),
    "mans_plan_tuned": (ctypes.c_int, [_sz, _sz, _u32, _u32, ctypes.c_double, ctypes.c_int,
                                       ctypes.POINTER(Cfg)]),
    "mans_tune_lookup": (ctypes.c_int, [_u32, ctypes.c_double, ctypes.c_uint64,
                                        ctypes.POINTER(TuneEntry)]),
    "mans_table_check": (ctypes.c_int, [_u32p, _u32]),
    "mans_decode": (ctypes.c_int, [_vp, _sz, _vp, _sz, _vp, _u32, _u32, _u32, _vp, _sz,
                                   ctypes.POINTER(Cfg), _vp]),
    "mans_aux_status": (ctypes.c_int, [_vp, _vp, _u32p]),
    "mans_timing_enable": (ctypes.c_int, [ctypes.c_int]),
    "mans_timing_collect": (ctypes.c_int, [ctypes.POINTER(ctypes.c_float), ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_int)]),
    "mans_decode_sync": (ctypes.c_int, [_vp, _sz, _vp, _sz, _vp, _u32, _u32, _u32, _vp, _sz,
                                        ctypes.POINTER(Cfg), _vp, _u32p]),
    "mans_aux_alloc": (ctypes.c_int, [_sz, _sz, _u32, ctypes.POINTER(Cfg),
                                      ctypes.POINTER(_vp), ctypes.POINTER(_sz)]),
    "mans_aux_free": (ctypes.c_int, [_vp]),
    "mans_table_upload": (ctypes.c_int, [_u32p, _u32, ctypes.POINTER(_vp)]),
    "mans_table_free": (ctypes.c_int, [_vp]),
    "mans_sync_stats_get": (ctypes.c_int, [_vp, _sz, _sz, _sz, _u32, ctypes.POINTER(Cfg), _vp,
                                           ctypes.POINTER(SyncStats)]),
}

_lib = None


def lib():
    """The loaded native library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int, what: str = "") -> None:
    if rc != 0:
        raise MansError(rc, what)


def version() -> str:
    return lib().mans_version().decode()


def plan(n_units: int, n_out: int, L: int, hint: dict | None = None) -> dict:
    h = Cfg(**(hint or {}))
    out = Cfg()
    check(lib().mans_plan(n_units, n_out, L, ctypes.byref(h), ctypes.byref(out)), "mans_plan")
    return out.as_dict()


def plan_tuned(n_units: int, n_out: int, L: int, block_units: int, meet_mult: float,
               capture: bool) -> dict:
    """The plan mans_plan makes from a measured table entry with these values."""
    out = Cfg()
    check(lib().mans_plan_tuned(n_units, n_out, L, block_units, meet_mult, int(capture),
                                ctypes.byref(out)), "mans_plan_tuned")
    return out.as_dict()


def tune_lookup(L: int, bits_per_symbol: float, n_out: int):
    """The measured table entry mans_plan uses (dict), or None."""
    e = TuneEntry()
    rc = lib().mans_tune_lookup(L, bits_per_symbol, n_out, ctypes.byref(e))
    if rc < 0 or rc > 1:
        raise MansError(rc, "mans_tune_lookup")
    return e.as_dict() if rc == 1 else None


def aux_size(n_units: int, cfg: dict) -> int:
    c = Cfg(**cfg)
    return int(lib().mans_aux_size(n_units, ctypes.byref(c)))


def aux_size_max(n_units: int) -> int:
    return int(lib().mans_aux_size_max(n_units))


def aux_size_max_any(n_units: int) -> int:
    """Aux bytes every plan of n_units units fits, symbol capture included."""
    return int(lib().mans_aux_size_max_any(n_units))


def table_check(table) -> int:
    """0 = decodable, 1 = single-symbol table, -1 = invalid (host check)."""
    import numpy as np
    t = np.ascontiguousarray(table, dtype=np.uint32)
    return int(lib().mans_table_check(t.ctypes.data_as(_u32p), t.size))


def sync_stats(d_aux: int, aux_bytes: int, n_units: int, n_out: int, L: int,
               cfg: dict | None = None, stream: int | None = None) -> dict:
    """What the synchronisation of the last decode in the workspace at
    d_aux cost (mans_sync_stats_get): merge-walk units decoded a second
    time, the longest walk, walks left to the walk pass, metadata bytes.
    Pass the decode's own arguments; waits for `stream`."""
    c = Cfg(**cfg) if cfg else None
    out = SyncStats()
    check(lib().mans_sync_stats_get(d_aux, aux_bytes, n_units, n_out, L,
                                    ctypes.byref(c) if c is not None else None, stream,
                                    ctypes.byref(out)), "mans_sync_stats_get")
    return {f: int(getattr(out, f)) for f, _ in SyncStats._fields_}


KERNELS = ("k_prep", "k_gwalk", "k_wwalk", "k_scan", "k_final")


def timing_enable(max_decodes: int) -> None:
    check(lib().mans_timing_enable(int(max_decodes)), "mans_timing_enable")


def timing_collect() -> tuple[dict, int]:
    """Summed milliseconds per kernel over the decodes timed since
    timing_enable, and the number of decodes (k_wwalk: its three passes)."""
    buf = (ctypes.c_float * len(KERNELS))()
    n = ctypes.c_int(0)
    check(lib().mans_timing_collect(buf, len(KERNELS), ctypes.byref(n)), "mans_timing_collect")
    return {k: float(buf[i]) for i, k in enumerate(KERNELS)}, int(n.value)
