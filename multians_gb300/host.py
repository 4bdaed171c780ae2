"""Host-side data preparation through the library's C entry points
(mans_host_*): seeded synthetic symbols and the reference's table
generation + tANS encoding, implemented in C++ in the library."""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from ._lib import MansError, lib

TABLE_SEED = 5   # the reference demo's SEED (src/main.cc:24)

_u8p = ctypes.POINTER(ctypes.c_uint8)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_szp = ctypes.POINTER(ctypes.c_size_t)


def _sig():
    L = lib()
    L.mans_host_gen_symbols.argtypes = [ctypes.c_uint64, ctypes.c_double, _u8p, ctypes.c_size_t]
    L.mans_host_gen_symbols.restype = ctypes.c_int
    L.mans_host_max_units.argtypes = [_u8p, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_uint32]
    L.mans_host_max_units.restype = ctypes.c_size_t
    L.mans_host_encode.argtypes = [_u8p, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_uint32, _u32p,
                                   _u32p, ctypes.c_size_t, _szp, _u32p, _u32p]
    L.mans_host_encode.restype = ctypes.c_int
    return L


@dataclass
class Encoded:
    symbols: np.ndarray   # uint8 source symbols
    units: np.ndarray     # uint32, n_units + 4 (CUHDInputBuffer order)
    n_units: int
    first_bit: int
    first_state: int
    table: np.ndarray     # uint32, L decoder words
    L: int

    @property
    def n(self) -> int:
        return int(self.symbols.size)

    @property
    def bits_per_symbol(self) -> float:
        return 32.0 * self.n_units / max(1, self.n)


def gen_symbols(seed: int, lam: float, n: int) -> np.ndarray:
    """n seeded symbols min(255, floor(-ln U / lam)); one zero byte of
    look-ahead padding follows the returned view."""
    buf = np.zeros(n + 1, dtype=np.uint8)
    rc = _sig().mans_host_gen_symbols(seed, lam, buf.ctypes.data_as(_u8p), n)
    if rc:
        raise MansError(rc, "mans_host_gen_symbols")
    return buf[:n]


def encode(symbols: np.ndarray, L: int, table_seed: int = TABLE_SEED) -> Encoded:
    sym = np.zeros(symbols.size + 8, dtype=np.uint8)
    sym[: symbols.size] = symbols
    L_ = _sig()
    cap = int(L_.mans_host_max_units(sym.ctypes.data_as(_u8p), symbols.size, L, table_seed))
    units = np.zeros(max(cap, 8), dtype=np.uint32)
    table = np.zeros(L, dtype=np.uint32)
    nu = ctypes.c_size_t(0)
    fb = ctypes.c_uint32(0)
    fs = ctypes.c_uint32(0)
    rc = L_.mans_host_encode(sym.ctypes.data_as(_u8p), symbols.size, L, table_seed,
                             table.ctypes.data_as(_u32p), units.ctypes.data_as(_u32p), units.size,
                             ctypes.byref(nu), ctypes.byref(fb), ctypes.byref(fs))
    if rc:
        raise MansError(rc, "mans_host_encode")
    n_units = int(nu.value)
    return Encoded(np.ascontiguousarray(symbols, dtype=np.uint8), units[: n_units + 4].copy(),
                   n_units, int(fb.value), int(fs.value), table, L)


def make_stream(seed: int, lam: float, n: int, L: int) -> Encoded:
    return encode(gen_symbols(seed, lam, n), L)
