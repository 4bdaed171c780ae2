"""ctypes bindings of the C oracle (``liboracle.so``) and of the reference's
own host code (``_ref/libmans_ref.so``, present only where the reference
sources were available to build it).  Test infrastructure only.

Streams are numpy ``uint32`` arrays in CUHDInputBuffer order (encoder units
reversed, multians_input_buffer.cc:29) followed by 4 zero padding units;
decoder tables are ``uint32`` arrays of packed CUHDCodetableItem words
(next_state | symbol << 16 | bits << 24, cuhd_codetable.h:20-24).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libmans_ref.so")

TABLE_SEED = 5  # the demo's SEED (src/main.cc:24) fed to the table generator

_u8p = ctypes.POINTER(ctypes.c_uint8)
_u32p = ctypes.POINTER(ctypes.c_uint32)
_sz = ctypes.c_size_t
_u32 = ctypes.c_uint32


def build(ref: bool | None = None) -> None:
    """Compiles liboracle.so, and libmans_ref.so when the reference sources
    are present (or when ``ref`` is True).  Where the reference tree is read
    from is the recipe's business (oracle/Makefile: MANS_REF_ROOT from the
    environment, else its own default)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    if ref is None:
        subprocess.run(["make", "-s", "-C", HERE, "ref-auto"], check=True)
    elif ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def _ptr(a: np.ndarray, t):
    return a.ctypes.data_as(t)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(ref=False)
        L = ctypes.CDLL(LIB_PATH)
        L.mo_gen_symbols.argtypes = [ctypes.c_uint64, ctypes.c_double, _u8p, _sz]
        L.mo_gen_symbols.restype = None
        L.mo_build_tables.argtypes = [_u8p, _sz, _u32, _u32, _u32p, _u32p, _u32p]
        L.mo_build_tables.restype = ctypes.c_int
        L.mo_max_units.argtypes = [_u32, _sz]
        L.mo_max_units.restype = _sz
        L.mo_encode.argtypes = [_u32p, _u32, _u32, _u8p, _sz, _u32p, _sz, _u32p, _u32p]
        L.mo_encode.restype = _sz
        L.mo_decode_seq.argtypes = [_u32p, _sz, _u32, _u32, _u32p, _u32, _u8p, _sz]
        L.mo_decode_seq.restype = ctypes.c_int
        L.mo_sync_points.argtypes = [_sz, _u32p, _sz, _u32, _u32, _u32p, _u32, _u32p]
        L.mo_sync_points.restype = ctypes.c_int
        L.mo_multicore_decode.argtypes = [_sz, _sz, _u32p, _sz, _u32, _u32, _u32p, _u32, _u8p, _sz]
        _pp = ctypes.POINTER(_u32p)
        _szp = ctypes.POINTER(_sz)
        L.mo_encode_segments.argtypes = [_pp, _szp, _sz, _u32, _u32, _u8p, _sz, _u32p, _sz,
                                         _u32p, _u32p]
        L.mo_encode_segments.restype = _sz
        L.mo_decode_segments.argtypes = [_u32p, _sz, _u32, _u32, _pp, _szp, _sz, _u32, _u8p,
                                         ctypes.POINTER(ctypes.c_uint64)]
        L.mo_decode_segments.restype = ctypes.c_int
        L.mo_multicore_decode.restype = ctypes.c_int
        L.mo_reverse_bytes.argtypes = [_u8p, _sz]
        L.mo_reverse_bytes.restype = None
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_LIB_PATH)


def ref():
    """The reference's own host code behind oracle/ref_shim.cc."""
    global _ref
    if _ref is None:
        R = ctypes.CDLL(REF_LIB_PATH)
        R.mref_decoder_table.argtypes = [_u8p, _sz, _u32, _u32, _u32p]
        R.mref_decoder_table.restype = ctypes.c_int
        R.mref_max_units.argtypes = [_u8p, _sz, _u32, _u32]
        R.mref_max_units.restype = _sz
        R.mref_encode.argtypes = [_u8p, _sz, _u32, _u32, _u32p, _u32p, _sz, _u32p, _u32p]
        R.mref_encode.restype = _sz
        R.mref_multicore_decode.argtypes = [_sz, _sz, _u32p, _sz, _u32, _u32, _u32p, _u32, _u8p, _sz]
        R.mref_multicore_decode.restype = ctypes.c_int
        _ref = R
    return _ref


# ---------------------------------------------------------------------------

@dataclass
class Stream:
    """One encoded stream plus what the decoder needs."""
    symbols: np.ndarray      # uint8, n (source order)
    units: np.ndarray        # uint32, n_units + 4 (CUHDInputBuffer order)
    n_units: int
    first_bit: int
    first_state: int
    table: np.ndarray        # uint32, L packed decoder words
    L: int

    @property
    def n(self) -> int:
        return int(self.symbols.size)

    @property
    def compressed_bytes(self) -> int:
        return self.n_units * 4

    @property
    def bits_per_symbol(self) -> float:
        return 32.0 * self.n_units / max(1, self.n)


def gen_symbols(seed: int, lam: float, n: int) -> np.ndarray:
    """Seeded synthetic symbols (one padding byte of 0 is appended for the
    encoder's read past the end and dropped from the returned view)."""
    buf = np.zeros(n + 1, dtype=np.uint8)
    lib().mo_gen_symbols(seed, lam, _ptr(buf, _u8p), n)
    return buf[:n]


def _padded(sym: np.ndarray) -> np.ndarray:
    buf = np.zeros(sym.size + 8, dtype=np.uint8)
    buf[: sym.size] = sym
    return buf


def build_tables(sym: np.ndarray, L: int, seed: int = TABLE_SEED):
    sym = np.ascontiguousarray(sym, dtype=np.uint8)
    enc = np.zeros(256 * L * 4, dtype=np.uint32)
    dec = np.zeros(L, dtype=np.uint32)
    ml = np.zeros(1, dtype=np.uint32)
    K = lib().mo_build_tables(_ptr(sym, _u8p), sym.size, L, seed, _ptr(enc, _u32p),
                              _ptr(dec, _u32p), _ptr(ml, _u32p))
    if K < 0:
        raise ValueError("table generation failed")
    return enc, dec, int(ml[0]), K


def encode(sym: np.ndarray, L: int, seed: int = TABLE_SEED) -> Stream:
    """Table generation + encoding with the oracle restatement."""
    enc, dec, ml, _ = build_tables(sym, L, seed)
    buf = _padded(sym)
    cap = lib().mo_max_units(ml, sym.size) + 4
    units = np.zeros(cap, dtype=np.uint32)
    fb = np.zeros(1, dtype=np.uint32)
    fs = np.zeros(1, dtype=np.uint32)
    nu = lib().mo_encode(_ptr(enc, _u32p), L, ml, _ptr(buf, _u8p), sym.size,
                         _ptr(units, _u32p), cap, _ptr(fb, _u32p), _ptr(fs, _u32p))
    if nu == 0:
        raise ValueError("encoding failed")
    return Stream(np.ascontiguousarray(sym, dtype=np.uint8), units[: nu + 4].copy(),
                  int(nu), int(fb[0]), int(fs[0]), dec, L)


def ref_encode(sym: np.ndarray, L: int, seed: int = TABLE_SEED) -> Stream:
    """Table generation + encoding with the reference's own code."""
    R = ref()
    buf = _padded(sym)
    cap = R.mref_max_units(_ptr(buf, _u8p), sym.size, L, seed) + 4
    units = np.zeros(cap, dtype=np.uint32)
    dec = np.zeros(L, dtype=np.uint32)
    fb = np.zeros(1, dtype=np.uint32)
    fs = np.zeros(1, dtype=np.uint32)
    nu = R.mref_encode(_ptr(buf, _u8p), sym.size, L, seed, _ptr(dec, _u32p),
                       _ptr(units, _u32p), cap, _ptr(fb, _u32p), _ptr(fs, _u32p))
    if nu == 0:
        raise ValueError("reference encoding failed")
    return Stream(np.ascontiguousarray(sym, dtype=np.uint8), units[: nu + 4].copy(),
                  int(nu), int(fb[0]), int(fs[0]), dec, L)


@dataclass
class SegStream:
    """A multi-table stream: one bitstream whose source segments were each
    encoded with their own table (mo_encode_segments).  Segment lists are in
    decode order: the source's last segment first."""
    symbols: np.ndarray      # uint8, source order (all segments)
    units: np.ndarray        # uint32, n_units + 4 (CUHDInputBuffer order)
    n_units: int
    first_bit: int
    first_state: int
    L: int
    tables: list             # uint32 arrays of L decoder words, decode order
    counts: list             # symbols per segment, decode order
    starts: list             # bit position of each segment's first codeword, decode order

    @property
    def n(self) -> int:
        return int(self.symbols.size)


def encode_segments(segs, L: int, seed: int = TABLE_SEED) -> SegStream:
    """Encodes source segments (uint8 arrays, source order), each with a table
    built from its own symbols, into one stream; the sequential multi-table
    decode gives the segments' start positions and must reproduce the
    source."""
    encs, decs, mls = [], [], []
    for sg in segs:
        enc, dec, ml, _ = build_tables(np.ascontiguousarray(sg, dtype=np.uint8), L, seed)
        encs.append(enc)
        decs.append(dec)
        mls.append(ml)
    sym = np.concatenate([np.ascontiguousarray(sg, dtype=np.uint8) for sg in segs])
    ends = np.cumsum([sg.size for sg in segs]).astype(np.uint64)
    buf = _padded(sym)
    cap = lib().mo_max_units(max(mls), sym.size) + 4
    units = np.zeros(cap, dtype=np.uint32)
    fb = np.zeros(1, dtype=np.uint32)
    fs = np.zeros(1, dtype=np.uint32)
    ptrs = (_u32p * len(encs))(*[_ptr(e, _u32p) for e in encs])
    ends_c = (ctypes.c_size_t * len(segs))(*[int(x) for x in ends])
    nu = lib().mo_encode_segments(ptrs, ends_c, len(segs), L, max(mls), _ptr(buf, _u8p),
                                  sym.size, _ptr(units, _u32p), cap, _ptr(fb, _u32p),
                                  _ptr(fs, _u32p))
    if nu == 0:
        raise ValueError("segment encoding failed")
    tables = decs[::-1]
    counts = [int(sg.size) for sg in segs][::-1]
    out = np.zeros(max(1, sym.size), dtype=np.uint8)
    starts = np.zeros(len(segs), dtype=np.uint64)
    u = np.ascontiguousarray(units[:nu])
    dptrs = (_u32p * len(tables))(*[_ptr(t, _u32p) for t in tables])
    cnt = (ctypes.c_size_t * len(counts))(*counts)
    rc = lib().mo_decode_segments(_ptr(u, _u32p), int(nu), int(fb[0]), int(fs[0]), dptrs, cnt,
                                  len(counts), L, _ptr(out, _u8p),
                                  starts.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
    if rc != 0 or not np.array_equal(out[: sym.size][::-1], sym):
        raise ValueError("segment stream does not decode back to its source")
    return SegStream(sym, units[: nu + 4].copy(), int(nu), int(fb[0]), int(fs[0]), L,
                     tables, counts, [int(x) for x in starts])


def decode_segments_seq(ss: SegStream) -> np.ndarray:
    """Sequential multi-table decode: symbols in decode order."""
    out = np.zeros(max(1, ss.n), dtype=np.uint8)
    starts = np.zeros(len(ss.counts), dtype=np.uint64)
    u = np.ascontiguousarray(ss.units[: ss.n_units])
    dptrs = (_u32p * len(ss.tables))(*[_ptr(t, _u32p) for t in ss.tables])
    cnt = (ctypes.c_size_t * len(ss.counts))(*ss.counts)
    rc = lib().mo_decode_segments(_ptr(u, _u32p), ss.n_units, ss.first_bit, ss.first_state,
                                  dptrs, cnt, len(ss.counts), ss.L, _ptr(out, _u8p),
                                  starts.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)))
    if rc != 0:
        raise ValueError("sequential segment decode failed")
    return out[: ss.n]


def make_stream(seed: int, lam: float, n: int, L: int) -> Stream:
    return encode(gen_symbols(seed, lam, n), L)


def decode_seq(st: Stream, n_out: int | None = None) -> np.ndarray:
    """Sequential decode; returns symbols in decode (reversed) order."""
    n_out = st.n if n_out is None else n_out
    out = np.zeros(max(1, n_out), dtype=np.uint8)
    u = np.ascontiguousarray(st.units[: st.n_units])
    rc = lib().mo_decode_seq(_ptr(u, _u32p), st.n_units, st.first_bit, st.first_state,
                             _ptr(st.table, _u32p), st.L, _ptr(out, _u8p), n_out)
    if rc != 0:
        raise ValueError("sequential decode failed")
    return out[:n_out]


def sync_points(st: Stream, S: int) -> np.ndarray:
    """True sync points (nsub x 4: unit, bit, exclusive offset, state)."""
    nsub = (st.n_units + S - 1) // S
    sp = np.zeros(nsub * 4, dtype=np.uint32)
    u = np.ascontiguousarray(st.units[: st.n_units])
    rc = lib().mo_sync_points(S, _ptr(u, _u32p), st.n_units, st.first_bit, st.first_state,
                              _ptr(st.table, _u32p), st.L, _ptr(sp, _u32p))
    if rc != 0:
        raise ValueError("sync point computation failed")
    return sp.reshape(nsub, 4)


def multicore_decode(st: Stream, S: int = 4, T: int = 4, n_out: int | None = None):
    """The reference method restated on T threads; returns (symbols in decode
    order, repair passes)."""
    n_out = st.n if n_out is None else n_out
    out = np.zeros(max(1, n_out), dtype=np.uint8)
    u = np.ascontiguousarray(st.units[: st.n_units])
    rc = lib().mo_multicore_decode(S, T, _ptr(u, _u32p), st.n_units, st.first_bit,
                                   st.first_state, _ptr(st.table, _u32p), st.L,
                                   _ptr(out, _u8p), n_out)
    if rc == -2:
        raise ValueError("multicore decode met a zero-bit cycle (single-symbol table)")
    if rc < 0:
        raise ValueError("multicore decode rejected its arguments")
    return out[:n_out], rc


def ref_multicore_decode(st: Stream, S: int = 4, T: int = 4, n_out: int | None = None):
    """MulticoreDecoder::decode of the reference itself (decode order)."""
    n_out = st.n if n_out is None else n_out
    out = np.zeros(max(1, n_out), dtype=np.uint8)
    u = np.ascontiguousarray(st.units[: st.n_units])
    ref().mref_multicore_decode(S, T, _ptr(u, _u32p), st.n_units, st.first_bit,
                                st.first_state, _ptr(st.table, _u32p), st.L,
                                _ptr(out, _u8p), n_out)
    return out[:n_out]
