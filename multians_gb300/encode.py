"""GPU encoder through the C ABI: byte histogram on the device, the
reference's table build on the host from it, the tANS encode on the device
(mans_histogram, mans_host_encode_tables, mans_encode).  The result equals
host.encode() bit for bit."""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import MansError, check, lib
from .host import TABLE_SEED

_u32p = ctypes.POINTER(ctypes.c_uint32)
_u64p = ctypes.POINTER(ctypes.c_uint64)
_vp = ctypes.c_void_p


def _sig():
    L = lib()
    L.mans_encode_blob_words.argtypes = [ctypes.c_uint32]
    L.mans_encode_blob_words.restype = ctypes.c_size_t
    L.mans_histogram.argtypes = [_vp, ctypes.c_size_t, _vp, _vp]
    L.mans_histogram.restype = ctypes.c_int
    L.mans_host_encode_tables.argtypes = [_u64p, ctypes.c_uint32, ctypes.c_uint32, _u32p, _u32p]
    L.mans_host_encode_tables.restype = ctypes.c_int
    L.mans_encode_max_units.argtypes = [ctypes.c_size_t, ctypes.c_uint32]
    L.mans_encode_max_units.restype = ctypes.c_size_t
    L.mans_encode_aux_size.argtypes = [ctypes.c_size_t, ctypes.c_uint32]
    L.mans_encode_aux_size.restype = ctypes.c_size_t
    L.mans_encode.argtypes = [_vp, ctypes.c_size_t, _vp, ctypes.c_uint32, _vp, ctypes.c_size_t,
                              _vp, ctypes.c_size_t, ctypes.c_uint32, _vp]
    L.mans_encode.restype = ctypes.c_int
    L.mans_encode_result.argtypes = [_vp, _vp, _u64p, _u32p, _u32p, _u32p]
    L.mans_encode_result.restype = ctypes.c_int
    L.mans_encode_sync.argtypes = [_vp, ctypes.c_size_t, _vp, ctypes.c_uint32, _vp,
                                   ctypes.c_size_t, _vp, ctypes.c_size_t, _vp, _u64p, _u32p, _u32p]
    L.mans_encode_sync.restype = ctypes.c_int
    return L


def tables_from_histogram(hist, L: int, table_seed: int = TABLE_SEED):
    """(decoder table uint32[L], encoder blob uint32[...]) from 256 byte counts."""
    h = np.ascontiguousarray(hist, dtype=np.uint64)
    lb = _sig()
    dec = np.zeros(L, dtype=np.uint32)
    blob = np.zeros(int(lb.mans_encode_blob_words(L)), dtype=np.uint32)
    check(lb.mans_host_encode_tables(h.ctypes.data_as(_u64p), L, table_seed,
                                      dec.ctypes.data_as(_u32p), blob.ctypes.data_as(_u32p)),
          "mans_host_encode_tables")
    return dec, blob


def encode(symbols, L: int, table_seed: int = TABLE_SEED, chunk: int = 0, stream=None):
    """Encodes uint8 symbols (numpy array or CUDA tensor) on the GPU.
    Returns (units CUDA int32 tensor of n_units + 4, n_units, first_bit,
    first_state, decoder table numpy uint32[L])."""
    import torch
    dev = torch.device("cuda")
    if not hasattr(symbols, "is_cuda"):
        symbols = torch.from_numpy(np.ascontiguousarray(symbols, dtype=np.uint8)).to(dev)
    n = int(symbols.numel())
    if n == 0:
        raise MansError(1, "encode: no symbols")
    st = torch.cuda.current_stream() if stream is None else stream
    sp = ctypes.c_void_p(st.cuda_stream)
    lb = _sig()
    hist = torch.empty(256, dtype=torch.int64, device=dev)
    check(lb.mans_histogram(symbols.data_ptr(), n, hist.data_ptr(), sp), "mans_histogram")
    dec, blob = tables_from_histogram(hist.cpu().numpy().astype(np.uint64), L, table_seed)
    d_blob = torch.from_numpy(blob.view(np.int32)).to(dev)
    cap = int(lb.mans_encode_max_units(n, L))
    units = torch.empty(cap, dtype=torch.int32, device=dev)
    aux = torch.empty(int(lb.mans_encode_aux_size(n, chunk)), dtype=torch.uint8, device=dev)
    nu = ctypes.c_uint64(0)
    fb = ctypes.c_uint32(0)
    fs = ctypes.c_uint32(0)
    if chunk:
        ds = ctypes.c_uint32(0)
        check(lb.mans_encode(symbols.data_ptr(), n, d_blob.data_ptr(), L, units.data_ptr(), cap,
                             aux.data_ptr(), aux.numel(), chunk, sp), "mans_encode")
        check(lb.mans_encode_result(aux.data_ptr(), sp, ctypes.byref(nu), ctypes.byref(fb),
                                    ctypes.byref(fs), ctypes.byref(ds)),
              f"mans_encode (device status 0x{ds.value:x})")
    else:
        check(lb.mans_encode_sync(symbols.data_ptr(), n, d_blob.data_ptr(), L, units.data_ptr(),
                                  cap, aux.data_ptr(), aux.numel(), sp, ctypes.byref(nu),
                                  ctypes.byref(fb), ctypes.byref(fs)), "mans_encode_sync")
    n_units = int(nu.value)
    return units[: n_units + 4], n_units, int(fb.value), int(fs.value), dec
