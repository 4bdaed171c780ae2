"""Python mirror of the reference decode call.

``CUHDGPUDecoder.decode`` takes the reference's arguments in the
reference's order (include/cuhd_gpu_decoder.h:24-35) with torch CUDA
tensors standing in for the GPU buffer classes; ``CUHDGPUDecoderMemory``
stands in for the decoder-memory class
(include/cuhd_gpu_decoder_memory.h:20-45).  Errors raise MansError where the
reference prints and exits (include/cuhd_cuda_definitions.h:21-28).
"""
from __future__ import annotations

import ctypes

from ._lib import Cfg, MansError, Status, check, lib, aux_size_max, aux_size_max_any


def _torch():
    import torch
    return torch


def _stream_ptr(stream):
    torch = _torch()
    if stream is None:
        stream = torch.cuda.current_stream()
    return ctypes.c_void_p(stream.cuda_stream)


def _dev_ptr(t, nbytes: int = 0, what: str = "tensor"):
    """Device address of a contiguous CUDA tensor holding at least `nbytes`
    bytes on the current device.  The C calls see only addresses, so a
    short buffer has to be refused here, before any kernel reads or writes
    past its end."""
    if not t.is_cuda:
        raise ValueError(f"{what}: expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError(f"{what}: expected a contiguous tensor")
    have = t.numel() * t.element_size()
    if have < nbytes:
        raise ValueError(f"{what}: {have} bytes, the call needs {nbytes}")
    if t.device.index is not None:
        cur = _torch().cuda.current_device()
        if t.device.index != cur:
            raise ValueError(f"{what}: on {t.device}, the current device is cuda:{cur}")
    return ctypes.c_void_p(t.data_ptr())


class CUHDGPUDecoderMemory:
    """Decoder scratch memory sized for ``num_units`` units.  The reference
    sizes it by (units, subsequence size, threads per block)
    (src/multians_gpu_decoder_memory.cc:13-19); here the size covers every
    geometry the planner may choose, symbol capture included, so a decode
    never needs more; the two hints are kept only for the signature."""

    def __init__(self, num_units: int, subsequence_size: int = 4, num_threads: int = 128,
                 device=None):
        self.num_units = int(num_units)
        self.subsequence_size = subsequence_size
        self.num_threads = num_threads
        self.device = device
        self.buf = None

    @property
    def nbytes(self) -> int:
        return aux_size_max_any(max(1, self.num_units))

    def allocate(self):
        if self.buf is None:
            torch = _torch()
            self.buf = torch.empty(self.nbytes, dtype=torch.uint8,
                                   device=self.device or "cuda")
        return self

    def free(self):
        self.buf = None

    def get(self):
        return self.buf


class CUHDGPUDecoder:
    @staticmethod
    def decode(input, input_size: int, output, output_size: int, table, aux,
               initial_state: int, initial_bit: int, number_of_states: int,
               max_codeword_length: int = 0, preferred_subsequence_size: int = 0,
               threads_per_block: int = 0, stream=None) -> int:
        """Same arguments as the reference; ``input`` is a CUDA uint32 tensor
        of units (CUHDInputBuffer order), ``table`` a CUDA uint32 tensor of
        packed CUHDCodetableItem words, ``output`` a CUDA uint8 tensor.
        Synchronous; returns the device status bits."""
        # unused by the reference too (.cu:217); the geometry is the planner's
        del max_codeword_length, preferred_subsequence_size, threads_per_block
        if aux.get() is None:
            raise MansError(Status.ERR_ARG, "CUHDGPUDecoder.decode: decoder memory not allocated")
        st = ctypes.c_uint32(0)
        rc = lib().mans_decode_sync(
            _dev_ptr(input, 4 * int(input_size), "input"), int(input_size),
            _dev_ptr(output, int(output_size), "output"), int(output_size),
            _dev_ptr(table, 4 * int(number_of_states), "table"), int(number_of_states),
            int(initial_state), int(initial_bit),
            _dev_ptr(aux.get()), aux.get().numel(), None, _stream_ptr(stream), ctypes.byref(st))
        check(rc, "CUHDGPUDecoder.decode")
        return int(st.value)


def decode_async(units, n_units: int, out, n_out: int, table, L: int, first_state: int,
                 first_bit: int, aux, cfg: dict | None = None, stream=None) -> None:
    """Enqueues one decode (mans_decode); no host synchronisation."""
    c = Cfg(**(cfg or {}))
    rc = lib().mans_decode(_dev_ptr(units, 4 * int(n_units), "units"), int(n_units),
                           _dev_ptr(out, int(n_out), "out"), int(n_out),
                           _dev_ptr(table, 4 * int(L), "table"), int(L),
                           int(first_state), int(first_bit),
                           _dev_ptr(aux), aux.numel(), ctypes.byref(c), _stream_ptr(stream))
    check(rc, "mans_decode")


def aux_status(aux, stream=None) -> int:
    st = ctypes.c_uint32(0)
    check(lib().mans_aux_status(_dev_ptr(aux), _stream_ptr(stream), ctypes.byref(st)),
          "mans_aux_status")
    return int(st.value)


def decode(units, n_units: int, n_out: int, table, first_state: int, first_bit: int,
           L: int | None = None, aux=None, out=None, stream=None, cfg: dict | None = None,
           source_order: bool = False):
    """Decodes one stream and returns the symbols (CUDA uint8): in decode
    order like the reference, or with ``source_order`` the i-th decoded
    symbol at out[n_out - 1 - i] (a full decode is then the source).

    ``units``/``table`` may be numpy arrays (copied to the device) or CUDA
    tensors."""
    if source_order:
        from ._lib import DECODE_SOURCE_ORDER
        cfg = dict(cfg or {})
        cfg["flags"] = cfg.get("flags", 0) | DECODE_SOURCE_ORDER
    torch = _torch()
    dev = torch.device("cuda")
    if not hasattr(units, "is_cuda"):
        import numpy as np
        units = torch.from_numpy(np.ascontiguousarray(units).view(np.int32)).to(dev)
    if not hasattr(table, "is_cuda"):
        import numpy as np
        table = torch.from_numpy(np.ascontiguousarray(table).view(np.int32)).to(dev)
    L = int(table.numel()) if L is None else int(L)
    if out is None:
        out = torch.empty(max(1, n_out), dtype=torch.uint8, device=dev)
    if aux is None:
        from ._lib import plan, aux_size
        need = max(aux_size_max(max(1, n_units)),
                   aux_size(n_units, plan(n_units, n_out, L, cfg or {})))
        aux = torch.empty(need, dtype=torch.uint8, device=dev)
    st = ctypes.c_uint32(0)
    rc = lib().mans_decode_sync(_dev_ptr(units, 4 * int(n_units), "units"), int(n_units),
                                _dev_ptr(out, int(n_out), "out"), int(n_out),
                                _dev_ptr(table, 4 * L, "table"), L,
                                int(first_state), int(first_bit),
                                _dev_ptr(aux), aux.numel(),
                                ctypes.byref(Cfg(**cfg)) if cfg else None,
                                _stream_ptr(stream), ctypes.byref(st))
    if rc != Status.OK:
        raise MansError(rc, f"decode (device status 0x{st.value:x})")
    return out[:n_out]
