"""multians_gb300: GB300-native (sm_103a) MULTIANS tANS decoding.

Python host mirror of the reference decode interface
(cuhd::CUHDGPUDecoder::decode, include/cuhd_gpu_decoder.h:24-35) over the
C ABI of ``libmultians_gb300.so`` (include/multians_gb300.h).  Device
buffers are torch CUDA tensors; nothing here computes on the CPU: if the
native library is missing the import fails.
"""
from __future__ import annotations

from ._lib import (  # noqa: F401
    LIB_PATH,
    MansError,
    Status,
    DEV_BAD_TABLE,
    DEV_SYNC_OVERFLOW,
    DEV_DEGENERATE,
    DEV_COUNT_MISMATCH,
    DECODE_SOURCE_ORDER,
    DECODE_NO_CAPTURE,
    DECODE_CAPTURE,
    PLAN_MODEL,
    DECODE_START_OFFSET,
    DECODE_SEEDS,
    DECODE_NO_SEEDS,
    plan_tuned,
    tune_lookup,
    lib,
    plan,
    aux_size,
    aux_size_max,
    aux_size_max_any,
    table_check,
    version,
)
from .decoder import (  # noqa: F401
    CUHDGPUDecoder,
    CUHDGPUDecoderMemory,
    decode,
    decode_async,
)

__all__ = [
    "CUHDGPUDecoder",
    "CUHDGPUDecoderMemory",
    "decode",
    "decode_async",
    "plan",
    "aux_size",
    "aux_size_max",
    "aux_size_max_any",
    "table_check",
    "version",
    "MansError",
    "Status",
]
