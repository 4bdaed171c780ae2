"""Host-side properties of batch planning (no GPU: the sizing calls touch no
device memory, so placeholder device addresses do).  The serving loop
reserves each request's workspace slice from a plan of that request alone
(mans_batch_slice_size) and then decodes a batch of them in those slices
(mans_batch_create_split): a stream's workspace inside a batch must never
exceed its slice, or the batch would write past it."""
import ctypes

import numpy as np
import pytest


def _descs(batch, specs):
    out = []
    for i, (n_units, n_out, L) in enumerate(specs):
        base = 0x100000 * (i + 1)   # 16-byte aligned placeholders, never dereferenced
        out.append(batch.StreamDesc(base, n_units, base + 0x80000, n_out, base + 0x40000, L,
                                    L, 32, 0))
    return out


def _sizes(mg, batch, descs):
    lib = mg.lib()
    lib.mans_batch_slice_size.argtypes = [ctypes.POINTER(batch.StreamDesc), ctypes.c_void_p,
                                          ctypes.POINTER(ctypes.c_size_t)]
    lib.mans_batch_header_size.argtypes = [ctypes.POINTER(batch.StreamDesc), ctypes.c_uint32,
                                           ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)]
    n = len(descs)
    arr = (batch.StreamDesc * n)(*descs)
    slices = []
    for i in range(n):
        v = ctypes.c_size_t()
        assert lib.mans_batch_slice_size(ctypes.byref(arr[i]), None, ctypes.byref(v)) == 0
        slices.append(v.value)
    hdr = ctypes.c_size_t()
    assert lib.mans_batch_header_size(arr, n, None, ctypes.byref(hdr)) == 0
    whole = ctypes.c_size_t()
    batch._sig()
    assert lib.mans_batch_workspace_size(arr, n, None, ctypes.byref(whole)) == 0
    return slices, hdr.value, whole.value


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_batch_slices_cover_batch_plans(mg, seed):
    """Batch-level region lengths only shrink a stream's workspace: the
    batch's data region never exceeds the slices planned one by one."""
    from multians_gb300 import batch
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(64):
        n_out = int(np.exp(rng.uniform(np.log(4_000), np.log(64 << 20))))
        bps = float(rng.uniform(0.7, 8.5))
        n_units = max(1, int(n_out * bps / 32))
        specs.append((n_units, n_out, int(rng.choice([1024, 4096]))))
    slices, hdr, whole = _sizes(mg, batch, _descs(batch, specs))
    assert whole - hdr <= sum(slices)


def test_batch_plans_one_stream_like_plain(mg):
    """A batch of one stream plans it like the plain path's model does (same
    slice as the plain workspace, to the 256-byte rounding, less the plain
    workspace's seeded-walk records: batches walk without seeds); batches
    keep the model where a plain decode reads the measured table."""
    from multians_gb300 import batch
    seed_records = 32 * 32 * 32 * 8   # slots x lanes x blocks x 8 bytes
    for n_units, n_out, L in ((50_339_428, 268_435_456, 1024), (120_000, 700_000, 4096)):
        slices, _, _ = _sizes(mg, batch, _descs(batch, [(n_units, n_out, L)]))
        plain = mg.aux_size(n_units, mg.plan(n_units, n_out, L, {"flags": mg.PLAN_MODEL}))
        assert abs(slices[0] - (plain - seed_records)) <= 256, (slices[0], plain)


def test_batch_slices_cover_edge_streams(mg):
    """The same bound for streams at the edges of the planner: one unit,
    one symbol, extreme compression ratios (zero-bit runs: many symbols per
    unit; 8+ bits per symbol), every table size, and an empty output."""
    from multians_gb300 import batch
    specs = [(1, 1, 1024), (1, 40, 4096), (4, 1, 256), (2, 512, 8192),
             (1_000, 400_000, 4096), (1_000, 3_000, 1024), (70_000, 260_000, 2048),
             (5_000_000, 20_000_000, 1024), (3, 0, 1024), (17, 33, 8192)]
    slices, hdr, whole = _sizes(mg, batch, _descs(batch, specs))
    assert whole - hdr <= sum(slices)
    assert all(s > 0 for s, (_, n_out, _) in zip(slices, specs) if n_out)


@pytest.mark.parametrize("field,value", [
    ("d_units", 0x100004), ("d_units", None), ("d_out", None), ("d_table", None),
    ("n_units", 0), ("n_units", 1 << 32), ("L", 1), ("L", 16384),
    ("first_state", 1023), ("first_state", 2048), ("first_bit", 33)])
def test_batch_refuses_bad_descriptors(mg, field, value):
    """A malformed stream descriptor fails the whole batch with
    MANS_ERR_ARG at sizing time, before any device work."""
    import ctypes
    from multians_gb300 import batch
    descs = _descs(batch, [(1000, 5000, 1024), (2000, 9000, 1024)])
    setattr(descs[1], field, value)
    batch._sig()
    arr = (batch.StreamDesc * 2)(*descs)
    out = ctypes.c_size_t()
    assert mg.lib().mans_batch_workspace_size(arr, 2, None, ctypes.byref(out)) == \
        mg.Status.ERR_ARG
