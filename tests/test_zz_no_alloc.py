"""The allocation-free decode entry point (mans_decode_noalloc), called
through the C ABI: for callers that cannot allocate device memory when they
decode, the workspace is a fixed device array inside the library.  Its
output must equal the regular entry point's, byte for byte (integer work:
the tolerance is zero), on two calls in a row -- the array keeps the first
call's contents, so the second call shows the decode does not depend on
what an earlier call left there.  Kept in its own file, collected last.

The CPU tests check the stated acceptance limits (the largest streams a
plan of which fits the array) and that bad arguments are refused before
any device work."""
import ctypes

import numpy as np
import pytest

SCRATCH = 32 << 20


def _noalloc(lib):
    f = lib.mans_decode_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                  ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                  ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32)]
    f.restype = ctypes.c_int
    g = lib.mans_noalloc_scratch_bytes
    g.argtypes = []
    g.restype = ctypes.c_size_t
    return f, g


def _fits(mg, n_units, n_out, L):
    """Whether a plan of the stream fits the array, tried in the order the
    synchronous decode tries them: the planner's, no capture, fewer slots."""
    c = {}
    for _ in range(8):
        p = mg.plan(n_units, n_out, L, c)
        if mg.aux_size(n_units, p) <= SCRATCH:
            return True
        if p["capture_bytes"]:
            c = dict(c, capture_bytes=0, flags=c.get("flags", 0) | mg.DECODE_NO_CAPTURE)
        elif p["walk_slots"] > 1:
            c = dict(p, walk_slots=p["walk_slots"] // 2)
        else:
            return False
    return False


def _limit_units(mg, bits_per_symbol, L):
    lo, hi = 1, 1 << 31
    while hi - lo > 1:
        m = (lo + hi) // 2
        if _fits(mg, m, int(m * 32 / bits_per_symbol), L):
            lo = m
        else:
            hi = m
    return lo


def test_documented_limits(mg):
    """The header, the notes and the integration guide state about 28
    million units at 6 bits/symbol and 7.7 million at 0.67 (L = 1024)."""
    assert mg.lib().mans_noalloc_scratch_bytes() == SCRATCH
    for bps, stated in ((6.0, 28e6), (8.6, 28e6), (0.67, 7.7e6)):
        got = _limit_units(mg, bps, 1024)
        assert abs(got - stated) / stated < 0.03, (bps, got)


def test_bad_arguments_refused_first(mg):
    """Argument errors come back as MANS_ERR_ARG whatever the stream size,
    before the array's address is looked up (no device is needed)."""
    noalloc, _ = _noalloc(mg.lib())
    ok = ctypes.c_void_p(1 << 20)   # never dereferenced: every case fails its checks
    odd = ctypes.c_void_p((1 << 20) + 4)
    st = ctypes.c_uint32(7)
    cases = [
        (None, 100, ok, 10, ok, 1024, 1024, 0),
        (odd, 100, ok, 10, ok, 1024, 1024, 0),
        (ok, 100, None, 10, ok, 1024, 1024, 0),
        (ok, 100, ok, 10, None, 1024, 1024, 0),
        (ok, 0, ok, 10, ok, 1024, 1024, 0),
        (ok, 1 << 33, ok, 10, ok, 1024, 1024, 0),
        (ok, 100, ok, 10, ok, 1, 1, 0),
        (ok, 100, ok, 10, ok, 16384, 16384, 0),
        (ok, 100, ok, 10, ok, 1024, 1023, 0),
        (ok, 100, ok, 10, ok, 1024, 2048, 0),
        (ok, 400_000_000, ok, 10, ok, 1024, 1024, 33),
    ]
    for c in cases:
        assert noalloc(*c, None, ctypes.byref(st)) == mg.Status.ERR_ARG, c
        assert st.value == 0
    assert noalloc(ok, 100, ok, 0, ok, 1024, 1024, 0, None, ctypes.byref(st)) == 0


@pytest.mark.gpu
def test_noalloc_matches_regular_decode_twice():
    import torch

    import multians_gb300 as mg
    from multians_gb300 import host

    lib = mg.lib()
    noalloc, scratch_bytes = _noalloc(lib)
    assert scratch_bytes() == SCRATCH
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    for seed, lam, n, L in ((11, 0.05, 3_000_000, 1024), (12, 2.0, 2_000_000, 4096)):
        st = host.make_stream(seed, lam, n, L)
        units = torch.from_numpy(st.units.view(np.int32)).cuda()
        table = torch.from_numpy(st.table.view(np.int32)).cuda()
        want = mg.decode(units, st.n_units, n, table, st.first_state, st.first_bit, L=L)
        want = want.cpu().numpy()
        assert np.array_equal(want[::-1], st.symbols)
        for _ in range(2):
            out = torch.full((n,), 0x5A, dtype=torch.uint8, device="cuda")
            status = ctypes.c_uint32(0xFFFF)
            rc = noalloc(ctypes.c_void_p(units.data_ptr()), st.n_units,
                         ctypes.c_void_p(out.data_ptr()), n, ctypes.c_void_p(table.data_ptr()),
                         L, st.first_state, st.first_bit, sp, ctypes.byref(status))
            assert rc == 0 and status.value == 0, (rc, status.value)
            assert np.array_equal(out.cpu().numpy(), want)


@pytest.mark.gpu
def test_noalloc_near_and_past_the_limit():
    """A stream just under the acceptance limit (it decodes with fewer walk
    slots, and re-plans inside the array if a walk runs out) equals the
    regular decode twice; one just over it is refused before any GPU work
    (its buffers are real and zero-filled all the same)."""
    import torch

    import multians_gb300 as mg
    from multians_gb300 import host

    lib = mg.lib()
    noalloc, _ = _noalloc(lib)
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    lam, L = 0.005, 1024
    limit = _limit_units(mg, 8.57, L)
    n = int(0.97 * limit * 32 / 8.57)
    st = host.make_stream(21, lam, n, L)
    assert _fits(mg, st.n_units, n, L) and st.n_units > 0.9 * limit
    assert mg.aux_size(st.n_units, mg.plan(st.n_units, n, L)) > SCRATCH  # planner's own: too big
    units = torch.from_numpy(st.units.view(np.int32)).cuda()
    table = torch.from_numpy(st.table.view(np.int32)).cuda()
    want = mg.decode(units, st.n_units, n, table, st.first_state, st.first_bit, L=L).cpu().numpy()
    assert np.array_equal(want[::-1], st.symbols)
    for _ in range(2):
        out = torch.full((n,), 0x5A, dtype=torch.uint8, device="cuda")
        status = ctypes.c_uint32(0xFFFF)
        rc = noalloc(ctypes.c_void_p(units.data_ptr()), st.n_units,
                     ctypes.c_void_p(out.data_ptr()), n, ctypes.c_void_p(table.data_ptr()),
                     L, st.first_state, st.first_bit, sp, ctypes.byref(status))
        assert rc == 0 and status.value == 0, (rc, status.value)
        assert np.array_equal(out.cpu().numpy(), want)
    del out, units
    over = int(limit * 1.05)
    n_over = int(over * 32 / 8.57)
    assert not _fits(mg, over, n_over, L)
    big_units = torch.zeros(over + 4, dtype=torch.int32, device="cuda")
    big_out = torch.zeros(n_over, dtype=torch.uint8, device="cuda")
    status = ctypes.c_uint32(0)
    rc = noalloc(ctypes.c_void_p(big_units.data_ptr()), over, ctypes.c_void_p(big_out.data_ptr()),
                 n_over, ctypes.c_void_p(table.data_ptr()), L, st.first_state, st.first_bit, sp,
                 ctypes.byref(status))
    assert rc == mg.Status.ERR_AUX_SMALL
    assert int(big_out.count_nonzero()) == 0
