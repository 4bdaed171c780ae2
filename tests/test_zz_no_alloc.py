"""The allocation-free decode entry point (mans_decode_noalloc), called
through the C ABI: for callers that cannot allocate device memory when they
decode, the workspace is a fixed device array inside the library.  Its
output must equal the regular entry point's, byte for byte (integer work:
the tolerance is zero), on two calls in a row -- the array keeps the first
call's contents, so the second call shows the decode does not depend on
what an earlier call left there.  Kept in its own file, collected last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


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


def test_noalloc_matches_regular_decode_twice():
    import torch

    import multians_gb300 as mg
    from multians_gb300 import host

    lib = mg.lib()
    noalloc, scratch_bytes = _noalloc(lib)
    assert scratch_bytes() == 32 << 20
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


def test_noalloc_rejects_streams_beyond_the_array():
    import torch

    import multians_gb300 as mg

    lib = mg.lib()
    noalloc, _ = _noalloc(lib)
    too_many = 400_000_000   # units: the planned workspace is far above 32 MiB
    dummy = torch.zeros(16, dtype=torch.int32, device="cuda")
    p = ctypes.c_void_p(dummy.data_ptr())
    status = ctypes.c_uint32(0)
    rc = noalloc(p, too_many, p, too_many * 5, p, 1024, 1024, 0,
                 ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), ctypes.byref(status))
    assert rc == mg.Status.ERR_AUX_SMALL
