"""Argument checks of the serving calls that need no device (a null server
handle, null outputs): they return MANS_ERR_ARG, and destroying a null
server is a no-op, as for free()."""
import ctypes

import numpy as np


def test_server_calls_refuse_null_handles(mg):
    from multians_gb300 import serve
    lib = serve._sig()
    t = np.zeros(1024, dtype=np.uint32)
    tid = ctypes.c_uint32()
    u32p = ctypes.POINTER(ctypes.c_uint32)
    assert lib.mans_server_add_table(None, t.ctypes.data_as(u32p), 1024, ctypes.byref(tid)) == \
        mg.Status.ERR_ARG
    req = (serve.RequestC * 1)()
    assert lib.mans_server_submit(None, req, 1) == mg.Status.ERR_ARG
    n = ctypes.c_size_t()
    buf = (serve.CompletionC * 4)()
    assert lib.mans_server_poll(None, buf, 4, ctypes.byref(n), 0) == mg.Status.ERR_ARG
    st = serve.StatsC()
    assert lib.mans_server_stats_get(None, ctypes.byref(st)) == mg.Status.ERR_ARG
    assert lib.mans_server_destroy(None) == mg.Status.OK
    assert lib.mans_server_create(None, None) == mg.Status.ERR_ARG
