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


def test_server_cfg_mirrors_header():
    """The Python mirror of mans_server_cfg has the header's fields, in its
    order and widths (small_bytes took the first reserved word)."""
    import os
    import re

    from multians_gb300 import serve
    hdr = open(os.path.join(os.path.dirname(__file__), "..", "include", "multians_gb300.h")).read()
    body = re.search(r"typedef struct \{([^}]*)\} mans_server_cfg;", hdr).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = re.findall(r"(uint64_t|uint32_t)\s+(\w+)(\[\d+\])?;", body)
    assert [f[1] for f in fields] == [f[0] for f in serve.ServerCfg._fields_]
    width = {"uint64_t": 8, "uint32_t": 4}
    assert sum(width[t] * (int(n[1:-1]) if n else 1) for t, _, n in fields) == \
        ctypes.sizeof(serve.ServerCfg) == 24
    assert serve.SMALL_OFF == 0xFFFFFFFF
