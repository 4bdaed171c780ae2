"""CPU tests of the native boundary: the library loads (no GPU needed) and
exports every entry point that include/*.h declares; host-side planning and
table checks behave."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")


def _declared_c_symbols():
    names = set()
    for f in os.listdir(INCLUDE):
        if not f.endswith(".h"):
            continue
        text = open(os.path.join(INCLUDE, f)).read()
        if 'extern "C"' not in text:
            continue
        for m in re.finditer(r"^\s*(?:[A-Za-z_][\w\s\*]*?)\b(mans_\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_entry_points():
    names = _declared_c_symbols()
    assert "mans_decode" in names and "mans_aux_size" in names


def test_library_exports_declared_symbols(mg):
    lib = mg.lib()
    out = subprocess.run(["nm", "-D", "--defined-only", mg.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    missing = [n for n in _declared_c_symbols() if n not in exported]
    assert not missing, missing
    for n in _declared_c_symbols():
        assert hasattr(lib, n)


def test_version(mg):
    assert mg.version().startswith("multians_gb300")


def test_plan_and_aux_sizes(mg):
    p = mg.plan(50_000_000, 268_435_456, 1024, {"flags": mg.DECODE_NO_CAPTURE})
    assert p["block_units"] >= 4 and p["region_blocks"] >= 1 and p["walk_slots"] >= 1
    assert p["capture_bytes"] == 0
    need = mg.aux_size(50_000_000, p)
    assert 0 < need <= mg.aux_size_max(50_000_000)
    small = mg.plan(1000, 5000, 4096)
    assert small["capture_bytes"] == 0   # too short
    assert mg.aux_size(1000, small) <= mg.aux_size_max(1000)


def test_capture_plan(mg):
    """6 bits per symbol at L = 1024 captures: one slice per region holding
    the region's symbols and a walk's with room to spare; low-entropy
    streams, short ones and L > 4096 do not."""
    n_units, n_out = 50_000_000, 268_435_456
    p = mg.plan(n_units, n_out, 1024)
    R = p["block_units"] * p["region_blocks"]
    per_region = n_out / n_units * R
    assert p["capture_bytes"] % 16 == 0 and p["capture_bytes"] >= 1.25 * per_region
    nblk = n_units // p["block_units"] + 1
    nreg = -(-nblk // p["region_blocks"])
    assert nreg <= 152 * 16 * 32   # the capture G pass keeps one wave
    extra = mg.aux_size(n_units, p) - mg.aux_size(n_units, dict(p, capture_bytes=0))
    assert extra >= nreg * p["capture_bytes"]
    assert mg.plan(20_000_000, 400_000_000, 1024)["capture_bytes"] == 0   # 1.6 bits/symbol
    assert mg.plan(20_000_000, 100_000_000, 8192)["capture_bytes"] == 0
    p4 = mg.plan(20_000_000, 100_000_000, 4096)   # L = 4096: half the resident lanes
    assert p4["capture_bytes"] > 0
    assert mg.plan(12_000_000, 64_000_000, 1024)["capture_bytes"] == 0    # short stream
    forced = mg.plan(1_000_000, 20_000_000, 1024, {"capture_bytes": 1000})
    assert forced["capture_bytes"] == 1008
    short = mg.plan(1_000_000, 5_000_000, 1024, {"flags": mg.DECODE_CAPTURE})
    assert short["capture_bytes"] > 0                                      # asked for
    assert mg.plan(1_000_000, 20_000_000, 1024, {"flags": mg.DECODE_CAPTURE})["capture_bytes"] == 0


def test_table_check(mg, oracle_lib):
    st = oracle_lib.make_stream(seed=1, lam=0.05, n=5000, L=1024)
    assert mg.table_check(st.table) == 0
    bad = st.table.copy()
    bad[0] = bad[0] & 0x00ffffff | (20 << 24)
    assert mg.table_check(bad) == -1
    one = oracle_lib.encode(np.full(10, 9, dtype=np.uint8), 1024)
    assert mg.table_check(one.table) == 1


def test_decode_rejects_bad_arguments_without_gpu(mg):
    """Argument checks run before any CUDA call."""
    import ctypes
    lib = mg.lib()
    dummy = ctypes.c_void_p(16)
    from multians_gb300._lib import Cfg
    c = Cfg()
    # first_state outside [L, 2L)
    rc = lib.mans_decode(dummy, 10, dummy, 10, dummy, 1024, 5, 0, dummy, 1 << 20,
                         ctypes.byref(c), None)
    assert rc == mg.Status.ERR_ARG
    # n_out == 0 is a no-op
    assert lib.mans_decode(None, 0, None, 0, None, 1024, 1024, 0, None, 0, None, None) == 0
    # aux too small
    rc = lib.mans_decode(dummy, 1000, dummy, 1000, dummy, 1024, 1024, 0, dummy, 8,
                         ctypes.byref(c), None)
    assert rc == mg.Status.ERR_AUX_SMALL


def test_table_upload_rejects_bad_tables(mg, oracle_lib):
    """mans_table_upload checks the table on the host before touching the
    device: bad tables and bad arguments fail without a GPU."""
    import ctypes
    st = oracle_lib.make_stream(seed=3, lam=0.05, n=5000, L=1024)
    bad = np.ascontiguousarray(st.table, dtype=np.uint32).copy()
    bad[3] = (bad[3] & 0x00FFFFFF) | (20 << 24)
    out = ctypes.c_void_p()
    p = bad.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
    assert mg.lib().mans_table_upload(p, 1024, ctypes.byref(out)) == mg.Status.ERR_TABLE
    assert mg.lib().mans_table_upload(p, 1, ctypes.byref(out)) == mg.Status.ERR_ARG
    assert mg.lib().mans_table_upload(None, 1024, ctypes.byref(out)) == mg.Status.ERR_ARG
    assert mg.lib().mans_aux_free(None) == 0 and mg.lib().mans_table_free(None) == 0


@pytest.mark.parametrize("L", [1024, 2048, 4096, 8192])
def test_plan_invariants(mg, L):
    """The planner's geometry over sizes and entropies: block sizes from the
    supported set, odd region lengths, walk slots within bounds, capture
    slices 16-byte multiples holding a region's expected symbols, and (for
    streams long enough to fill it) at most one wave of G-pass lanes."""
    # resident lanes of the capturing G pass (shared memory bounds them)
    lanes_capture = {1024: 152 * 2 * 256, 2048: 152 * 3 * 128, 4096: 152 * 2 * 128}
    for n_out in (10_000, 3_000_000, 64 << 20, 256 << 20, 2 << 30):
        for bps in (0.67, 1.5, 3.8, 6.0, 8.6):
            n_units = max(1, int(n_out * bps / 32))
            p = mg.plan(n_units, n_out, L)
            assert p["block_units"] in (4, 8, 16)
            assert p["region_blocks"] % 2 == 1 and p["region_blocks"] >= 8
            assert 1 <= p["walk_slots"] <= 12
            cap = p["capture_bytes"]
            assert cap % 16 == 0
            want_cap = n_units >= 16 << 20 and bps >= 2.0 and L <= 4096
            assert (cap > 0) == want_cap, (n_out, bps, L, p)
            R = p["block_units"] * p["region_blocks"]
            if cap:
                assert cap >= n_out / n_units * R   # a region's symbols fit
                nblk = n_units // p["block_units"] + 1
                nreg = -(-nblk // p["region_blocks"])
                if R < 4096:   # not clamped by the longest region
                    assert nreg <= lanes_capture[L], (nreg, p)
            assert mg.aux_size(n_units, p) > 0


def test_sync_stats_argument_checks(mg):
    """mans_sync_stats_get refuses bad arguments and a workspace smaller
    than the plan's before it touches the device (no GPU needed)."""
    lib = mg.lib()
    from multians_gb300._lib import SyncStats, Cfg
    import ctypes
    out = SyncStats()
    n_units, n_out, L = 50_000, 260_000, 1024
    plan = Cfg(**mg.plan(n_units, n_out, L))
    fake = ctypes.c_void_p(0x100000)   # never dereferenced: every case fails first
    assert lib.mans_sync_stats_get(None, 1 << 30, n_units, n_out, L, ctypes.byref(plan), None,
                                   ctypes.byref(out)) == mg.Status.ERR_ARG
    assert lib.mans_sync_stats_get(fake, 1 << 30, 0, n_out, L, ctypes.byref(plan), None,
                                   ctypes.byref(out)) == mg.Status.ERR_ARG
    assert lib.mans_sync_stats_get(fake, 1 << 30, n_units, 0, L, ctypes.byref(plan), None,
                                   ctypes.byref(out)) == mg.Status.ERR_ARG
    assert lib.mans_sync_stats_get(fake, 1 << 30, n_units, n_out, 1, ctypes.byref(plan), None,
                                   ctypes.byref(out)) == mg.Status.ERR_ARG
    assert lib.mans_sync_stats_get(fake, 1 << 30, n_units, n_out, L, ctypes.byref(plan), None,
                                   None) == mg.Status.ERR_ARG
    need = mg.aux_size(n_units, mg.plan(n_units, n_out, L))
    assert lib.mans_sync_stats_get(fake, need - 256, n_units, n_out, L, ctypes.byref(plan), None,
                                   ctypes.byref(out)) == mg.Status.ERR_AUX_SMALL


def test_aux_size_max_covers_every_uncaptured_plan(mg):
    """mans_aux_size_max(n_units) is enough for the plan of any output size
    and table size without capture (what CUHDGPUDecoderMemory allocates
    before it sees the output size)."""
    for n_units in (1, 3, 17, 1000, 65_537, 1 << 20, 12_732_195, 50_339_428, 577_000_000):
        cap = mg.aux_size_max(n_units)
        for sym_per_unit in (0.03, 1.0, 3.7, 5.3, 8.4, 21.0, 48.0, 200.0):
            n_out = max(1, int(n_units * sym_per_unit))
            for L in (2, 256, 1024, 2048, 4096, 8192):
                p = mg.plan(n_units, n_out, L, {"flags": mg.DECODE_NO_CAPTURE})
                assert mg.aux_size(n_units, p) <= cap, (n_units, n_out, L, p)


def test_aux_size_max_any_covers_every_plan(mg):
    """mans_aux_size_max_any(n_units) is enough for the planner's own plan
    (symbol capture included) of any output size and table size: the
    drop-in decoder memory reserves it at allocate(), so its decode never
    needs more memory."""
    for n_units in (1, 17, 65_537, 1 << 20, 16 << 20, 17_000_000, 50_339_428, 200_000_000):
        cap = mg.aux_size_max_any(n_units)
        assert cap >= mg.aux_size_max(n_units)
        for sym_per_unit in (0.03, 1.0, 2.0, 3.7, 5.3, 8.4, 12.0, 15.9, 16.0, 21.0, 200.0):
            n_out = max(1, int(n_units * sym_per_unit))
            for L in (2, 256, 512, 1024, 2048, 4096, 8192):
                p = mg.plan(n_units, n_out, L)
                assert mg.aux_size(n_units, p) <= cap, (n_units, n_out, L, p)


def _bad_decode_args():
    a = 0x100000   # 16-byte aligned placeholder addresses, never dereferenced
    good = dict(units=a, n_units=1000, out=a, n_out=5000, table=a, L=1024, first_state=1500,
                first_bit=7, aux=a, aux_bytes=1 << 30)
    cases = {
        "misaligned units": {"units": a + 4},
        "null units": {"units": None},
        "null out": {"out": None},
        "null table": {"table": None},
        "null aux": {"aux": None},
        "no units": {"n_units": 0},
        "too many units": {"n_units": 1 << 32},
        "L = 1": {"L": 1, "first_state": 1},
        "L above 8192": {"L": 16384, "first_state": 16384},
        "first_state below L": {"first_state": 1023},
        "first_state at 2L": {"first_state": 2048},
        "first_bit above 32": {"first_bit": 33},
    }
    return [(name, {**good, **bad}) for name, bad in cases.items()]


@pytest.mark.parametrize("name,args", _bad_decode_args(), ids=[c[0] for c in _bad_decode_args()])
def test_decode_entry_points_reject_bad_arguments(mg, name, args):
    """Every malformed argument is refused with MANS_ERR_ARG before any
    CUDA call, by the asynchronous and the synchronous decode."""
    import ctypes
    lib = mg.lib()
    v = ctypes.c_void_p
    pos = (v(args["units"]), args["n_units"], v(args["out"]), args["n_out"], v(args["table"]),
           args["L"], args["first_state"], args["first_bit"], v(args["aux"]), args["aux_bytes"],
           None, None)
    assert lib.mans_decode(*pos) == mg.Status.ERR_ARG, name
    st = ctypes.c_uint32(0)
    assert lib.mans_decode_sync(*pos, ctypes.byref(st)) == mg.Status.ERR_ARG, name


def test_start_offset_flag_widens_first_bit(mg):
    """MANS_DECODE_START_OFFSET: first_bit is a start offset below 128 bits;
    without the flag the reference's 0..32 range stands.  Refusals come
    before any CUDA call (placeholder addresses are never dereferenced)."""
    import ctypes
    lib = mg.lib()
    a = 0x100000
    v = ctypes.c_void_p
    st = ctypes.c_uint32(0)

    def call(first_bit, flags):
        cfg = mg._lib.Cfg(flags=flags)
        return lib.mans_decode_sync(v(a), 1000, v(a), 5000, v(a), 1024, 1500, first_bit, None,
                                    1 << 30, ctypes.byref(cfg), None, ctypes.byref(st))
    # a null workspace fails the checks either way; the first_bit bound is
    # what differs: 33 and 127 pass it only with the flag, 128 never
    for fb, flags in ((33, 0), (127, 0), (128, mg.DECODE_START_OFFSET)):
        assert call(fb, flags) == mg.Status.ERR_ARG, (fb, flags)
    plan = mg._lib.Cfg(flags=mg.DECODE_START_OFFSET)
    assert lib.mans_decode(v(a + 4), 1000, v(a), 5000, v(a), 1024, 1500, 100, v(a), 1 << 30,
                           ctypes.byref(plan), None) == mg.Status.ERR_ARG   # misaligned units


def test_trajectory_query_refuses_bad_arguments(mg):
    import ctypes

    from multians_gb300 import shard
    be = shard.GpuBackend.__new__(shard.GpuBackend)   # signatures only
    lib = mg.lib()
    f = lib.mans_trajectory_query
    f.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_uint32,
                  ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_size_t,
                  ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_uint64),
                  ctypes.c_uint32, ctypes.POINTER(shard.Point), ctypes.c_void_p,
                  ctypes.POINTER(ctypes.c_uint32)]
    f.restype = ctypes.c_int
    g = lib.mans_trajectory_aux_size
    g.argtypes = [ctypes.c_size_t, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_uint32]
    g.restype = ctypes.c_size_t
    assert g(1000, 5000, 1024, 0) == 0 and g(1000, 5000, 1024, 1025) == 0
    need = g(1000, 5000, 1024, 4)
    assert need > mg.aux_size_max(1000)
    a = 0x100000
    q = (ctypes.c_uint64 * 4)(0, 32, 64, 96)
    out = (shard.Point * 4)()
    st = ctypes.c_uint32(0)
    v = ctypes.c_void_p
    base = [v(a), 1000, v(a), 1024, 1500, 32, 0, 5000, v(a), need, q, 4, out, None,
            ctypes.byref(st)]
    cases = {0: v(a + 4), 8: v(None), 9: 100, 11: 0}   # misaligned units, no aux, small aux, nq 0
    for i, bad in cases.items():
        args = list(base)
        args[i] = bad
        assert f(*args) == mg.Status.ERR_ARG, i
    args = list(base)
    args[5] = 33   # first_bit past 32 without the start-offset flag
    assert f(*args) == mg.Status.ERR_ARG
