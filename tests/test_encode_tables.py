"""CPU check of the GPU encoder's compact table: for every present byte s
and state X in [L, 2L), k = (X + delta_s) >> 16, the code X mod 2^k and
next[base_s + (X >> k)] reproduce the reference encoder table entry
(next_state, code_sequence, code_length) the oracle builds, and the decoder
table from the byte histogram equals the one built from the buffer."""
import numpy as np
import pytest


@pytest.mark.parametrize("L,lam", [(1024, 0.05), (1024, 2.0), (4096, 0.005), (4096, 0.7),
                                   (256, 0.3), (8192, 0.05)])
def test_compact_table_matches_reference_table(mg, oracle_lib, L, lam):
    from multians_gb300 import encode
    O = oracle_lib
    st = O.make_stream(seed=int(lam * 1000) + L, lam=lam, n=200_000, L=L)
    hist = np.bincount(st.symbols, minlength=256).astype(np.uint64)
    dec, blob = encode.tables_from_histogram(hist, L)
    assert np.array_equal(dec, st.table)
    enc = O.build_tables(st.symbols, L)[0].reshape(256, L, 4)   # next, code, len, sym
    delta = blob[0:512:2].astype(np.uint64)
    base = blob[1:512:2].astype(np.uint64)
    nxt = blob[512:].view(np.uint16)
    X = np.arange(L, 2 * L, dtype=np.uint64)
    for s in np.nonzero(hist)[0]:
        k = ((X + delta[s]) & 0xFFFFFFFF) >> 16
        code = X & ((np.uint64(1) << k) - np.uint64(1))
        idx = (base[s] + (X >> k)) & 0xFFFFFFFF
        assert np.array_equal(k, enc[s, :, 2].astype(np.uint64)), s
        assert np.array_equal(code, enc[s, :, 1].astype(np.uint64)), s
        assert np.array_equal(nxt[idx.astype(np.int64)], enc[s, :, 0]), s


@pytest.mark.parametrize("bad", [
    {"sym": None}, {"sym": 0x100008}, {"blob": None}, {"blob": 0x200002}, {"units": None},
    {"aux": None}, {"n": 0}, {"L": 1}, {"L": 1000}, {"L": 16384},
    {"aux_bytes": 16}, {"cap_units": 1}])
def test_encode_refuses_bad_arguments(mg, bad):
    """mans_encode refuses malformed arguments (MANS_ERR_ARG) and short
    workspaces or unit buffers (MANS_ERR_AUX_SMALL) before any device work."""
    import ctypes
    from multians_gb300 import encode
    lib = encode._sig()
    vp = ctypes.c_void_p
    n, L = 100_000, 1024
    a = dict(sym=0x100000, blob=0x200000, units=0x300000, aux=0x400000, n=n, L=L,
             aux_bytes=1 << 30, cap_units=lib.mans_encode_max_units(n, L))
    a.update(bad)
    rc = lib.mans_encode(vp(a["sym"]), a["n"], vp(a["blob"]), a["L"], vp(a["units"]),
                         a["cap_units"], vp(a["aux"]), a["aux_bytes"], 0, None)
    want = mg.Status.ERR_AUX_SMALL if {"aux_bytes", "cap_units"} & set(bad) else \
        mg.Status.ERR_ARG
    assert rc == want, (bad, rc)
