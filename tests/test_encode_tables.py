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
