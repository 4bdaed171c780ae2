"""The oracle's multi-table encoder (mo_encode_segments): with one segment
it is the plain encoder (the reference's ANSEncoder restated), bit for bit;
with several it round-trips through the sequential multi-table decode."""
import numpy as np


def test_one_segment_is_the_plain_encoder(oracle_lib):
    O = oracle_lib
    for seed, lam, L in ((1, 0.05, 1024), (2, 2.0, 4096), (3, 0.005, 1024)):
        sym = O.gen_symbols(seed, lam, 50_000)
        a = O.encode(sym, L)
        b = O.encode_segments([sym], L)
        assert (a.n_units, a.first_bit, a.first_state) == (b.n_units, b.first_bit, b.first_state)
        assert np.array_equal(a.units[: a.n_units], b.units[: b.n_units])
        assert np.array_equal(a.table, b.tables[0])
        assert b.starts == [32 - b.first_bit]


def test_segments_round_trip(oracle_lib):
    O = oracle_lib
    segs = [O.gen_symbols(11, 0.3, 7000), O.gen_symbols(12, 1.5, 9000), O.gen_symbols(13, 0.02, 3)]
    ss = O.encode_segments(segs, 2048)
    assert ss.counts == [3, 9000, 7000]
    assert ss.starts[0] == 32 - ss.first_bit and ss.starts == sorted(ss.starts)
    assert np.array_equal(O.decode_segments_seq(ss)[::-1], np.concatenate(segs))
