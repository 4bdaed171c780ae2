"""Multi-table streams on the GPU (multians_gb300/segments.py): source
segments each encoded with their own table into one bitstream, the state
carried across segment ends (the oracle's mo_encode_segments), decoded with
one guessed-start pass per segment, the chained start states and one
batched decode.  The output equals the oracle's sequential multi-table
decode and the source, byte for byte."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).to("cuda")


def _run(O, segs, L, prefix=None):
    from multians_gb300 import segments
    ss = O.encode_segments(segs, L)
    got, info = segments.decode_segments(_dev(ss.units), ss.n_units, ss.first_state,
                                         ss.first_bit, L, ss.tables, ss.counts, ss.starts,
                                         prefix_units=prefix)
    got = got.cpu().numpy()
    assert np.array_equal(got, O.decode_segments_seq(ss))
    assert np.array_equal(got[::-1], ss.symbols)
    return info


@pytest.mark.parametrize("L", [1024, 4096])
def test_three_tables(mg, oracle_lib, L):
    O = oracle_lib
    segs = [O.gen_symbols(1, 0.05, 300_000), O.gen_symbols(2, 1.0, 200_000),
            O.gen_symbols(3, 0.2, 250_000)]
    _run(O, segs, L)


def test_many_short_segments(mg, oracle_lib):
    O = oracle_lib
    rng = np.random.default_rng(5)
    segs = [O.gen_symbols(100 + i, float(rng.uniform(0.01, 2.0)), int(rng.integers(1, 20_000)))
            for i in range(24)]
    _run(O, segs, 1024)


def test_low_entropy_segment_and_forced_full_queries(mg, oracle_lib):
    """A nearly constant segment (two symbols, mostly zero-bit codewords, so
    segments end on zero-bit codewords at the next one's start bit) between
    two others; a one-unit prefix makes the guessed and true starts miss each
    other, so the exact full-segment query runs."""
    O = oracle_lib
    rng = np.random.default_rng(3)
    flat = np.where(rng.random(5000) < 0.998, 9, 10).astype(np.uint8)
    segs = [O.gen_symbols(7, 0.05, 100_000), flat, O.gen_symbols(8, 0.5, 100_000),
            O.gen_symbols(9, 0.05, 50_000)]
    info = _run(O, segs, 1024, prefix=1)
    assert info["full_segment_queries"] >= 1


def test_single_symbol_table_before_the_last_segment_is_refused(mg, oracle_lib):
    from multians_gb300 import segments
    O = oracle_lib
    ss = O.encode_segments([O.gen_symbols(1, 0.05, 20_000), O.gen_symbols(2, 0.05, 20_000)], 1024)
    tables = list(ss.tables)
    tables[0] = np.full(1024, 0, np.uint32) | (np.arange(1024, 2048, dtype=np.uint32)) | (7 << 16)
    assert mg.table_check(tables[0]) == 1
    with pytest.raises(mg.MansError):
        segments.decode_segments(_dev(ss.units), ss.n_units, ss.first_state, ss.first_bit,
                                 1024, tables, ss.counts, ss.starts)


def test_one_segment_is_a_plain_stream(mg, oracle_lib):
    """A single segment is an ordinary stream: the segment decoder gives the
    plain decoder's output."""
    import torch
    from multians_gb300 import segments
    O = oracle_lib
    sym = O.gen_symbols(31, 0.05, 200_000)
    st = O.encode(sym, 1024)
    got, info = segments.decode_segments(_dev(st.units), st.n_units, st.first_state,
                                         st.first_bit, 1024, [st.table], [st.n],
                                         [32 - st.first_bit])
    plain = mg.decode(_dev(st.units), st.n_units, st.n, _dev(st.table), st.first_state,
                      st.first_bit, L=1024)
    assert torch.equal(got, plain)
    assert np.array_equal(got.cpu().numpy()[::-1], sym)
