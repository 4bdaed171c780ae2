"""CPU tests of the stream container: pack / parse round trip, the units
and table where the header says, corrupt or short buffers rejected."""
import numpy as np
import pytest


def test_container_roundtrip(mg):
    from multians_gb300 import container, host
    st = host.make_stream(5, 0.3, 10_000, 1024)
    buf = container.pack_encoded(st)
    info = container.parse(buf)
    assert (info.n_symbols, info.n_units, info.L) == (st.n, st.n_units, 1024)
    assert (info.first_state, info.first_bit) == (st.first_state, st.first_bit)
    assert info.units_offset % 16 == 0
    t = buf[info.table_offset: info.table_offset + 4 * info.L].view(np.uint32)
    u = buf[info.units_offset: info.units_offset + 4 * info.n_units].view(np.uint32)
    assert np.array_equal(t, st.table) and np.array_equal(u, st.units[: st.n_units])


def test_container_rejects_damage(mg):
    from multians_gb300 import container, host
    st = host.make_stream(6, 0.05, 5_000, 4096)
    buf = container.pack_encoded(st)
    for pos in (0, 9, 17, 33, 50):
        bad = buf.copy()
        bad[pos] ^= 0x40
        with pytest.raises(mg.MansError):
            container.parse(bad)
    with pytest.raises(mg.MansError):
        container.parse(buf[: len(buf) - 4])     # units cut short
    with pytest.raises(mg.MansError):
        container.parse(buf[:40])


def test_container_write_into_caller_buffer(mg):
    """Packing into a caller's buffer writes the same bytes when it is large
    enough and refuses (no write past its end) when it is not."""
    from multians_gb300 import container, host
    st = host.make_stream(7, 0.2, 3_000, 1024)
    ref = container.pack_encoded(st)
    out = np.full(ref.size + 32, 0xA5, dtype=np.uint8)
    container.pack_encoded(st, out=out[: ref.size])
    assert np.array_equal(out[: ref.size], ref)
    assert np.all(out[ref.size:] == 0xA5)
    short = np.full(ref.size + 32, 0x5A, dtype=np.uint8)
    with pytest.raises(mg.MansError):
        container.pack_encoded(st, out=short[: ref.size - 4])
    assert np.all(short == 0x5A)


def test_container_write_rejects_bad_fields(mg):
    from multians_gb300 import container, host
    st = host.make_stream(8, 0.05, 2_000, 1024)
    args = dict(units=st.units, n_units=st.n_units, n_symbols=st.n, table=st.table,
                first_state=st.first_state, first_bit=st.first_bit)
    for bad in ({"first_state": 1023}, {"first_state": 2048}, {"first_bit": 33},
                {"table": st.table[:1]}, {"table": np.zeros(8193, np.uint32)}):
        with pytest.raises(mg.MansError):
            container.pack(**{**args, **bad})
    with pytest.raises(ValueError):
        container.pack(**{**args, "n_units": st.units.size + 1})
