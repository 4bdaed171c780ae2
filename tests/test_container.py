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
