"""GPU parity of the plain decode path: the CUDA decoder, called through the
C ABI, against the C oracle and the source symbols, byte for byte."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LAMBDAS = [0.005, 0.05, 0.2, 1.0, 2.0]


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).to("cuda")


def _gpu_decode(mg, st, n_out=None, cfg=None, sync=True):
    import torch
    n_out = st.n if n_out is None else n_out
    units = _dev(st.units)
    table = _dev(st.table)
    out = torch.full((max(1, n_out),), 0xAB, dtype=torch.uint8, device="cuda")
    if cfg is None or sync:
        mg.decode(units, st.n_units, n_out, table, st.first_state, st.first_bit, L=st.L, out=out,
                  cfg=cfg)
    else:
        from multians_gb300.decoder import decode_async, aux_status
        full = mg.plan(st.n_units, n_out, st.L, cfg)
        aux = torch.empty(mg.aux_size(st.n_units, full), dtype=torch.uint8, device="cuda")
        decode_async(units, st.n_units, out, n_out, table, st.L, st.first_state,
                     st.first_bit, aux, full)
        s = aux_status(aux)
        assert s == 0, f"device status 0x{s:x}"
    return out[:n_out].cpu().numpy()


@pytest.mark.parametrize("L", [1024, 4096, 8192])
@pytest.mark.parametrize("lam", LAMBDAS)
def test_roundtrip_vs_oracle(mg, oracle_lib, L, lam):
    """Up to L = 8192, the largest table the shared-memory decoder holds."""
    O = oracle_lib
    st = O.make_stream(seed=1000 + int(lam * 1000) + L, lam=lam, n=300_000, L=L)
    got = _gpu_decode(mg, st)
    want = O.decode_seq(st)
    assert np.array_equal(got, want)
    assert np.array_equal(got[::-1], st.symbols)


@pytest.mark.parametrize("n", [1, 2, 3, 7, 31, 32, 33, 100, 1000, 4097])
def test_tiny_streams(mg, oracle_lib, n):
    O = oracle_lib
    for lam in (0.05, 2.0):
        st = O.make_stream(seed=n * 7 + 1, lam=lam, n=n, L=1024)
        got = _gpu_decode(mg, st)
        assert np.array_equal(got[::-1], st.symbols), (n, lam)


@pytest.mark.parametrize("cfg", [
    {"block_units": 4, "region_blocks": 1, "walk_slots": 8},
    {"block_units": 4, "region_blocks": 4, "walk_slots": 8},
    {"block_units": 8, "region_blocks": 8, "walk_slots": 8},
    {"block_units": 16, "region_blocks": 64, "walk_slots": 2},
    {"block_units": 32, "region_blocks": 16, "walk_slots": 4, "threads": 64},
])
def test_geometries(mg, oracle_lib, cfg):
    """Short regions force walks that cross several regions."""
    O = oracle_lib
    st = O.make_stream(seed=77, lam=0.2, n=60_000, L=1024)
    got = _gpu_decode(mg, st, cfg=cfg)
    assert np.array_equal(got[::-1], st.symbols)


@pytest.mark.parametrize("L", [4096, 8192])
def test_long_blocks_at_low_bits_per_symbol(mg, oracle_lib, L):
    """16-unit blocks at 1.5 bits per symbol ask the final pass for large
    staging buffers; the decoder caps them to what fits its shared memory
    (a warp whose range does not fit writes it directly) instead of failing
    the launch."""
    O = oracle_lib
    st = O.make_stream(seed=L + 15, lam=1.0, n=400_000, L=L)
    for cfg in ({"block_units": 16, "flags": mg.DECODE_NO_CAPTURE},
                {"block_units": 16, "region_blocks": 301, "flags": mg.DECODE_NO_CAPTURE}):
        got = _gpu_decode(mg, st, cfg=cfg)
        assert np.array_equal(got[::-1], st.symbols), cfg


@pytest.mark.parametrize("L,lam,cfg", [
    (4096, 0.05, {"block_units": 8, "region_blocks": 9, "walk_slots": 12}),
    (4096, 0.5, {"block_units": 4, "region_blocks": 9, "walk_slots": 12}),
    (1024, 0.005, {"block_units": 16, "region_blocks": 9, "walk_slots": 6}),
    (1024, 2.0, {"block_units": 4, "region_blocks": 9, "walk_slots": 12}),
])
def test_walks_across_regions(mg, oracle_lib, L, lam, cfg):
    """Sync distances of several regions: merge walks run on with two
    cursors, which follow the trajectories of the regions they cross."""
    O = oracle_lib
    st = O.make_stream(seed=4242 + L, lam=lam, n=300_000, L=L)
    got = _gpu_decode(mg, st, cfg=cfg)
    assert np.array_equal(got[::-1], st.symbols)


def test_async_geometry_clean(mg, oracle_lib):
    """Long regions with spare slots: one asynchronous pass, status clean."""
    O = oracle_lib
    st = O.make_stream(seed=78, lam=0.05, n=400_000, L=1024)
    got = _gpu_decode(mg, st, cfg={"block_units": 16, "region_blocks": 64, "walk_slots": 4},
                      sync=False)
    assert np.array_equal(got[::-1], st.symbols)


def test_overflow_replans(mg, oracle_lib):
    """Regions far shorter than the sync distance with few slots overflow;
    the synchronous entry point re-plans and still decodes exactly."""
    import torch
    import ctypes
    O = oracle_lib
    st = O.make_stream(seed=5, lam=0.2, n=200_000, L=4096)
    from multians_gb300.decoder import decode_async, aux_status
    units = _dev(st.units)
    table = _dev(st.table)
    cfg = mg.plan(st.n_units, st.n, st.L, {"block_units": 4, "region_blocks": 1, "walk_slots": 1})
    aux = torch.empty(mg.aux_size_max(st.n_units), dtype=torch.uint8, device="cuda")
    out = torch.empty(st.n, dtype=torch.uint8, device="cuda")
    decode_async(units, st.n_units, out, st.n, table, st.L, st.first_state, st.first_bit, aux, cfg)
    s = aux_status(aux)
    assert s & mg.DEV_SYNC_OVERFLOW
    got = mg.decode(units, st.n_units, st.n, table, st.first_state, st.first_bit, L=st.L, aux=aux)
    assert np.array_equal(got.cpu().numpy()[::-1], st.symbols)


@pytest.mark.parametrize("short", [1, 12_345, 49_000, 49_963, 49_999])
def test_short_output_is_bounded(mg, oracle_lib, short):
    """An output size below the symbol count writes exactly that prefix,
    also when the cut falls among the last blocks of the stream."""
    O = oracle_lib
    st = O.make_stream(seed=9, lam=0.05, n=50_000, L=1024)
    want = O.decode_seq(st)
    got = _gpu_decode(mg, st, n_out=short)
    assert np.array_equal(got, want[:short])


def test_first_bit_zero(mg, oracle_lib):
    """Streams whose final encoder unit holds no data bit (first_bit = 0)."""
    O = oracle_lib
    found = 0
    for seed in range(400):
        st = O.make_stream(seed=seed, lam=1.0, n=997 + seed, L=1024)
        if st.first_bit != 0:
            continue
        found += 1
        got = _gpu_decode(mg, st)
        assert np.array_equal(got[::-1], st.symbols), seed
        if found >= 3:
            break
    assert found > 0


def test_multicore_port_agrees(mg, oracle_lib):
    O = oracle_lib
    st = O.make_stream(seed=31, lam=0.05, n=1 << 20, L=1024)
    mc, _ = O.multicore_decode(st, S=4, T=8)
    got = _gpu_decode(mg, st)
    assert np.array_equal(got, mc)


def test_single_symbol_stream(mg, oracle_lib):
    """A constant input builds a single-symbol table (every entry a zero-bit
    self loop); the decoder fills the output with that symbol."""
    O = oracle_lib
    sym = np.full(5000, 17, dtype=np.uint8)
    st = O.encode(sym, 1024)
    assert mg.table_check(st.table) == 1
    got = _gpu_decode(mg, st)
    assert np.array_equal(got, sym)


def test_bad_table_rejected(mg, oracle_lib):
    O = oracle_lib
    st = O.make_stream(seed=3, lam=0.05, n=10_000, L=1024)
    bad = st.table.copy()
    bad[5] = (bad[5] & 0x00ffffff) | (15 << 24)  # next state leaves [L, 2L)
    assert mg.table_check(bad) == -1
    import torch
    out = torch.empty(st.n, dtype=torch.uint8, device="cuda")
    with pytest.raises(mg.MansError):
        mg.decode(_dev(st.units), st.n_units, st.n, _dev(bad), st.first_state, st.first_bit,
                  L=st.L, out=out)


@pytest.mark.parametrize("L,lam", [(1024, 0.05), (1024, 2.0), (4096, 0.005), (4096, 1.0)])
@pytest.mark.parametrize("shift", [0, 3, 13])
def test_source_order_output(mg, oracle_lib, L, lam, shift):
    """MANS_DECODE_SOURCE_ORDER: the final pass writes the i-th decoded
    symbol to out[n_out - 1 - i], at any output alignment; full decodes give
    the source, short ones the mirrored prefix."""
    import torch
    O = oracle_lib
    st = O.make_stream(seed=300 + L + int(lam * 100), lam=lam, n=200_003, L=L)
    units, table = _dev(st.units), _dev(st.table)
    big = torch.full((st.n + 64,), 0xCD, dtype=torch.uint8, device="cuda")
    out = big[shift: shift + st.n]
    mg.decode(units, st.n_units, st.n, table, st.first_state, st.first_bit, L=L, out=out,
              source_order=True)
    assert np.array_equal(out.cpu().numpy(), st.symbols)
    b = big.cpu().numpy()
    assert (b[:shift] == 0xCD).all() and (b[shift + st.n:] == 0xCD).all()
    want = O.decode_seq(st)
    for short in (1, 4097, st.n - 7):
        o2 = torch.full((short,), 0xCD, dtype=torch.uint8, device="cuda")
        mg.decode(units, st.n_units, short, table, st.first_state, st.first_bit, L=L, out=o2,
                  source_order=True)
        assert np.array_equal(o2.cpu().numpy(), want[:short][::-1]), short
