"""GPU parity of symbol capture: the sync passes keep the symbols they decode
and the final pass copies the blocks whose owning trajectory was captured.
Every case must give the oracle's output byte for byte, with capture on, off,
forced on where the planner would not choose it, and with capture slices too
small to hold a region (a mix of copied and decoded blocks in one warp)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LAMBDAS = [0.005, 0.05, 0.2, 1.0, 2.0]


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).to("cuda")


def _decode(mg, st, cfg, n_out=None, source_order=False):
    import torch
    n_out = st.n if n_out is None else n_out
    out = torch.full((max(1, n_out) + 16,), 0xAB, dtype=torch.uint8, device="cuda")
    full = mg.plan(st.n_units, n_out, st.L, cfg)
    aux = torch.empty(mg.aux_size(st.n_units, full), dtype=torch.uint8, device="cuda")
    got = mg.decode(_dev(st.units), st.n_units, n_out, _dev(st.table), st.first_state,
                    st.first_bit, L=st.L, out=out, aux=aux, cfg=cfg,
                    source_order=source_order)
    tail = out[n_out:].cpu().numpy()
    assert (tail == 0xAB).all(), "wrote past n_out"
    return got.cpu().numpy(), full


@pytest.mark.parametrize("lam", LAMBDAS)
def test_capture_on_off_forced(mg, oracle_lib, lam):
    O = oracle_lib
    st = O.make_stream(seed=7100 + int(lam * 1000), lam=lam, n=400_000, L=1024)
    want = O.decode_seq(st)
    auto, plan = _decode(mg, st, {})
    off, p_off = _decode(mg, st, {"flags": mg.DECODE_NO_CAPTURE})
    forced, p_forced = _decode(mg, st, {"capture_bytes": 4096})
    assert p_off["capture_bytes"] == 0 and p_forced["capture_bytes"] == 4096
    assert plan["capture_bytes"] == 0   # too short for capture by default
    assert np.array_equal(auto, want)
    assert np.array_equal(off, want)
    assert np.array_equal(forced, want)


@pytest.mark.parametrize("cap", [16, 48, 160, 640])
def test_small_slices_mix_copy_and_decode(mg, oracle_lib, cap):
    """Slices that hold only the first blocks of a region: later blocks are
    decoded, so warps mix both kinds of lanes."""
    O = oracle_lib
    st = O.make_stream(seed=7200 + cap, lam=0.05, n=300_000, L=1024)
    want = O.decode_seq(st)
    got, _ = _decode(mg, st, {"capture_bytes": cap})
    assert np.array_equal(got, want)
    rev, _ = _decode(mg, st, {"capture_bytes": cap}, source_order=True)
    assert np.array_equal(rev, st.symbols)


@pytest.mark.parametrize("cfg", [
    {"block_units": 4, "region_blocks": 1, "walk_slots": 8},
    {"block_units": 4, "region_blocks": 4, "walk_slots": 8},
    {"block_units": 8, "region_blocks": 3, "walk_slots": 12},
    {"block_units": 16, "region_blocks": 9, "walk_slots": 4},
])
@pytest.mark.parametrize("lam", [0.05, 0.2])
def test_capture_geometries(mg, oracle_lib, cfg, lam):
    """Short regions: merge walks cross whole regions, blocks are owned at
    walk depth >= 2 and follow other regions' trajectories."""
    O = oracle_lib
    st = O.make_stream(seed=7300 + cfg["region_blocks"] * 10 + int(lam * 100), lam=lam,
                       n=250_000, L=1024)
    want = O.decode_seq(st)
    cfg = dict(cfg, capture_bytes=2048)
    got, p = _decode(mg, st, cfg)
    assert p["capture_bytes"] == 2048
    assert np.array_equal(got, want)
    rev, _ = _decode(mg, st, cfg, source_order=True)
    assert np.array_equal(rev, st.symbols)


@pytest.mark.parametrize("lam", [0.05, 0.2])
@pytest.mark.parametrize("shift", [0, 1, 5, 13])
def test_capture_source_order_phases(mg, oracle_lib, lam, shift):
    """Output buffers at every 16-byte phase: the segment copies write the
    staging buffer at that phase, forwards and reversed."""
    import torch
    O = oracle_lib
    st = O.make_stream(seed=7400 + shift, lam=lam, n=200_000, L=1024)
    for src_order in (False, True):
        base = torch.full((st.n + 64,), 0xAB, dtype=torch.uint8, device="cuda")
        out = base[shift:shift + st.n]
        mg.decode(_dev(st.units), st.n_units, st.n, _dev(st.table), st.first_state,
                  st.first_bit, L=st.L, out=out, source_order=src_order,
                  cfg={"capture_bytes": 4096})
        got = out.cpu().numpy()
        assert np.array_equal(got if src_order else got[::-1], st.symbols)
        b = base.cpu().numpy()
        assert (b[:shift] == 0xAB).all() and (b[shift + st.n:] == 0xAB).all()


@pytest.mark.parametrize("short", [1, 77, 4096, 150_001])
def test_capture_short_output(mg, oracle_lib, short):
    """Only the first n_out decoded symbols are written, captured or not."""
    O = oracle_lib
    st = O.make_stream(seed=7500 + short, lam=0.05, n=200_000, L=1024)
    want = O.decode_seq(st)[:short]
    got, p = _decode(mg, st, {"capture_bytes": 8192}, n_out=short)
    assert np.array_equal(got, want)


def test_capture_tiny_streams(mg, oracle_lib):
    O = oracle_lib
    for n in (1, 2, 3, 31, 32, 33, 100, 1000, 4097):
        st = O.make_stream(seed=7600 + n, lam=0.05, n=n, L=1024)
        got, _ = _decode(mg, st, {"capture_bytes": 256})
        assert np.array_equal(got[::-1], st.symbols), n


def test_batch_mixes_capture(mg, oracle_lib):
    """One batch with capturing streams (forced, at every entropy and at
    L = 4096) and one kept out of capture by its flags."""
    import torch

    from multians_gb300 import batch
    O = oracle_lib
    sts = [O.make_stream(seed=7700 + i, lam=lam, n=n, L=L)
           for i, (lam, n, L) in enumerate([(0.05, 200_000, 1024), (2.0, 150_000, 1024),
                                            (0.05, 120_000, 4096), (0.2, 90_000, 1024),
                                            (0.005, 3_000, 1024), (0.05, 180_000, 1024)])]
    keep, descs = [], []
    for i, st in enumerate(sts):
        u, t = _dev(st.units), _dev(st.table)
        o = torch.full((st.n,), 0xAB, dtype=torch.uint8, device="cuda")
        keep.append((u, t, o))
        descs.append(batch.desc(u, st.n_units, o, st.n, t, st.L, st.first_state, st.first_bit,
                                source_order=bool(i % 2), capture=(i != 5)))
    b = batch.Batch(descs, hint={"capture_bytes": 4096})
    s = torch.cuda.current_stream()
    b.decode(s)
    acc, per = b.status(s)
    assert acc == 0 and per == [0] * len(sts), per
    for i, (st, (_, _, o)) in enumerate(zip(sts, keep)):
        got = o.cpu().numpy()
        assert np.array_equal(got if i % 2 else got[::-1], st.symbols), i
    b.close()


def test_default_capture_large_stream(mg):
    """A stream long enough for the planner to capture on its own (16 Mi
    units and more): the round trip through the default path, both orders."""
    from multians_gb300 import host
    st = host.make_stream(7800, 0.05, 96 << 20, 1024)
    p = mg.plan(st.n_units, st.n, st.L)
    assert st.n_units >= 16 << 20 and p["capture_bytes"] > 0
    got = mg.decode(_dev(st.units), st.n_units, st.n, _dev(st.table), st.first_state,
                    st.first_bit, L=st.L).cpu().numpy()
    assert np.array_equal(got[::-1], st.symbols)
    got = mg.decode(_dev(st.units), st.n_units, st.n, _dev(st.table), st.first_state,
                    st.first_bit, L=st.L, source_order=True).cpu().numpy()
    assert np.array_equal(got, st.symbols)
    # a workspace with no room for the capture the planner picks (the size
    # of the plan without it) still decodes: without capture
    import torch

    from multians_gb300.decoder import aux_status, decode_async
    small = mg.aux_size(st.n_units, mg.plan(st.n_units, st.n, st.L,
                                             {"flags": mg.DECODE_NO_CAPTURE}))
    assert small < mg.aux_size(st.n_units, p) and small <= mg.aux_size_max(st.n_units)
    aux = torch.empty(small, dtype=torch.uint8, device="cuda")
    out = torch.full((st.n,), 0xAB, dtype=torch.uint8, device="cuda")
    decode_async(_dev(st.units), st.n_units, out, st.n, _dev(st.table), st.L, st.first_state,
                 st.first_bit, aux, {})
    assert aux_status(aux) == 0
    assert np.array_equal(out.cpu().numpy()[::-1], st.symbols)


def test_capture_single_symbol_and_bad_table(mg, oracle_lib):
    """With capture asked for, a single-symbol table still fills the output
    (the copy pass does it) and a bad table is still rejected."""
    import torch
    O = oracle_lib
    sym = np.full(50_000, 17, dtype=np.uint8)
    st = O.encode(sym, 1024)
    assert mg.table_check(st.table) == 1
    got, p = _decode(mg, st, {"capture_bytes": 1024})
    assert p["capture_bytes"] == 1024 and np.array_equal(got, sym)
    st = O.make_stream(seed=7900, lam=0.05, n=100_000, L=1024)
    bad = st.table.copy()
    bad[5] = (bad[5] & 0x00ffffff) | (15 << 24)
    out = torch.empty(st.n, dtype=torch.uint8, device="cuda")
    with pytest.raises(mg.MansError):
        mg.decode(_dev(st.units), st.n_units, st.n, _dev(bad), st.first_state, st.first_bit,
                  L=st.L, out=out, cfg={"capture_bytes": 4096})


@pytest.mark.parametrize("lam", [0.05, 0.5])
def test_capture_forced_at_8192_states(mg, oracle_lib, lam):
    """The largest table (64 KB in shared memory) with capture forced on:
    the capturing G pass, walks and fallback still fit and agree."""
    O = oracle_lib
    st = O.make_stream(seed=7950 + int(lam * 10), lam=lam, n=250_000, L=8192)
    want = O.decode_seq(st)
    got, p = _decode(mg, st, {"capture_bytes": 8192})
    assert p["capture_bytes"] == 8192
    assert np.array_equal(got, want)
    rev, _ = _decode(mg, st, {"capture_bytes": 8192}, source_order=True)
    assert np.array_equal(rev, st.symbols)
