"""GPU parity of the batched path: many uneven streams, each with its own
table, decoded in one launch of each kernel (direct and as a CUDA graph),
each output byte-identical to its source and to the plain decoder."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _streams(host, specs):
    import torch
    out = []
    for seed, lam, n, L in specs:
        st = host.make_stream(seed, lam, n, L)
        units = torch.from_numpy(st.units.view(np.int32)).cuda()
        table = torch.from_numpy(st.table.view(np.int32)).cuda()
        dst = torch.full((max(1, n),), 0xCD, dtype=torch.uint8, device="cuda")
        out.append((st, units, table, dst))
    return out


def _descs(batch, streams):
    return [batch.desc(u, st.n_units, o, st.n, t, st.L, st.first_state, st.first_bit)
            for st, u, t, o in streams]


def test_batch_uneven_streams_direct_and_graph(mg):
    import torch

    from multians_gb300 import batch, host
    rng = np.random.default_rng(7)
    specs = []
    for i in range(60):
        n = int(np.exp(rng.uniform(np.log(10), np.log(400_000))))
        lam = float(rng.uniform(0.01, 2.0))
        L = (1024, 4096, 8192)[i % 3]   # shared tables of 8, 32 and 64 KB in one batch
        specs.append((1000 + i, lam, n, L))
    specs += [(5, 0.05, 1, 1024), (6, 2.0, 2, 1024), (7, 0.3, 33, 4096)]
    streams = _streams(host, specs)
    b = batch.Batch(_descs(batch, streams))
    s = torch.cuda.current_stream()
    for mode in ("direct", "graph", "graph"):
        for _, _, _, o in streams:
            o.fill_(0xCD)
        (b.decode if mode == "direct" else b.graph_decode)(s)
        acc, per = b.status(s)
        assert acc & ~mg.DEV_DEGENERATE == 0, per
        for st, u, t, o in streams:
            got = o[: st.n].cpu().numpy()
            assert np.array_equal(got[::-1], st.symbols), (mode, st.n, st.L)
    b.close()


def test_batch_matches_plain_decoder(mg):
    import torch

    from multians_gb300 import batch, host
    specs = [(21, 0.05, 500_000, 1024), (22, 1.0, 300_000, 4096), (23, 0.005, 200_000, 1024)]
    streams = _streams(host, specs)
    b = batch.Batch(_descs(batch, streams))
    s = torch.cuda.current_stream()
    b.decode(s)
    assert b.status(s)[0] == 0
    for st, u, t, o in streams:
        plain = mg.decode(u, st.n_units, st.n, t, st.first_state, st.first_bit, L=st.L)
        assert torch.equal(plain, o[: st.n])
    b.close()


def test_batch_per_stream_status_and_special_streams(mg, oracle_lib):
    """A bad table flags only its own stream; single-symbol and empty-output
    streams ride along."""
    import torch

    from multians_gb300 import batch, host
    good = _streams(host, [(31, 0.2, 100_000, 1024), (32, 0.05, 80_000, 1024)])
    bad_st, bu, bt, bo = _streams(host, [(33, 0.05, 50_000, 1024)])[0]
    bad = bad_st.table.copy()
    bad[7] = (bad[7] & 0x00ffffff) | (15 << 24)
    bt = torch.from_numpy(bad.view(np.int32)).cuda()
    one = oracle_lib.encode(np.full(4000, 42, dtype=np.uint8), 1024)
    ou = torch.from_numpy(one.units.view(np.int32)).cuda()
    ot = torch.from_numpy(one.table.view(np.int32)).cuda()
    oo = torch.zeros(4000, dtype=torch.uint8, device="cuda")
    descs = _descs(batch, good)
    descs.append(batch.desc(bu, bad_st.n_units, bo, bad_st.n, bt, 1024, bad_st.first_state,
                            bad_st.first_bit))
    descs.append(batch.desc(ou, one.n_units, oo, 4000, ot, 1024, one.first_state, one.first_bit))
    descs.append(batch.desc(ou, one.n_units, oo, 0, ot, 1024, one.first_state, one.first_bit))
    b = batch.Batch(descs)
    s = torch.cuda.current_stream()
    b.decode(s)
    acc, per = b.status(s)
    assert per[0] == 0 and per[1] == 0
    assert per[2] & mg.DEV_BAD_TABLE
    assert per[3] == mg.DEV_DEGENERATE and per[4] == 0
    for st, u, t, o in good:
        assert np.array_equal(o[: st.n].cpu().numpy()[::-1], st.symbols)
    assert bool((oo == 42).all())
    b.close()


def test_batch_mixed_output_orders(mg):
    """Streams of one batch choose their output order independently."""
    import torch

    from multians_gb300 import batch, host
    specs = [(41 + i, (0.05, 0.7, 2.0)[i % 3], 50_000 + 9_973 * i, (1024, 4096)[i % 2])
             for i in range(12)]
    streams = _streams(host, specs)
    descs = [batch.desc(u, st.n_units, o, st.n, t, st.L, st.first_state, st.first_bit,
                        source_order=bool(i % 2))
             for i, (st, u, t, o) in enumerate(streams)]
    b = batch.Batch(descs)
    s = torch.cuda.current_stream()
    b.graph_decode(s)
    assert b.status(s)[0] == 0
    for i, (st, u, t, o) in enumerate(streams):
        got = o[: st.n].cpu().numpy()
        assert np.array_equal(got if i % 2 else got[::-1], st.symbols), i
    b.close()
