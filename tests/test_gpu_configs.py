"""GPU parity at the sizes and geometries of the benchmark workloads.

The small-stream tests elsewhere run the planner's short-stream geometries;
these run the ones the workloads themselves get:

- the reference's own CPU-runnable case (src/main.cc:19-32 decodes 1024-state
  tables; here 16 MiB of lambda = 0.05 symbols), against the oracle's
  sequential decode, the oracle's port of the reference's MulticoreDecoder
  (src/multicore_decoder.cc:17-90, S = 4) and the source;
- the two walk-heavy points of the 256 MiB sweep (L = 4096 at lambda = 1.0
  and 0.2, 1.5 and 3.8 bits per symbol, where merge walks are longest) at
  64 MiB with the planner's own geometry;
- the 2 GiB worst-case-sync streams' geometry (the planner's choice for
  2 GiB at L = 4096, lambda = 0.005 and 2.0: long regions, and symbol
  capture at 8.6 bits per symbol) forced onto 128 MiB streams of the same
  statistics;
- a 256-stream draw of the 4096-stream batch workload (sizes log-uniform in
  [4 KB, 4 MB], lambda ~ U[0.01, 1], own L = 1024 tables) through the
  one-call batch entry point, every stream against the plain decoder and
  its source.

Every comparison is byte for byte."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MiB = 1 << 20


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).to("cuda")


def _decode(mg, st, cfg=None):
    import torch
    out = torch.full((st.n,), 0xAB, dtype=torch.uint8, device="cuda")
    mg.decode(_dev(st.units), st.n_units, st.n, _dev(st.table), st.first_state, st.first_bit,
              L=st.L, out=out, cfg=cfg)
    return out.cpu().numpy()


def _plan_used(mg, st, cfg=None):
    return mg.plan(st.n_units, st.n, st.L, cfg)


def test_reference_case_16MiB(mg, oracle_lib):
    """16 MiB, lambda = 0.05, L = 1024: the GPU output equals the oracle's
    sequential decode, its MulticoreDecoder port and the source."""
    O = oracle_lib
    st = O.make_stream(seed=5, lam=0.05, n=16 * MiB, L=1024)
    got = _decode(mg, st)
    want = O.decode_seq(st)
    assert np.array_equal(got, want)
    mc, _ = O.multicore_decode(st, S=4, T=16)
    assert np.array_equal(got, mc)
    assert np.array_equal(got[::-1], st.symbols)


@pytest.mark.parametrize("lam", [1.0, 0.2])
def test_walk_heavy_64MiB_L4096(mg, oracle_lib, lam):
    """L = 4096 at 1.5 and 3.8 bits per symbol, the sweep's longest merge
    walks, with the planner's default geometry (and, at 3.8 bits per
    symbol, its choice of symbol capture)."""
    O = oracle_lib
    st = O.make_stream(seed=4096 + int(lam * 10), lam=lam, n=64 * MiB, L=4096)
    plan = _plan_used(mg, st)
    got = _decode(mg, st)
    assert np.array_equal(got, O.decode_seq(st)), plan
    assert np.array_equal(got[::-1], st.symbols)


@pytest.mark.parametrize("lam", [0.005, 2.0])
def test_2GiB_geometry_on_128MiB(mg, oracle_lib, lam):
    """The geometry the planner picks for a 2 GiB stream (L = 4096) applied
    to a 128 MiB stream of the same bits per symbol: the same region and
    block lengths, walk slots and capture slice, fewer regions."""
    O = oracle_lib
    st = O.make_stream(seed=2048 + int(lam * 1000), lam=lam, n=128 * MiB, L=4096)
    n_big = 2 << 30
    units_big = int(round(st.n_units * (n_big / st.n)))
    big = mg.plan(units_big, n_big, 4096)
    cfg = {k: big[k] for k in ("block_units", "region_blocks", "walk_slots", "capture_bytes")}
    if not cfg["capture_bytes"]:
        cfg["flags"] = mg.DECODE_NO_CAPTURE
        del cfg["capture_bytes"]
    used = mg.plan(st.n_units, st.n, 4096, cfg)
    assert used["region_blocks"] == big["region_blocks"]
    assert used["block_units"] == big["block_units"]
    assert (used["capture_bytes"] > 0) == (big["capture_bytes"] > 0)
    got = _decode(mg, st, cfg=cfg)
    assert np.array_equal(got, O.decode_seq(st)), (big, used)
    assert np.array_equal(got[::-1], st.symbols)


def test_batch_workload_draw_256(mg):
    """256 streams of the batch workload's distribution through
    mans_decode_batch; each equals the plain decoder's output and its
    source."""
    import concurrent.futures as cf
    import os

    import torch

    from multians_gb300 import batch, host
    from multians_gb300.bench_workloads import batched_specs
    specs = batched_specs(20261203, 4096)[:256]
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 8) as ex:
        sts = list(ex.map(lambda sp: host.make_stream(*sp), specs))
    keep, descs = [], []
    for st in sts:
        u, t = _dev(st.units), _dev(st.table)
        o = torch.full((st.n,), 0xCD, dtype=torch.uint8, device="cuda")
        keep.append((u, t, o))
        descs.append(batch.desc(u, st.n_units, o, st.n, t, st.L, st.first_state, st.first_bit))
    acc, per = batch.decode_batch(descs, stream=torch.cuda.current_stream())
    assert acc & ~mg.DEV_DEGENERATE == 0, per
    for st, (u, t, o) in zip(sts, keep):
        got = o.cpu().numpy()
        assert np.array_equal(got[::-1], st.symbols), (st.n, st.L)
        plain = torch.full((st.n,), 0xAB, dtype=torch.uint8, device="cuda")
        mg.decode(u, st.n_units, st.n, t, st.first_state, st.first_bit, L=st.L, out=plain)
        assert np.array_equal(plain.cpu().numpy(), got), (st.n, st.L)
