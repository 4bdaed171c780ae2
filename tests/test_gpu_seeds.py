"""GPU parity of seeded merge walks (MANS_DECODE_SEEDS): a warp's last long
walk is finished with the warp's idle lanes decoding from guessed states
ahead of it.  The output must equal the oracle's sequential decode byte for
byte with seeds forced on and forced off, and the seeded path must actually
run (the sync statistics count the walks it finished)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).to("cuda")


def _decode(mg, st, hint):
    import torch
    from multians_gb300 import _lib
    from multians_gb300.decoder import aux_status, decode_async
    plan = mg.plan(st.n_units, st.n, st.L, hint)
    aux = torch.empty(mg.aux_size(st.n_units, plan), dtype=torch.uint8, device="cuda")
    out = torch.full((st.n + 16,), 0xAB, dtype=torch.uint8, device="cuda")
    decode_async(_dev(st.units), st.n_units, out, st.n, _dev(st.table), st.L, st.first_state,
                 st.first_bit, aux, plan)
    status = aux_status(aux)
    assert status == 0, f"device status 0x{status:x}"
    stats = _lib.sync_stats(aux.data_ptr(), aux.numel(), st.n_units, st.n, st.L, plan)
    got = out.cpu().numpy()
    assert (got[st.n:] == 0xAB).all(), "wrote past n_out"
    return got[:st.n], plan, stats


CASES = [
    # (lambda, L, symbols, geometry hint): walk-heavy streams
    (1.0, 4096, 6_000_000, {}),
    (0.2, 1024, 6_000_000, {}),
    (2.0, 4096, 4_000_000, {}),
    # short regions: seeded walks that cross several regions look the next
    # region's trajectory up through other walks' records
    (1.0, 4096, 6_000_000, {"block_units": 16, "region_blocks": 31, "walk_slots": 12}),
    (0.2, 1024, 4_000_000, {"block_units": 16, "region_blocks": 15, "walk_slots": 12}),
    # the headline's distribution
    (0.05, 1024, 6_000_000, {}),
]


@pytest.mark.parametrize("lam,L,n,geo", CASES)
def test_seeded_walks_match_oracle(mg, oracle_lib, lam, L, n, geo):
    O = oracle_lib
    st = O.make_stream(seed=9100 + int(lam * 100) + L + len(geo), lam=lam, n=n, L=L)
    want = O.decode_seq(st)
    on, plan_on, s_on = _decode(mg, st, dict(geo, flags=mg.DECODE_SEEDS))
    off, plan_off, s_off = _decode(mg, st, dict(geo, flags=mg.DECODE_NO_SEEDS))
    assert plan_on["flags"] & mg.DECODE_SEEDS and not plan_off["flags"] & mg.DECODE_SEEDS
    assert np.array_equal(off, want)
    assert np.array_equal(on, want)
    assert s_off["seeded_walks"] == 0
    # the merge points may differ (a seeded walk can stop at a later block
    # start where both trajectories agree), the walks' count may not
    assert s_on["walks"] == s_off["walks"]
    if lam >= 0.2:
        assert s_on["seeded_walks"] > 0, s_on


def test_seeded_walks_with_capture(mg, oracle_lib):
    """Symbol capture on: a seeded walk stops capturing; its blocks are
    decoded by the final pass."""
    O = oracle_lib
    st = O.make_stream(seed=9200, lam=0.2, n=6_000_000, L=1024)
    want = O.decode_seq(st)
    got, plan, stats = _decode(mg, st, {"flags": mg.DECODE_SEEDS | mg.DECODE_CAPTURE})
    assert plan["capture_bytes"] > 0
    assert stats["seeded_walks"] > 0, stats
    assert np.array_equal(got, want)
