"""The planner's choice of seeded merge walks (MANS_DECODE_SEEDS), on the
CPU: on from 1 to 4.5 bits per symbol (to 7 at L >= 4096), where the GB300
sweep found them faster, off elsewhere, and as the hint forces it."""


def test_planner_turns_seeds_on_where_walks_are_long(mg):
    on = mg.DECODE_SEEDS
    assert mg.plan(12_700_000, 256 << 20, 4096)["flags"] & on          # 1.5 bits/symbol
    assert mg.plan(50_339_428, 256 << 20, 4096)["flags"] & on          # 6 bits, L = 4096
    assert mg.plan(33_000_000, 256 << 20, 1024)["flags"] & on          # 3.8 bits/symbol
    assert not mg.plan(50_339_428, 256 << 20, 1024)["flags"] & on      # 6 bits, L = 1024
    assert not mg.plan(3_145_728, 16 << 20, 1024)["flags"] & on
    assert not mg.plan(5_620_000, 256 << 20, 1024)["flags"] & on       # 0.67 bits/symbol
    assert not mg.plan(72_150_000, 256 << 20, 4096)["flags"] & on      # 8.6 bits/symbol


def test_hint_forces_seeds(mg):
    on, off = mg.DECODE_SEEDS, mg.DECODE_NO_SEEDS
    assert not mg.plan(12_700_000, 256 << 20, 4096, {"flags": off})["flags"] & on
    assert mg.plan(50_339_428, 256 << 20, 1024, {"flags": on})["flags"] & on
    # a plan given back as a hint keeps its choice
    p = mg.plan(12_700_000, 256 << 20, 4096)
    assert mg.plan(12_700_000, 256 << 20, 4096, p)["flags"] & on
