"""The measured planner table (multians_gb300/csrc/mans_tune_table.h,
written by multians_gb300/tune.py from decodes timed on GB300) and the
planner's use of it: for a stream like each entry's, mans_tune_lookup returns
that entry and mans_plan returns the plan the entry prescribes (the same as
mans_plan_tuned with its values); explicit hints and MANS_PLAN_MODEL keep the
model; batches keep the model."""
import os
import re

import pytest

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                      "multians_gb300", "csrc", "mans_tune_table.h")
ROW = re.compile(r"^\s*\{(\d+), ([\d.]+)f, ([01]), (\d+), ([\d.]+)f, ([01]), ([\d.]+)f, ([\d.]+)f\},")


def _entries():
    out = []
    with open(HEADER) as f:
        for ln in f:
            m = ROW.match(ln)
            if m and int(m.group(1)) > 0:
                L, bps, large, B, mult, cap, g, mg_ = m.groups()
                out.append(dict(L=int(L), bps=float(bps), large=int(large), block_units=int(B),
                                meet_mult=float(mult), capture=int(cap), gbps=float(g),
                                model_gbps=float(mg_)))
    return out


def _stream(e):
    n_out = (256 << 20) if e["large"] else (16 << 20)
    n_units = int(round(n_out * e["bps"] / 32))
    return n_units, n_out


def test_table_is_measured():
    ents = _entries()
    assert len(ents) >= 40
    assert {e["L"] for e in ents} == {1024, 2048, 4096, 8192}
    assert {e["large"] for e in ents} == {0, 1}
    for e in ents:
        assert e["block_units"] in (4, 8, 16)
        assert e["capture"] == 0 or e["L"] <= 4096
        # the sweep keeps the fastest plan, the model's among the candidates
        assert e["gbps"] >= 0.97 * e["model_gbps"], e


@pytest.mark.parametrize("e", _entries(), ids=lambda e: f"L{e['L']}-bps{e['bps']}-{e['large']}")
def test_planner_returns_the_table_entry(mg, e):
    n_units, n_out = _stream(e)
    got = mg.tune_lookup(e["L"], 32.0 * n_units / n_out, n_out)
    assert got is not None
    for k in ("L", "large", "block_units", "capture"):
        assert got[k] == e[k], (k, got, e)
    assert abs(got["meet_mult"] - e["meet_mult"]) < 1e-6
    assert abs(got["bits_per_symbol"] - e["bps"]) < 1e-3
    # capture as measured, from 16 Mi units on (where capture pays at all)
    cap = bool(e["capture"]) and n_units >= 16 << 20
    plan = mg.plan(n_units, n_out, e["L"])
    assert plan == mg.plan_tuned(n_units, n_out, e["L"], e["block_units"], e["meet_mult"], cap)
    assert plan["block_units"] == e["block_units"]
    assert (plan["capture_bytes"] > 0) == cap


def test_hints_and_model_flag_bypass_the_table(mg):
    n_units, n_out, L = 12_800_000, 256 << 20, 1024   # 1.5 bits/symbol: the table differs
    tuned = mg.plan(n_units, n_out, L)
    model = mg.plan(n_units, n_out, L, {"flags": mg.PLAN_MODEL})
    assert tuned["block_units"] != model["block_units"] or \
        tuned["region_blocks"] != model["region_blocks"]
    fixed = mg.plan(n_units, n_out, L, {"block_units": 8})
    assert fixed["block_units"] == 8
    # a table plan given back as the hint keeps its geometry and its capture choice
    assert mg.plan(n_units, n_out, L, tuned) == tuned


def test_lookup_outside_the_table(mg):
    assert mg.tune_lookup(512, 6.0, 1 << 28) is None
    assert mg.tune_lookup(16384, 6.0, 1 << 28) is None
    # nearest bits per symbol within the same L and size class
    assert mg.tune_lookup(1024, 5.0, 1 << 28)["bits_per_symbol"] == pytest.approx(6.001, abs=1e-3)
    assert mg.tune_lookup(1024, 5.0, 1 << 20)["large"] == 0
