"""Measured autotuner of the decode planner (run on a GB300).

    python -m multians_gb300.tune [--out multians_gb300/csrc/mans_tune_table.h]
                                  [--json sweep.json] [--sizes 16,256]
                                  [--L 1024,2048,4096,8192]
                                  [--lam 0.005,0.05,0.2,1.0,2.0]

For every table size L, stream size (MiB of symbols) and lambda of the
generator (the reference's symbol distribution, about 0.67 .. 8.6 bits per
symbol), one seeded stream is encoded and decoded with every candidate
plan: units per block B in {4, 8, 16}, shortest region in mean merge
distances m in {1.5, 2, 3, 4, 6, 8, 12}, symbol capture off / on (on only
for L <= 4096, where its rings fit in shared memory).  Candidates that give
the same geometry are timed once; a candidate whose merge walks run out of
slots is dropped.  Each plan is timed with CUDA events over three decodes
after one warm-up, inputs resident in HBM; the fastest one is checked
bit-exact against the source and written as the entry of (L, bits per
symbol, size class) in the C header the planner compiles (mans_plan reads
it; MANS_PLAN_MODEL and explicit hints bypass it).  The model's own plan is
timed beside it and both figures go into the entry.

The reference has no tuner: its subsequence size and threads per block are
caller arguments (include/cuhd_gpu_decoder.h:24-35) and its
CUHDUtil::optimal_subsequence_size (src/multians_util.cc:74-86) is unused.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import datetime
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_OUT = os.path.join(HERE, "csrc", "mans_tune_table.h")
BLOCKS = (4, 8, 16)
MEET_MULTS = (1.5, 2.0, 3.0, 4.0, 6.0, 8.0, 12.0)
CAPTURE_MAX_L = 4096


def _time_plan(mg, st, units, table, out, aux, cfg, stream, reps=3):
    """ms per decode with this plan, or None if its walks ran out of slots."""
    import torch

    from .decoder import aux_status, decode_async

    def one():
        decode_async(units, st.n_units, out, st.n, table, st.L, st.first_state, st.first_bit,
                     aux, cfg, stream=stream)

    try:
        one()
    except mg.MansError as e:   # a plan the decoder refuses is not a candidate
        print(f"  plan {cfg} refused: {e}", flush=True)
        return None
    if aux_status(aux, stream) & mg.DEV_SYNC_OVERFLOW:
        return None
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        one()
    e1.record(stream)
    torch.cuda.synchronize()
    if aux_status(aux, stream):
        return None
    return e0.elapsed_time(e1) / reps


def sweep_stream(mg, st, log):
    """Times every candidate plan on one stream; returns the record."""
    import torch

    dev = torch.device("cuda")
    stream = torch.cuda.current_stream(dev)
    units = torch.from_numpy(st.units.view(np.int32)).to(dev)
    table = torch.from_numpy(st.table.view(np.int32)).to(dev)
    out = torch.empty(max(1, st.n), dtype=torch.uint8, device=dev)
    cands, seen = [], {}
    for cap in (False, True):
        if cap and st.L > CAPTURE_MAX_L:
            continue
        for B in BLOCKS:
            for m in MEET_MULTS:
                cfg = mg.plan_tuned(st.n_units, st.n, st.L, B, m, cap)
                key = (cfg["block_units"], cfg["region_blocks"], cfg["walk_slots"],
                       cfg["capture_bytes"] > 0)
                if key in seen:
                    continue
                seen[key] = len(cands)
                cands.append({"block_units": B, "meet_mult": m, "capture": cap, "cfg": cfg})
    model = mg.plan(st.n_units, st.n, st.L, {"flags": mg.PLAN_MODEL})
    need = max([mg.aux_size(st.n_units, c["cfg"]) for c in cands] +
               [mg.aux_size(st.n_units, model)])
    aux = torch.empty(need, dtype=torch.uint8, device=dev)
    model_ms = _time_plan(mg, st, units, table, out, aux, model, stream)
    for c in cands:
        c["ms"] = _time_plan(mg, st, units, table, out, aux, c["cfg"], stream)
    valid = [c for c in cands if c["ms"] is not None]
    best = min(valid, key=lambda c: c["ms"])
    # the winner, timed again and checked against the source
    best["ms"] = min(best["ms"], _time_plan(mg, st, units, table, out, aux, best["cfg"], stream))
    exact = bool(np.array_equal(out.cpu().numpy()[::-1], st.symbols))
    rec = {"L": st.L, "n": st.n, "n_units": st.n_units,
           "bps": round(st.bits_per_symbol, 4), "model": model,
           "model_ms": model_ms, "best": {k: best[k] for k in ("block_units", "meet_mult",
                                                               "capture", "cfg", "ms")},
           "bit_exact": exact, "candidates": [
               {k: c[k] for k in ("block_units", "meet_mult", "capture", "cfg", "ms")}
               for c in cands]}
    log(f"L={st.L:5d} n={st.n >> 20:4d}MiB bps={st.bits_per_symbol:5.2f}: best B={best['block_units']} "
        f"m={best['meet_mult']} cap={int(best['capture'])} {st.n / best['ms'] / 1e6:7.1f} GB/s, "
        f"model {st.n / model_ms / 1e6 if model_ms else float('nan'):7.1f} GB/s, "
        f"{len(valid)}/{len(cands)} plans, exact={exact}")
    return rec


def write_header(records, path, command):
    rows = []
    for r in sorted(records, key=lambda r: (r["n"] > (32 << 20), r["L"], r["bps"])):
        b = r["best"]
        gbps = r["n"] / b["ms"] / 1e6
        mg_ = r["n"] / r["model_ms"] / 1e6 if r["model_ms"] else 0.0
        rows.append(f"    {{{r['L']}, {r['bps']:.3f}f, {int(r['n'] > (32 << 20))}, {b['block_units']}, "
                    f"{b['meet_mult']:.1f}f, {int(b['capture'])}, {gbps:.1f}f, {mg_:.1f}f}},")
    when = datetime.datetime.now(datetime.timezone.utc).strftime("%Y-%m-%d %H:%M UTC")
    text = f"""// Measured planner table, written by multians_gb300/tune.py from decodes
// timed on GB300; read by mans_plan (mans_decode.cu).  Do not edit by hand:
// run the tool again.
//   command: {command}
//   measured: {when}, {len(rows)} entries
// Each entry: the stream it was measured on (L, bits per symbol, size
// class: 1 = 256 MiB of symbols, 0 = 16 MiB) and the fastest plan found
// (units per block, shortest region in mean merge distances, capture), with
// its decoded GB/s and the model's plan's on the same stream.
#pragma once

#include <cstdint>

namespace mans {{

struct TuneEntry {{
    uint32_t L;            // table size the entry was measured at
    float bps;             // bits per symbol of the swept stream
    uint32_t large;        // 1: measured on 256 MiB of symbols, 0: on 16 MiB
    uint32_t block_units;  // units per block
    float meet_mult;       // shortest region, in mean meeting distances
    uint32_t capture;      // symbol capture on
    float gbps;            // decoded GB/s of this choice in the sweep
    float model_gbps;      // decoded GB/s of the model's own plan there
}};

constexpr TuneEntry kTuneTable[] = {{
{chr(10).join(rows)}
}};
constexpr uint32_t kTuneCount = sizeof(kTuneTable) / sizeof(kTuneTable[0]);

}}  // namespace mans
"""
    with open(path, "w") as f:
        f.write(text)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=DEFAULT_OUT)
    ap.add_argument("--json", default=None)
    ap.add_argument("--sizes", default="16,256", help="MiB of symbols per stream")
    ap.add_argument("--L", default="1024,2048,4096,8192")
    ap.add_argument("--lam", default="0.005,0.05,0.2,1.0,2.0")
    ap.add_argument("--seed", type=int, default=20261204)
    args = ap.parse_args(argv)
    import torch

    import multians_gb300 as mg
    from multians_gb300 import host
    if not torch.cuda.is_available():
        raise SystemExit("the tuning sweep times decodes on a GPU")
    sizes = [float(x) for x in args.sizes.split(",")]
    Ls = [int(x) for x in args.L.split(",")]
    lams = [float(x) for x in args.lam.split(",")]
    records = []
    log = lambda s: print(s, flush=True)  # noqa: E731
    for mib in sizes:
        n = int(mib * (1 << 20))
        for L in Ls:
            specs = [(args.seed + i, lam, n, L) for i, lam in enumerate(lams)]
            with cf.ThreadPoolExecutor(max_workers=len(specs)) as ex:
                sts = list(ex.map(lambda sp: host.make_stream(*sp), specs))
            for st in sts:
                records.append(sweep_stream(mg, st, log))
                torch.cuda.empty_cache()
            del sts
    command = "python -m multians_gb300.tune " + " ".join(
        f"--{k} {v}" for k, v in (("sizes", args.sizes), ("L", args.L), ("lam", args.lam)))
    write_header(records, args.out, command)
    if args.json:
        with open(args.json, "w") as f:
            json.dump(records, f)
    log(f"wrote {args.out} ({len(records)} entries)")


if __name__ == "__main__":
    main()
