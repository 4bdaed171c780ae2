"""Batched and served workloads of bench.py.

batched: 4096 independent streams, sizes log-uniform in [4 KB, 4 MB] of
uint8 symbols, each with its own lambda ~ U[0.01, 1], its own L = 1024
table and its own encoding.  value = decoded GB/s of one CUDA-graph replay
of the batched decode over all streams; the same streams through a loop of
plain per-stream decodes launched from C (mans_decode_loop: cached plans,
one mans_decode per stream, asynchronous, one CUDA stream) are timed beside
it, with each stream's GPU time.
"""
from __future__ import annotations

import concurrent.futures as cf
import json
import os
import statistics
import time

import numpy as np

METRIC = "decoded GB/s on 1 GB300 (plain vs batched/served) + %HBM roofline; p50/p99; bit-exact"


def _encode_many(specs, threads):
    from multians_gb300 import host

    def one(sp):
        seed, lam, n, L = sp
        return host.make_stream(seed, lam, n, L)

    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        return list(ex.map(one, specs))


def batched_specs(seed: int, count: int = 4096, lo: float = 4096, hi: float = 4 << 20):
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), count)).astype(np.int64)
    lams = rng.uniform(0.01, 1.0, count)
    return [(seed * 7919 + i, float(lams[i]), int(sizes[i]), 1024) for i in range(count)]


def measure_batched(args, ws, rank, local):
    """The batched workload's bench line (None on ranks other than 0)."""
    import torch

    import multians_gb300 as mg
    from multians_gb300 import batch

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    count = int(os.environ.get("MANS_BATCH_STREAMS", "4096"))
    specs = batched_specs(args.seed + rank, count)
    t0 = time.time()
    sts = _encode_many(specs, os.cpu_count() or 8)
    gen_s = time.time() - t0
    total_sym = sum(st.n for st in sts)
    total_comp = sum(st.n_units * 4 for st in sts)
    # all streams packed into one unit buffer (each stream 16-byte aligned)
    # and one output buffer, as a caller batching many streams keeps them,
    # so the host copies are one per direction
    offs = np.zeros(len(sts) + 1, dtype=np.int64)
    for i, st in enumerate(sts):
        offs[i + 1] = offs[i] + ((st.units.size + 3) & ~3)
    h_units_all = torch.zeros(int(offs[-1]), dtype=torch.int32).pin_memory()
    hu_np = h_units_all.numpy()
    for i, st in enumerate(sts):
        hu_np[offs[i]: offs[i] + st.units.size] = st.units.view(np.int32)
    d_units_all = h_units_all.to(dev)
    units = [d_units_all[int(offs[i]): int(offs[i]) + st.units.size] for i, st in enumerate(sts)]
    tables = [torch.from_numpy(st.table.view(np.int32)).to(dev) for st in sts]
    oo = np.concatenate([[0], np.cumsum([st.n for st in sts])])
    d_out_all = torch.empty(int(oo[-1]), dtype=torch.uint8, device=dev)
    outs = [d_out_all[int(oo[i]): int(oo[i + 1])] for i in range(len(sts))]
    stream = torch.cuda.current_stream(dev)

    # batched decode
    cap = not getattr(args, "no_capture", False)
    descs = [batch.desc(u, st.n_units, o, st.n, t, st.L, st.first_state, st.first_bit, capture=cap)
             for st, u, t, o in zip(sts, units, tables, outs)]
    b = batch.Batch(descs)
    for _ in range(max(3, args.warmup)):
        b.graph_decode(stream)
    acc, per = b.status(stream)
    n_overflow = sum(1 for x in per if x & mg.DEV_SYNC_OVERFLOW)
    n_redone = b.fixup(stream) if n_overflow else 0
    acc, per = b.status(stream)
    ok = acc & ~mg.DEV_DEGENERATE == 0
    for st, o in zip(sts, outs):
        if not ok:
            break
        ok = bool(np.array_equal(o.cpu().numpy()[::-1], st.symbols))
    steps = max(3, args.steps)
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    torch.cuda.synchronize(dev)
    from bench import ClockSampler
    with ClockSampler(local) as clk:
        evs[0].record(stream)
        for i in range(steps):
            b.graph_decode(stream)
            evs[i + 1].record(stream)
        torch.cuda.synchronize(dev)
    per_ms = sorted(evs[i].elapsed_time(evs[i + 1]) for i in range(steps))
    batch_ms = evs[0].elapsed_time(evs[-1]) / steps
    # per-kernel split: the same batch launched without the graph, events
    # around each kernel (outside the timed region)
    from multians_gb300 import _lib
    _lib.timing_enable(3)
    for _ in range(3):
        b.decode(stream)
    launches_per_batch = int(mg.lib().mans_last_launch_count())   # kernels of one batch decode
    torch.cuda.synchronize(dev)
    kern_ms, kern_n = _lib.timing_collect()
    _lib.timing_enable(0)
    kernel_ms = {k: round(v / max(1, kern_n), 4) for k, v in kern_ms.items()}

    # loop of plain decodes over the same streams, launched from C
    # (mans_decode_loop) the way a C++ caller runs it: plans cached and
    # workspaces allocated up front, one mans_decode per stream on one stream
    hint = None if cap else {"flags": mg.DECODE_NO_CAPTURE}
    plans = [mg.plan(st.n_units, st.n, st.L, hint) for st in sts]
    auxes = [torch.empty(mg.aux_size(st.n_units, p), dtype=torch.uint8, device=dev)
             for st, p in zip(sts, plans)]
    loop = batch.Loop(descs, plans, auxes)
    loop.run(stream)
    torch.cuda.synchronize(dev)
    l0, l1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    lsteps = 3
    l0.record(stream)
    for _ in range(lsteps):
        loop_launches = loop.run(stream)
    l1.record(stream)
    torch.cuda.synchronize(dev)
    loop_ms = l0.elapsed_time(l1) / lsteps
    # per-stream GPU time: an event after each stream's decode (one more run)
    sev = [torch.cuda.Event(enable_timing=True) for _ in range(len(sts) + 1)]
    for e in sev:
        e.record(stream)   # creates the events
    torch.cuda.synchronize(dev)
    sev[0].record(stream)
    loop.run(stream, events=sev[1:])
    torch.cuda.synchronize(dev)
    per_stream = np.array([sev[i].elapsed_time(sev[i + 1]) for i in range(len(sts))])
    loop_ok = all(np.array_equal(o.cpu().numpy()[::-1], st.symbols)
                  for st, o in zip(sts, outs))
    del auxes, loop

    # e2e: the packed host units -> device, graph decode, all symbols back
    h_out_all = torch.empty(int(oo[-1]), dtype=torch.uint8).pin_memory()
    e2e_times = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        d_out_all.fill_(0xCD)
        e0.record(stream)
        d_units_all.copy_(h_units_all, non_blocking=True)
        b.graph_decode(stream)
        h_out_all.copy_(d_out_all, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        e2e_times.append(e0.elapsed_time(e1))
    e2e_serial_ms = sorted(e2e_times)[1]
    if n_overflow:
        b.fixup(stream)
        h_out_all.copy_(d_out_all)
    ho_np = h_out_all.numpy()
    e2e_ok = all(np.array_equal(ho_np[oo[i]: oo[i + 1]][::-1], st.symbols)
                 for i, st in enumerate(sts))

    # pipelined e2e, as a streaming caller runs it: a second buffer set and
    # batch; step i's input copy, decode and output copy on three streams,
    # each waiting only on what it reads or overwrites (the decode of step
    # i overlaps the input copy of step i+1 and the output copy of step
    # i-1); every step still moves all its bytes
    e2e_ms = e2e_serial_ms
    pipelined = n_overflow == 0
    if pipelined:
        d_units2 = torch.empty_like(d_units_all)
        d_out2 = torch.empty_like(d_out_all)
        h_out2 = torch.empty_like(h_out_all).pin_memory()
        units2 = [d_units2[int(offs[i]): int(offs[i]) + st.units.size] for i, st in enumerate(sts)]
        outs2 = [d_out2[int(oo[i]): int(oo[i + 1])] for i in range(len(sts))]
        descs2 = [batch.desc(u, st.n_units, o, st.n, t, st.L, st.first_state, st.first_bit,
                             capture=cap) for st, u, t, o in zip(sts, units2, tables, outs2)]
        b2 = batch.Batch(descs2)
        b2.graph_decode(stream)
        sets = [(d_units_all, d_out_all, h_out_all, b), (d_units2, d_out2, h_out2, b2)]
        s_in, s_out = torch.cuda.Stream(dev), torch.cuda.Stream(dev)

        def run(nsteps):
            ev = lambda: torch.cuda.Event()  # noqa: E731
            t0 = torch.cuda.Event(enable_timing=True)
            t1 = torch.cuda.Event(enable_timing=True)
            in_done, dec_done, out_done = [], [], []
            t0.record(s_in)
            for i in range(nsteps):
                du, do, ho, bb = sets[i & 1]
                with torch.cuda.stream(s_in):
                    if i >= 2:
                        s_in.wait_event(dec_done[i - 2])
                    du.copy_(h_units_all, non_blocking=True)
                    in_done.append(ev())
                    in_done[i].record(s_in)
                stream.wait_event(in_done[i])
                if i >= 2:
                    stream.wait_event(out_done[i - 2])
                bb.graph_decode(stream)
                dec_done.append(ev())
                dec_done[i].record(stream)
                s_out.wait_event(dec_done[i])
                with torch.cuda.stream(s_out):
                    ho.copy_(do, non_blocking=True)
                    out_done.append(ev())
                    out_done[i].record(s_out)
            t1.record(s_out)
            torch.cuda.synchronize(dev)
            return t0.elapsed_time(t1) / nsteps, (nsteps - 1) & 1

        run(2)
        # the bench's own K steps (the pipeline fills and drains once per
        # run); median of three: the host links are shared
        runs = [run(max(6, args.steps)) for _ in range(3)]
        e2e_ms = sorted(r[0] for r in runs)[1]
        last = runs[-1][1]
        acc2, _ = sets[last][3].status(stream)
        hl = sets[last][2].numpy()
        e2e_ok = e2e_ok and (acc2 & ~mg.DEV_DEGENERATE) == 0 and all(
            np.array_equal(hl[oo[i]: oo[i + 1]][::-1], st.symbols) for i, st in enumerate(sts))
        b2.close()
        del d_units2, d_out2, h_out2
    b.close()
    from bench import max_over_ranks, measured_peaks, replica_rate
    batch_ms, e2e_ms, e2e_serial_ms, loop_ms = max_over_ranks(
        [batch_ms, e2e_ms, e2e_serial_ms, loop_ms], dev)
    if rank != 0:
        return None
    hbm, kind = measured_peaks()
    value = replica_rate(total_sym, ws, batch_ms)
    alg = (total_comp + total_sym) / (batch_ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": ws,
        "steps": steps, "warmup": args.warmup, "ms_per_step": round(batch_ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic",
        "config": {"workload": f"batched {count} streams log-uniform [4KB,4MB] lambda~U[0.01,1] L=1024",
                   "n_streams": count, "n_symbols": total_sym, "compressed_bytes": total_comp,
                   "seed": args.seed, "mode": "one CUDA-graph replay of the batched decode",
                   "l2": "inputs larger than L2, no flush"},
        "bit_exact": bool(ok and e2e_ok),
        "sync_overflow_streams": n_overflow, "streams_redone": n_redone,
        "latency_ms": {"p50": round(per_ms[len(per_ms) // 2], 4),
                       "p99": round(per_ms[min(len(per_ms) - 1, int(0.99 * len(per_ms)))], 4)},
        "kernel_ms": kernel_ms,
        "loop_of_plain": {"ms": round(loop_ms, 3),
                          "value": round(total_sym / (loop_ms / 1e3) / 1e9, 3),
                          "speedup_batched_vs_loop": round(loop_ms / batch_ms, 3),
                          "launched_from": "C (mans_decode_loop: cached plans, one "
                                           "mans_decode per stream, one CUDA stream)",
                          "kernels": int(loop_launches), "bit_exact": bool(loop_ok),
                          "per_stream_ms": {"mean": round(float(per_stream.mean()), 4),
                                            "p50": round(float(np.median(per_stream)), 4),
                                            "p99": round(float(np.quantile(per_stream, 0.99)), 4),
                                            "max": round(float(per_stream.max()), 4)}},
        "roofline": {"bound": "hbm", "kernel": "batched decode (4 kernels)",
                     "achieved": round(alg, 2), "peak": hbm, "peak_kind": kind, "unit": "GB/s",
                     "frac": round(alg / hbm, 4), "traffic": None,
                     "alg_bytes_per_launch": total_comp + total_sym},
        "cpu_baseline": None,
        "e2e": {"value": round(ws * total_sym / (e2e_ms / 1e3) / 1e9, 3), "unit": "GB/s",
                "h2d_bytes_per_step": int(offs[-1]) * 4, "d2h_bytes_per_step": total_sym,
                "bit_exact": bool(e2e_ok),
                "pipelined": "2 buffer sets and batches; H2D, graph decode, D2H on 3 streams"
                if pipelined else None,
                "serial_value": round(ws * total_sym / (e2e_serial_ms / 1e3) / 1e9, 3)},
        "gpu_launches": launches_per_batch * steps,
        "clocks": clk.summary(),
        "gen_seconds": round(gen_s, 2),
    }
    return line


def run_batched(args, ws, rank, local):
    line = measure_batched(args, ws, rank, local)
    if line is not None:
        print(json.dumps(line), flush=True)


def run_encode(args, ws, rank, local):
    """GPU encode of the plain workload's stream (256 MiB, lambda, L): value =
    encoded source bytes per second with the symbols resident in HBM
    (histogram, table build from it on the host, encode); e2e adds the
    symbols' host->device copy and the units' copy back.  The units are
    checked against the host encoder's.  cpu_baseline: the host encoder
    (the reference's ANSEncoder restated) on a bounded prefix."""
    import torch

    from multians_gb300 import encode, host

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    n = int(args.mb * (1 << 20))
    sym = host.gen_symbols(args.seed + rank, args.lam, n)
    h_sym = torch.from_numpy(sym).pin_memory()
    d_sym = h_sym.to(dev)
    stream = torch.cuda.current_stream(dev)
    for _ in range(max(3, args.warmup)):
        units, n_units, fb, fs, dec = encode.encode(d_sym, args.L)
    torch.cuda.synchronize(dev)
    steps = max(3, args.steps)
    from bench import ClockSampler
    t_dev = []
    with ClockSampler(local) as clk:
        for _ in range(steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            units, n_units, fb, fs, dec = encode.encode(d_sym, args.L)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            t_dev.append(e0.elapsed_time(e1))
    # e2e: symbols in from pinned host memory, units back
    h_units = torch.empty(units.numel(), dtype=torch.int32).pin_memory()
    t_e2e = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        d2 = h_sym.to(dev, non_blocking=True)
        u2, nu2, fb2, fs2, _ = encode.encode(d2, args.L)
        h_units[: u2.numel()].copy_(u2, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        t_e2e.append(e0.elapsed_time(e1))
    # parity with the host encoder (full stream) and its time on a prefix
    t0 = time.perf_counter()
    ref = host.encode(sym, args.L)
    host_s = time.perf_counter() - t0
    exact = (n_units, fb, fs) == (ref.n_units, ref.first_bit, ref.first_state) and bool(
        np.array_equal(units.cpu().numpy().view(np.uint32), ref.units))
    from bench import max_over_ranks
    ms, e2e_med = max_over_ranks([statistics.median(t_dev), statistics.median(t_e2e)], dev)
    if rank != 0:
        return
    line = {
        "metric": "encoded GB/s on 1 GB300 (source bytes / s), bit-exact with the reference encoder",
        "value": round(ws * n / (ms / 1e3) / 1e9, 3), "unit": "GB/s", "n_gpus": ws,
        "steps": steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic",
        "config": {"workload": f"encode {args.mb:g}MiB lambda={args.lam} L={args.L}",
                   "n_symbols": n, "n_units": n_units, "seed": args.seed,
                   "step": "histogram + host table build + 6 encode kernels"},
        "bit_exact": exact,
        "e2e": {"value": round(ws * n / (e2e_med / 1e3) / 1e9, 3),
                "unit": "GB/s", "h2d_bytes_per_step": n, "d2h_bytes_per_step": int(u2.numel()) * 4},
        "cpu_baseline": {"value": round(n / host_s / 1e9, 4), "unit": "GB/s", "cores": 1,
                         "kind": "port", "sample": "the whole stream, the library's host encoder "
                                                   "(the reference's ANSEncoder restated), one core"},
        # k_hist, then k_enc_g, k_enc_w, k_enc_scan, k_enc_total, k_enc_final, k_enc_tail
        "gpu_launches": 7 * steps,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)


def run(args, ws, rank, local):
    """Under torchrun every rank runs its own replica of the workload; the
    reported times are the slowest rank's (bench.max_over_ranks)."""
    import torch
    if ws > 1:
        import torch.distributed as dist
        dev = torch.device("cuda", local)
        torch.cuda.set_device(dev)
        dist.init_process_group("nccl", device_id=dev)
    try:
        if args.workload == "encode":
            return run_encode(args, ws, rank, local)
        if args.workload == "batched":
            return run_batched(args, ws, rank, local)
        if args.workload == "served":
            from multians_gb300 import serve_bench
            return serve_bench.run(args, ws, rank, local)
        raise ValueError(args.workload)
    finally:
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
