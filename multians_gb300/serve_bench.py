"""Served workload of bench.py: a Poisson stream of decode requests through
the serving loop (mans_server_*).

Trace: 20 000 requests (MANS_SERVE_REQUESTS), Poisson arrivals at a seeded
rate (--rate, requests/s; default 50 000/s, above the loop's capacity, so
the value is the loop's throughput), each naming one stream of a pool of
pre-encoded streams (MANS_SERVE_POOL, default 64): sizes log-uniform in
[1 KB, 64 MB] of uint8 symbols, lambda ~ U[0.005, 2], L in {1024, 4096},
every stream with its own table, all tables resident in the server.  The
pool stands in for 20 000 distinct streams, whose encoding on the host would
take longer than the whole measurement; every request is a full decode.

  value  device-resident requests (MANS_REQ_DEVICE_IO): decoded bytes of
         the trace / (last completion - first arrival)
  e2e    the same trace with page-locked host inputs and outputs: the server
         copies units in and symbols out for every request
  latency_ms          p50/p99 of completion - arrival at half the measured
                      e2e capacity (host buffers)
  latency_ms_saturated  the same under the saturating trace
  bit_exact  a verification replay of the first MANS_SERVE_VERIFY (2000)
             requests in waves in which no two requests share a stream:
             every output compared with its source
  loop_of_plain  the same prefix as one plain decode per request with a
                 status read after each (a request-at-a-time service)
"""
from __future__ import annotations

import concurrent.futures as cf
import ctypes
import json
import os
import time

import numpy as np

METRIC = "decoded GB/s on 1 GB300 (plain vs batched/served) + %HBM roofline; p50/p99; bit-exact"


def pool_specs(seed: int, count: int, lo: float = 1024, hi: float = 64 << 20):
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), count)).astype(np.int64)
    lams = rng.uniform(0.005, 2.0, count)
    Ls = rng.choice([1024, 4096], count)
    return [(seed * 104729 + i, float(lams[i]), int(sizes[i]), int(Ls[i])) for i in range(count)]


def trace(seed: int, n: int, pool: int, rate: float):
    rng = np.random.default_rng(seed + 1)
    entry = rng.integers(0, pool, n)
    offs = np.cumsum(rng.exponential(1.0 / rate, n))
    return entry, (offs * 1e9).astype(np.uint64)


def _np_dtype(cstruct):
    names = [f for f, _ in cstruct._fields_]
    fmt = {ctypes.c_void_p: np.uint64, ctypes.c_uint64: np.uint64, ctypes.c_uint32: np.uint32,
           ctypes.c_int32: np.int32}
    return np.dtype({"names": names,
                     "formats": [fmt[t] for _, t in cstruct._fields_],
                     "offsets": [getattr(cstruct, f).offset for f in names],
                     "itemsize": ctypes.sizeof(cstruct)})


class Replay:
    """Prebuilt request array for one trace and one buffer set."""

    def __init__(self, serve, entry, units_ptr, out_ptr, sts, tids, device_io, capture=True):
        self.serve = serve
        n = entry.size
        self.arr = (serve.RequestC * n)()
        v = np.frombuffer(self.arr, dtype=_np_dtype(serve.RequestC))
        v["units"] = np.asarray(units_ptr, dtype=np.uint64)[entry]
        v["n_units"] = np.array([st.n_units for st in sts], dtype=np.uint64)[entry]
        v["out"] = np.asarray(out_ptr, dtype=np.uint64)[entry]
        v["n_out"] = np.array([st.n for st in sts], dtype=np.uint64)[entry]
        v["table"] = np.asarray(tids, dtype=np.uint32)[entry]
        v["first_state"] = np.array([st.first_state for st in sts], dtype=np.uint32)[entry]
        v["first_bit"] = np.array([st.first_bit for st in sts], dtype=np.uint32)[entry]
        v["flags"] = ((serve.REQ_DEVICE_IO if device_io else 0) |
                      (0 if capture else serve.REQ_NO_CAPTURE))
        v["tag"] = np.arange(n, dtype=np.uint64)
        self.view = v
        self.n = n
        self.cdt = _np_dtype(serve.CompletionC)

    def run(self, srv, offs_ns, count=None, timeout_s=600.0):
        """Submits requests at their arrival times, collects completions;
        returns (arrival_ns, done_ns, status) arrays indexed by tag."""
        n = self.n if count is None else count
        t0 = self.serve.now_ns() + 2_000_000
        arrivals = (offs_ns[:n] + np.uint64(t0)).astype(np.uint64)
        self.view["arrival_ns"][:n] = arrivals
        done = np.zeros(n, dtype=np.uint64)
        status = np.full(n, -1, dtype=np.int64)
        dev_status = np.zeros(n, dtype=np.uint32)
        submitted = completed = 0
        t_end = time.monotonic() + timeout_s
        while completed < n:
            now = self.serve.now_ns()
            k = int(np.searchsorted(arrivals, np.uint64(now), side="right"))
            if k > submitted:
                srv.submit_array(self.arr, submitted, k - submitted)
                submitted = k
            if submitted < n:
                wait = int(min(500, max(0, (int(arrivals[submitted]) - now) // 1000)))
            else:
                wait = 2000
            buf, c = srv.poll_raw(wait_us=wait)
            if c:
                cv = np.frombuffer(buf, dtype=self.cdt, count=c)
                tags = cv["tag"].astype(np.int64)
                done[tags] = cv["done_ns"]
                status[tags] = cv["status"]
                dev_status[tags] = cv["dev_status"]
                completed += c
            if time.monotonic() > t_end:
                raise RuntimeError(f"served trace: {completed}/{n} completions before timeout")
        return arrivals, done, status, dev_status


def _pcts(lat_ns):
    s = np.sort(lat_ns.astype(np.float64)) / 1e6
    return {"p50": round(float(s[len(s) // 2]), 3),
            "p99": round(float(s[min(len(s) - 1, int(0.99 * len(s)))]), 3),
            "mean": round(float(s.mean()), 3), "max": round(float(s[-1]), 3)}


def measure(args, ws, rank, local):
    """The served workload's bench line (None on ranks other than 0)."""
    import torch

    import multians_gb300 as mg
    from multians_gb300 import host, serve
    from multians_gb300.decoder import aux_status, decode_async

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    n_req = int(os.environ.get("MANS_SERVE_REQUESTS", "20000"))
    n_pool = int(os.environ.get("MANS_SERVE_POOL", "64"))
    n_verify = min(n_req, int(os.environ.get("MANS_SERVE_VERIFY", "2000")))
    budget = int(float(os.environ.get("MANS_SERVE_BUDGET_GB", "16")) * (1 << 30))
    rate = float(getattr(args, "rate", 0) or 50_000.0)
    seed = args.seed + rank

    t0 = time.time()
    specs = pool_specs(seed, n_pool)
    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 8) as ex:
        sts = list(ex.map(lambda sp: host.make_stream(*sp), specs))
    gen_s = time.time() - t0
    entry, offs = trace(seed, n_req, n_pool, rate)
    sym_bytes = np.array([st.n for st in sts], dtype=np.int64)
    comp_bytes = np.array([st.n_units * 4 for st in sts], dtype=np.int64)
    total_sym = int(sym_bytes[entry].sum())
    total_comp = int(comp_bytes[entry].sum())

    d_units = [torch.from_numpy(st.units.view(np.int32)).to(dev) for st in sts]
    d_out = [torch.empty(max(1, st.n), dtype=torch.uint8, device=dev) for st in sts]
    h_units = [torch.from_numpy(st.units.view(np.int32)).pin_memory() for st in sts]
    h_out = [torch.empty(max(1, st.n), dtype=torch.uint8).pin_memory() for st in sts]

    inflight = int(os.environ.get("MANS_SERVE_INFLIGHT", "0"))   # 0: the library default
    small = int(os.environ.get("MANS_SERVE_SMALL", "0"))         # 0: the library default
    srv = serve.Server(budget_bytes=budget, max_inflight=inflight, small_bytes=small)
    tids = [srv.add_table(st.table) for st in sts]
    cap = not getattr(args, "no_capture", False)
    rp_dev = Replay(serve, entry, [t.data_ptr() for t in d_units], [t.data_ptr() for t in d_out],
                    sts, tids, device_io=True, capture=cap)
    rp_host = Replay(serve, entry, [t.data_ptr() for t in h_units], [t.data_ptr() for t in h_out],
                     sts, tids, device_io=False, capture=cap)

    # verification replay: waves with no stream twice, every output checked
    ok = True
    i = 0
    vstart = time.time()
    while i < n_verify and ok:
        seen, j = set(), i
        while j < n_verify and int(entry[j]) not in seen:
            seen.add(int(entry[j]))
            j += 1
        for e in seen:
            h_out[e].fill_(0xCD)
        srv.submit_array(rp_host.arr, i, j - i)
        got = srv.wait(j - i, timeout_s=300)
        ok = all(c.status == 0 for c in got)
        for e in seen:
            st = sts[e]
            ok = ok and bool(np.array_equal(h_out[e].numpy()[: st.n][::-1], st.symbols))
        i = j
    verify_s = time.time() - vstart

    # warm-up, then the timed device-resident replays
    for _ in range(max(1, min(args.warmup, 2))):
        rp_dev.run(srv, offs)
    steps = max(1, min(args.steps, 3))
    s0 = srv.stats()
    from bench import ClockSampler
    spans, sat_lat = [], []
    all_ok = True
    with ClockSampler(local) as clk:
        for _ in range(steps):
            arr_ns, done_ns, status, dstat = rp_dev.run(srv, offs)
            all_ok &= bool((status == 0).all())
            spans.append((int(done_ns.max()) - int(arr_ns.min())) / 1e9)
            sat_lat.append(done_ns.astype(np.int64) - arr_ns.astype(np.int64))
    s1 = srv.stats()
    dev_s = sum(spans) / len(spans)

    # e2e: same trace, host buffers (copies in and out inside the server)
    arr_ns, done_ns, status, _ = rp_host.run(srv, offs)
    all_ok &= bool((status == 0).all())
    e2e_s = (int(done_ns.max()) - int(arr_ns.min())) / 1e9
    sat_e2e_lat = done_ns.astype(np.int64) - arr_ns.astype(np.int64)

    # latency at half the measured e2e capacity
    lat_rate = 0.5 * n_req / e2e_s
    entry_lat, offs_lat = trace(seed + 17, n_req, n_pool, lat_rate)
    rp_lat = Replay(serve, entry_lat, [t.data_ptr() for t in h_units],
                    [t.data_ptr() for t in h_out], sts, tids, device_io=False, capture=cap)
    arr_l, done_l, status_l, _ = rp_lat.run(srv, offs_lat)
    all_ok &= bool((status_l == 0).all())
    lat = done_l.astype(np.int64) - arr_l.astype(np.int64)
    lat_bytes = int(sym_bytes[entry_lat].sum())
    # latency by request size: the sizes span 1 KB .. 64 MB, so the tail is
    # the large requests' own decode time plus queueing behind them
    req_sz = sym_bytes[entry_lat]
    by_size = {}
    for name, lo, hi in (("<1MB", 0, 1 << 20), ("1-16MB", 1 << 20, 16 << 20),
                         (">=16MB", 16 << 20, 1 << 62)):
        sel = (req_sz >= lo) & (req_sz < hi)
        if sel.any():
            by_size[name] = dict(_pcts(lat[sel]), requests=int(sel.sum()))
    lat_span = (int(done_l.max()) - int(arr_l.min())) / 1e9
    stats = srv.stats()
    srv.close()

    # a request-at-a-time service with the plain decoder, on the verified prefix
    plans = [mg.plan(st.n_units, st.n, st.L, None if cap else {"flags": mg.DECODE_NO_CAPTURE})
             for st in sts]
    tabs = [torch.from_numpy(st.table.view(np.int32)).to(dev) for st in sts]
    aux = torch.empty(max(mg.aux_size(st.n_units, p) for st, p in zip(sts, plans)),
                      dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    nl = n_verify
    torch.cuda.synchronize(dev)
    lt0 = time.perf_counter()
    for k in range(nl):
        e = int(entry[k])
        st = sts[e]
        decode_async(d_units[e], st.n_units, d_out[e], st.n, tabs[e], st.L, st.first_state,
                     st.first_bit, aux, plans[e], stream=stream)
        aux_status(aux, stream)
    loop_s = time.perf_counter() - lt0
    loop_bytes = int(sym_bytes[entry[:nl]].sum())
    served_prefix_bps = total_sym / dev_s

    if rank != 0:
        return None
    from bench import measured_peaks
    hbm, kind = measured_peaks()
    value = ws * total_sym / dev_s / 1e9
    alg = (total_comp + total_sym) / dev_s / 1e9
    batches = (s1["batches"] - s0["batches"]) / steps
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": ws,
        "steps": steps, "warmup": args.warmup, "ms_per_step": round(dev_s * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic",
        "config": {"workload": f"served {n_req} Poisson requests log-uniform [1KB,64MB] "
                               f"lambda~U[0.005,2] L in {{1024,4096}}, 16 GB budget",
                   "requests": n_req, "pool_streams": n_pool, "rate_rps": rate,
                   "budget_bytes": budget, "n_symbols": total_sym, "compressed_bytes": total_comp,
                   "mean_request_bytes": round(total_sym / n_req), "seed": args.seed,
                   "step": "one replay of the whole trace, device-resident requests",
                   "l2": "inputs larger than L2, no flush"},
        "bit_exact": bool(ok and all_ok), "verified_requests": n_verify,
        "latency_ms": dict(_pcts(lat), load="half the measured e2e capacity",
                           rate_rps=round(lat_rate, 1),
                           achieved_gbs=round(lat_bytes / lat_span / 1e9, 3),
                           by_request_size=by_size),
        "latency_ms_saturated": dict(_pcts(np.concatenate(sat_lat)), e2e=_pcts(sat_e2e_lat)),
        "loop_of_plain": {"requests": nl, "seconds": round(loop_s, 3),
                          "value": round(loop_bytes / loop_s / 1e9, 3),
                          "speedup_served_vs_loop": round((served_prefix_bps * loop_s) / loop_bytes, 3)},
        "roofline": {"bound": "hbm", "kernel": "served batches (4 kernels each)",
                     "achieved": round(alg, 2), "peak": hbm, "peak_kind": kind, "unit": "GB/s",
                     "frac": round(alg / hbm, 4), "traffic": None,
                     "alg_bytes_per_step": total_comp + total_sym},
        "cpu_baseline": None,
        "e2e": {"value": round(ws * total_sym / e2e_s / 1e9, 3), "unit": "GB/s",
                "h2d_bytes_per_step": total_comp, "d2h_bytes_per_step": total_sym},
        "gpu_launches": int(round((s1["kernel_launches"] - s0["kernel_launches"]) / steps)),
        "server": {"small_request_bytes": (0 if small == serve.SMALL_OFF else (small or 1 << 20)),
                   "batches_per_step": round(batches, 1), "largest_batch": stats["largest_batch"],
                   "admission_waits": stats["admission_waits"], "range_peak": stats["range_peak"],
                   "streams_redone": stats["streams_redone"], "failed": stats["failed"]},
        "clocks": clk.summary(),
        "gen_seconds": round(gen_s, 2), "verify_seconds": round(verify_s, 2),
    }
    return line


def run(args, ws, rank, local):
    line = measure(args, ws, rank, local)
    if line is not None:
        print(json.dumps(line), flush=True)

