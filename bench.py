"""Benchmark of the MULTIANS decode path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload plain|batched|served|encode] [--mb 256] [--lam 0.05] [--L 1024]

One JSON line on stdout (rank 0).  The default workload is the plain
single-stream decode of a 256 MB stream (lambda = 0.05, L = 1024 states):
seeded synthetic uint8 symbols, the reference's table generator and encoder
(the library's C++ implementation of them), one raw stream.

  value   decoded GB/s (decoded bytes / s) with the stream and the output
          resident in HBM; each step is one full decode (five or six kernels).
  e2e     the same metric through the public C ABI with host buffers: per
          step the pinned-host units and table go host->device, the decode
          runs, the decoded bytes come back device->host; steps pipelined
          over two buffer sets (input copy, decode and output copy of
          neighbouring steps overlap), with the one-stream serial figure
          beside it.
  roofline  the dominant kernel: algorithmic bytes per launch / its mean
          launch time (CUDA events around every kernel in the timed
          region), against the measured HBM copy bandwidth.
  cpu_baseline  the reference's multicore CPU method on the host cores, on
          a bounded sample of the same workload.
  issue_roofline  each kernel's instruction-issue utilisation from the
          committed ncu summary of this workload (profiles/).
  sync    what the synchronisation cost beside the algorithmic bytes:
          units the merge walks decoded a second time, walks handed to the
          walk pass, metadata bytes (read back from the workspace after the
          correctness decode, outside the timed region).

  batched, served  sub-records measured in the same run after the headline
          (leave them out with --no-subrecords): the 4096-stream batch as
          one CUDA-graph replay, with a loop of plain decodes launched from
          C over the same streams beside it (speedup_batched_vs_loop), and
          the 20 000-request Poisson trace through the serving loop with
          p50/p99 latency; each with its own e2e, clocks and bit-exact flag.
          --workload batched|served prints either as the whole line.

Multi-GPU: the decode of one stream does not shard across processes here;
every rank decodes its own replica stream ("replicas only", weak scaling)
and value sums the ranks' decoded bytes over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "decoded GB/s on 1 GB300 (plain vs batched/served) + %HBM roofline; p50/p99; bit-exact"
HBM_FALLBACK_GBS = 6800.0
# Speed of the reference's own MulticoreDecoder build relative to the
# oracle's port of it (which the reference arm times where the reference
# sources are absent): same machine, same threads, same stream.
REFERENCE_VS_PORT = {
    "ratio": round(0.234 / 0.432, 3),
    "how": "x86 container, 8 threads, 32 MiB of the headline workload (lambda=0.05, L=1024): "
           "reference build 0.234 GB/s, port 0.432 GB/s; the port is faster, so a ratio "
           "against the port understates the speed-up over the reference",
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["plain", "batched", "served", "encode"], default="plain")
    ap.add_argument("--mb", type=float, default=256.0, help="stream size in MiB of symbols")
    ap.add_argument("--lam", type=float, default=0.05)
    ap.add_argument("--L", type=int, default=1024)
    ap.add_argument("--seed", type=int, default=20261203)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-capture", action="store_true",
                    help="decode without symbol capture (MANS_DECODE_NO_CAPTURE)")
    ap.add_argument("--seeds", choices=["auto", "on", "off"], default="auto",
                    help="seeded merge walks: the planner's choice, or forced "
                         "(MANS_DECODE_SEEDS / MANS_DECODE_NO_SEEDS)")
    ap.add_argument("--cpu-sample-mb", type=float, default=32.0)
    ap.add_argument("--no-subrecords", action="store_true",
                    help="plain workload: leave out the batched and served sub-records")
    ap.add_argument("--rate", type=float, default=0.0,
                    help="served workload: Poisson arrival rate, requests/s (0 = 50000)")
    return ap.parse_args()


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(prefix="mans_clocks_", suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.out, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.out.close()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for ln in f:
                parts = [x.strip() for x in ln.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(values, device=None):
    """Each value's maximum over the ranks (one all_reduce; the identity in
    a single process): the slowest replica sets a multi-GPU run's times."""
    import torch
    import torch.distributed as dist
    vals = [float(v) for v in values]
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return vals
    t = torch.tensor(vals, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.tolist()]


def replica_rate(per_rank, ws, ms):
    """Whole-job GB/s of ws replicas that each process per_rank bytes, over
    the slowest replica's ms."""
    return ws * per_rank / (ms / 1e3) / 1e9


def workload_config(args, n_symbols, n_units):
    """The `config` both arms print for the plain workload (identical keys
    and values, so the two lines can be matched)."""
    return {"workload": f"plain {args.mb:g}MiB lambda={args.lam} L={args.L}",
            "n_symbols": int(n_symbols), "n_units": int(n_units), "lambda": args.lam,
            "L": args.L, "seed": args.seed}


def planner_report(mg, st, args):
    """Where the decode's plan came from: the measured table entry the
    planner used (multians_gb300/tune.py wrote it from GB300 timings), or the
    model where the table has none or the run fixed the capture."""
    entry = None if args.no_capture else mg.tune_lookup(st.L, st.bits_per_symbol, st.n)
    return {"source": "measured table" if entry else "model", "entry": entry}


def make_workload(args, rank):
    from multians_gb300 import host
    n = int(args.mb * (1 << 20))
    t0 = time.time()
    st = host.make_stream(args.seed + rank, args.lam, n, args.L)
    return st, time.time() - t0


def profile_figures(workload: str, captured: bool):
    """The committed ncu figures of a plain workload (profiles/traffic_*.txt
    and profiles/issue_*.txt, tab-separated rows): the kernel
    each timing slot of the decode stands for (with symbol capture the
    final-pass slot is the copy pass), DRAM bytes per launch and instruction
    issue utilisation (% of cycles) by kernel.  Rows are keyed by kernel,
    workload and capture mode; where no profile of that workload and mode
    is committed the dictionaries are empty (the bench line then says null,
    not another kernel's figure)."""
    key = workload + (" capture" if captured else " no-capture")
    kernel_of = ({"k_gwalk": "k_gwalk<1>", "k_wwalk": "k_wwalk<1>", "k_final": "k_copy<0>"}
                 if captured else
                 {"k_gwalk": "k_gwalk<0>", "k_wwalk": "k_wwalk<0>", "k_final": "k_final<0>"})

    def rows(prefix):
        out = {}
        pdir = os.path.join(ROOT, "profiles")
        names = sorted(os.listdir(pdir)) if os.path.isdir(pdir) else []
        for name in names:
            if not (name.startswith(prefix + "_") and name.endswith(".txt")):
                continue
            with open(os.path.join(pdir, name)) as f:
                for ln in f:
                    parts = ln.rstrip("\n").split("\t")
                    if len(parts) == 3 and not parts[0].startswith("#") and parts[1] == key:
                        out[parts[0]] = parts[2]
        return out

    traffic = {k: int(v) for k, v in rows("traffic").items()}
    issue = {k: float(v) for k, v in rows("issue").items()}
    inst = {k: int(v) for k, v in rows("inst").items()}
    return kernel_of, traffic, issue, inst


def cpu_baseline(st, sample_mb: float):
    """The reference's multicore method (oracle port; the reference build
    when present) on a bounded prefix-sized sample of the same workload."""
    from oracle import oracle as O
    n = min(st.n, int(sample_mb * (1 << 20)))
    sym = st.symbols[:n]
    sst = O.encode(sym, st.L)
    cores = os.cpu_count() or 1
    nsub = (sst.n_units + 3) // 4
    T = max(1, min(cores, nsub))
    use_ref = O.ref_available()
    times = []
    for _ in range(5):
        t0 = time.perf_counter()
        if use_ref:
            out = O.ref_multicore_decode(sst, S=4, T=T)
        else:
            out, _ = O.multicore_decode(sst, S=4, T=T)
        times.append(time.perf_counter() - t0)
    ok = bool((out[::-1] == sym).all())
    t = statistics.median(times)
    return {"value": round(n / t / 1e9, 4), "unit": "GB/s", "cores": T,
            "kind": "reference" if use_ref else "port",
            "sample": f"{n >> 20} MiB prefix of the workload's symbols, re-encoded; "
                      f"MulticoreDecoder method S=4, T={T}; median of 5; bit-exact={ok}"}


def run_reference(args, ws, rank):
    """The reference's own CPU implementation of the path on this workload
    (oracle/_ref when built, else the oracle's restatement of it)."""
    if rank != 0:
        return
    from oracle import oracle as O
    n = int(args.mb * (1 << 20))
    st = O.make_stream(args.seed, args.lam, n, args.L)   # same bytes as the GPU arm's stream
    ost = st
    cores = os.cpu_count() or 1
    T = max(1, min(cores, (st.n_units + 3) // 4))
    use_ref = O.ref_available()
    dec = (lambda: O.ref_multicore_decode(ost, S=4, T=T)) if use_ref else \
        (lambda: O.multicore_decode(ost, S=4, T=T)[0])
    for _ in range(max(0, args.warmup)):
        dec()
    times = []
    out = None
    for _ in range(args.steps):
        t0 = time.perf_counter()
        out = dec()
        times.append(time.perf_counter() - t0)
    ok = bool((out[::-1] == st.symbols).all())
    tot = sum(times)
    v = st.n * len(times) / tot / 1e9
    times_ms = sorted(x * 1e3 for x in times)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "GB/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(tot / len(times) * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
        "config": workload_config(args, st.n, st.n_units),
        "bit_exact": ok,
        "latency_ms": {"p50": round(times_ms[len(times_ms) // 2], 3),
                       "p99": round(times_ms[min(len(times_ms) - 1, int(0.99 * len(times_ms)))], 3)},
        "cpu_baseline": {"value": round(v, 4), "unit": "GB/s", "cores": T,
                         "kind": "reference" if use_ref else "port",
                         "sample": f"the full workload per step; MulticoreDecoder method S=4, T={T}"},
        "e2e": {"value": round(v, 4), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "reference_vs_port": REFERENCE_VS_PORT if not use_ref else
        {"ratio": 1.0, "how": "this run timed the reference's own build"},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, ws, rank, local):
    import numpy as np
    import torch

    import multians_gb300 as mg
    from multians_gb300 import _lib
    from multians_gb300.decoder import decode_async, aux_status

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)

    st, gen_s = make_workload(args, rank)
    n = st.n
    units_h = torch.from_numpy(st.units.view(np.int32)).pin_memory()
    table_h = torch.from_numpy(st.table.view(np.int32)).pin_memory()
    units = units_h.to(dev)
    table = table_h.to(dev)
    out = torch.empty(n, dtype=torch.uint8, device=dev)
    out_h = torch.empty(n, dtype=torch.uint8).pin_memory()
    hint_flags = (mg.DECODE_NO_CAPTURE if args.no_capture else 0) | \
        {"auto": 0, "on": mg.DECODE_SEEDS, "off": mg.DECODE_NO_SEEDS}[args.seeds]
    cfg = mg.plan(st.n_units, n, st.L, {"flags": hint_flags} if hint_flags else None)
    aux = torch.empty(mg.aux_size(st.n_units, cfg), dtype=torch.uint8, device=dev)
    want = torch.from_numpy(np.ascontiguousarray(st.symbols[::-1])).to(dev)
    stream = torch.cuda.current_stream(dev)

    def one():
        decode_async(units, st.n_units, out, n, table, st.L, st.first_state, st.first_bit,
                     aux, cfg, stream=stream)

    # warm-up + correctness
    for _ in range(max(3, args.warmup)):
        one()
    status = aux_status(aux, stream)
    bit_exact = bool(torch.equal(out, want)) and status == 0
    del want
    # what the synchronisation cost beside the algorithmic bytes (read back
    # from the workspace of the last decode; outside every timed region)
    try:
        sync = _lib.sync_stats(aux.data_ptr(), aux.numel(), st.n_units, n, st.L, cfg,
                               stream.cuda_stream)
        sync["reread_bytes"] = 4 * sync["walk_units"]
        sync["reread_frac_of_stream"] = round(sync["walk_units"] / st.n_units, 4)
        sync["host_round_trips"] = 0
    except Exception as e:   # a report field: never fails the bench line
        sync = {"error": str(e)}

    # timed region: device-resident decode
    launches_per = mg.lib().mans_last_launch_count()
    _lib.timing_enable(args.steps)
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        evs[0].record(stream)
        for i in range(args.steps):
            one()
            evs[i + 1].record(stream)
        torch.cuda.synchronize(dev)
    if ws > 1:
        dist.barrier()
    per_ms = [evs[i].elapsed_time(evs[i + 1]) for i in range(args.steps)]
    total_ms = evs[0].elapsed_time(evs[-1])
    kern_ms, kern_n = _lib.timing_collect()
    _lib.timing_enable(0)
    status |= aux_status(aux, stream)
    bit_exact = bit_exact and bool(torch.equal(out, torch.from_numpy(
        np.ascontiguousarray(st.symbols[::-1])).to(dev))) and status == 0
    (total_ms,) = max_over_ranks([total_ms], dev)

    # e2e: host buffers through the C ABI, copies inside the timed region.
    # Serial: per step H2D, decode, D2H on one stream.  Pipelined, the way a
    # streaming caller runs it: two device and two host buffer sets; step
    # i's H2D on an input copy stream, its decode on the compute stream and
    # its D2H on an output copy stream, each waiting only on what it reads
    # or overwrites, so step i+1's input copy and step i-1's output copy run
    # under step i's decode.  Every step still moves its own bytes.
    h2d = st.units.nbytes + st.table.nbytes
    d2h = n
    # the bench's own K steps (the pipeline fills and drains once per run)
    e2e_steps = max(3, args.steps)
    for _ in range(2):
        units.copy_(units_h, non_blocking=True)
        table.copy_(table_h, non_blocking=True)
        one()
        out_h.copy_(out, non_blocking=True)
    torch.cuda.synchronize(dev)
    serial_runs = []
    for _ in range(3):   # median of three runs: the host links are shared with other GPUs
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(e2e_steps):
            units.copy_(units_h, non_blocking=True)
            table.copy_(table_h, non_blocking=True)
            one()
            out_h.copy_(out, non_blocking=True)
        e1.record(stream)
        torch.cuda.synchronize(dev)
        serial_runs.append(e0.elapsed_time(e1) / e2e_steps)
    e2e_serial_ms = statistics.median(serial_runs)
    e2e_ok = bool(np.array_equal(out_h.numpy(), st.symbols[::-1]))

    units2 = [units, torch.empty_like(units)]
    table2 = [table, torch.empty_like(table)]
    out2 = [out, torch.empty_like(out)]
    out_h2 = [out_h, torch.empty(n, dtype=torch.uint8).pin_memory()]
    s_in, s_out = torch.cuda.Stream(dev), torch.cuda.Stream(dev)

    def pipelined(steps):
        ev = lambda: torch.cuda.Event(enable_timing=False)  # noqa: E731
        in_done, dec_done, out_done = [], [], []
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(s_in)
        for i in range(steps):
            k = i & 1
            with torch.cuda.stream(s_in):
                if i >= 2:
                    s_in.wait_event(dec_done[i - 2])   # decode i-2 read units[k]
                units2[k].copy_(units_h, non_blocking=True)
                table2[k].copy_(table_h, non_blocking=True)
                in_done.append(ev())
                in_done[i].record(s_in)
            stream.wait_event(in_done[i])
            if i >= 2:
                stream.wait_event(out_done[i - 2])     # D2H i-2 read out[k]
            decode_async(units2[k], st.n_units, out2[k], n, table2[k], st.L, st.first_state,
                         st.first_bit, aux, cfg, stream=stream)
            dec_done.append(ev())
            dec_done[i].record(stream)
            s_out.wait_event(dec_done[i])
            with torch.cuda.stream(s_out):
                out_h2[k].copy_(out2[k], non_blocking=True)
                out_done.append(ev())
                out_done[i].record(s_out)
        t1.record(s_out)
        torch.cuda.synchronize(dev)
        return t0.elapsed_time(t1) / steps, (steps - 1) & 1

    pipelined(2)
    runs = [pipelined(e2e_steps) for _ in range(3)]
    e2e_ms = statistics.median(r[0] for r in runs)
    last = runs[-1][1]
    e2e_ok = e2e_ok and bool(np.array_equal(out_h2[last].numpy(), st.symbols[::-1]))
    e2e_ok = e2e_ok and aux_status(aux, stream) == 0
    del units2, table2, out2, out_h2
    # the slowest rank's step times, as for the device-resident value
    e2e_ms, e2e_serial_ms = max_over_ranks([e2e_ms, e2e_serial_ms], dev)

    if rank != 0:
        if ws > 1:
            dist.destroy_process_group()
        return

    ms = total_ms / args.steps
    value = replica_rate(n, ws, ms)
    hbm, peak_kind = measured_peaks()
    comp_bytes = st.n_units * 4
    # dominant kernel and its algorithmic bytes per launch
    mean_k = {k: v / max(1, kern_n) for k, v in kern_ms.items()}
    dom = max(mean_k, key=lambda k: mean_k[k])
    # k_gwalk reads the stream once; k_wwalk's re-reads are overhead, not
    # algorithmic bytes; k_final writes the symbols (and without capture
    # reads the stream again; with capture it reads the captured symbols,
    # which like the G pass's capture writes are overhead)
    captured = cfg.get("capture_bytes", 0) > 0
    alg = {"k_gwalk": comp_bytes, "k_wwalk": 0, "k_final": n if captured else comp_bytes + n,
           "k_prep": st.L * 4, "k_scan": 0}[dom]
    achieved = alg / (mean_k[dom] / 1e3) / 1e9
    wl = f"plain {args.mb:g}MiB lambda={args.lam} L={args.L}"
    kernel_of, t_rows, issue, inst = profile_figures(wl, captured)
    traffic = t_rows.get(kernel_of.get(dom))
    per_sorted = sorted(per_ms)
    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_baseline(st, args.cpu_sample_mb)
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
        "data": "synthetic",
        "config": workload_config(args, n, st.n_units),
        "stream": {"compressed_bytes": comp_bytes,
                   "bits_per_symbol": round(st.bits_per_symbol, 4)},
        "geometry": cfg,
        "planner": planner_report(mg, st, args),
        "l2": "inputs larger than L2 (stream + output > 129 MB), no flush",
        "parallelism": "replicas" if ws > 1 else "single",
        "bit_exact": bit_exact,
        "latency_ms": {"p50": round(per_sorted[len(per_sorted) // 2], 4),
                       "p99": round(per_sorted[min(len(per_sorted) - 1,
                                                   int(0.99 * len(per_sorted)))], 4)},
        "decode_roofline": {"bytes": comp_bytes + n,
                            "achieved_gbs": round((comp_bytes + n) / (ms / 1e3) / 1e9, 2),
                            "frac_of_measured": round((comp_bytes + n) / (ms / 1e3) / 1e9 / hbm, 4),
                            "frac_of_8tbs": round((comp_bytes + n) / (ms / 1e3) / 1e9 / 8000, 4)},
        "kernel_ms": {k: round(v, 4) for k, v in mean_k.items()},
        "sync": sync,
        "roofline": {"bound": "hbm", "kernel": kernel_of.get(dom, dom),
                     "timing_slot": dom, "achieved": round(achieved, 2),
                     "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4), "traffic": traffic,
                     "alg_bytes_per_launch": alg},
        "issue_roofline": {"issue_active_pct": issue, "dominant": kernel_of.get(dom, dom),
                           "inst_per_symbol": {k: round(v / n, 2) for k, v in inst.items()},
                           "source": "ncu smsp__issue_active and thread instructions of "
                                     "one-kernel captures of this workload (profiles/)"}
        if issue else None,
        "cpu_baseline": cpu,
        "e2e": {"value": round(replica_rate(n, ws, e2e_ms), 3), "unit": "GB/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "bit_exact": e2e_ok,
                "pipelined": "2 buffer sets; H2D, decode, D2H on 3 streams",
                "serial_value": round(replica_rate(n, ws, e2e_serial_ms), 3)},
        "gpu_launches": launches_per * args.steps,
        "clocks": clk.summary(),
        "gen_seconds": round(gen_s, 2),
    }
    if not args.no_subrecords:
        line.update(subrecords(args, ws, rank, local))
    print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


# keys of a workload line that repeat the headline's and are left out of its
# sub-record
_SUB_DROP = ("metric", "n_gpus", "higher_is_better", "scaling", "vs_baseline", "dtype", "data",
             "warmup")


def subrecords(args, ws, rank, local):
    """The batched (4096 streams) and served (20 000 requests) workloads,
    measured after the plain headline in the same run, as sub-records of its
    line.  Every rank runs them (replicas); rank 0 reports."""
    import torch
    from multians_gb300 import bench_workloads, serve_bench
    out = {}
    for name, fn in (("batched", bench_workloads.measure_batched),
                     ("served", serve_bench.measure)):
        torch.cuda.empty_cache()
        t0 = time.time()
        try:
            sub = fn(args, ws, rank, local)
        except Exception as e:   # a sub-record never costs the headline its line
            sub = {"error": f"{type(e).__name__}: {e}"}
        if sub is not None:
            sub = {k: v for k, v in sub.items() if k not in _SUB_DROP}
            sub["wall_seconds"] = round(time.time() - t0, 1)
            out[name] = sub
    if "batched" in out and "loop_of_plain" in out["batched"]:
        out["speedup_batched_vs_loop"] = out["batched"]["loop_of_plain"].get(
            "speedup_batched_vs_loop")
    return out


def main():
    args = parse()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    if args.workload != "plain":
        from multians_gb300 import bench_workloads
        bench_workloads.run(args, ws, rank, local)
        return
    run_ours(args, ws, rank, local)


if __name__ == "__main__":
    main()
