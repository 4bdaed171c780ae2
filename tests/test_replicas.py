"""Multi-GPU runs are replicas only (one stream's decode does not shard
here): every rank decodes its own stream and the reported times are the
slowest rank's.  This checks that aggregation (bench.max_over_ranks,
bench.replica_rate) with two gloo ranks on the CPU."""
import json
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, outdir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    sys.path.insert(0, ROOT)
    import bench
    # rank r took 1 + r ms for the decode and 10 - r ms end to end
    times = bench.max_over_ranks([1.0 + rank, 10.0 - rank])
    rate = bench.replica_rate(1e9, ws, times[0])
    dist.barrier()
    dist.destroy_process_group()
    with open(os.path.join(outdir, f"r{rank}.json"), "w") as f:
        json.dump({"times": times, "rate": rate}, f)


def test_replica_times_are_the_slowest_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    if not torch.distributed.is_available():
        pytest.skip("torch.distributed is not available")
    ws = 2
    mp.start_processes(_worker, args=(ws, _free_port(), str(tmp_path)), nprocs=ws,
                       join=True, start_method="spawn")
    res = [json.load(open(tmp_path / f"r{r}.json")) for r in range(ws)]
    for r in res:
        assert r["times"] == [2.0, 10.0]           # max over ranks, per value
        assert abs(r["rate"] - 1000.0) < 1e-9      # 2 ranks x 1 GB / 2 ms


def test_single_process_is_the_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks([3.0, 4.5]) == [3.0, 4.5]
    assert bench.replica_rate(2e9, 1, 4.0) == pytest.approx(500.0)
