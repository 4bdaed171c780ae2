"""GPU side of splitting one stream over ranks: the trajectory query
(mans_trajectory_query) against a sequential decode, and the sharded decode
(multians_gb300/shard.py) with two processes on this GPU exchanging over
gloo (every kernel is launched by one process and waits on nothing of the
other's; the exchange is host-side), its concatenated output byte for byte
equal to the oracle's sequential decode and the source."""
import json
import os
import socket
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).to("cuda")


@pytest.mark.parametrize("L,lam", [(1024, 0.05), (4096, 1.0), (1024, 2.0)])
def test_trajectory_query_matches_sequential_decode(mg, oracle_lib, L, lam):
    from multians_gb300 import shard
    from test_shard import SeqBackend
    O = oracle_lib
    st = O.make_stream(seed=L + int(100 * lam), lam=lam, n=150_000, L=L)
    be = shard.GpuBackend(_dev(st.units), _dev(st.table), L, n_out_hint=st.n)
    seq = SeqBackend(st.units, st.table, L)
    end = 32 * st.n_units
    qs = sorted({0, 5, 32, 1000, 4097, end // 3, end // 2 + 7, end - 40, end - 1, end})
    for start in ((st.first_state, st.first_bit), (st.first_state, 32), (L + 17, 25)):
        got = be.query(start[0], start[1], st.n_units, qs)
        want = seq.query(start[0], start[1], st.n_units, qs)
        assert got == want, start
    # from the true start the count at the stream end is the symbol count less
    # any zero-bit codewords sitting exactly at the end
    pos, state, found, count = be.query(st.first_state, st.first_bit, st.n_units, [end])[0]
    assert found and count <= st.n


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, outdir, stream_file):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.cuda.set_device(0)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    sys.path.insert(0, ROOT)
    from multians_gb300 import shard
    d = np.load(stream_file)
    n_units, n, L, fs, fb = (int(x) for x in d["meta"])
    sl = shard.make_slice(n_units, n, L, fs, fb, ws, rank)
    held = d["units"][sl.u0: sl.u0 + sl.units_held]
    units = torch.from_numpy(np.ascontiguousarray(held).view(np.int32)).cuda()
    table = torch.from_numpy(d["table"].view(np.int32)).cuda()
    be = shard.GpuBackend(units, table, L, n_out_hint=n // ws)
    off, out, info = shard.decode_sharded(be, sl)
    dist.barrier()
    dist.destroy_process_group()
    np.save(os.path.join(outdir, f"out{rank}.npy"), out.cpu().numpy())
    with open(os.path.join(outdir, f"info{rank}.json"), "w") as f:
        json.dump(dict(info, offset=off), f)


@pytest.mark.parametrize("lam,L,mib", [(0.05, 1024, 16), (1.0, 4096, 4)])
def test_sharded_decode_two_ranks(tmp_path, oracle_lib, lam, L, mib):
    import torch.multiprocessing as mp
    O = oracle_lib
    st = O.make_stream(seed=int(lam * 100) + L, lam=lam, n=mib << 20, L=L)
    f = str(tmp_path / "stream.npz")
    np.savez(f, units=st.units, table=st.table,
             meta=np.array([st.n_units, st.n, st.L, st.first_state, st.first_bit], np.int64))
    ws = 2
    mp.start_processes(_worker, args=(ws, _free_port(), str(tmp_path), f), nprocs=ws,
                       join=True, start_method="spawn")
    infos = [json.load(open(tmp_path / f"info{r}.json")) for r in range(ws)]
    got = np.concatenate([np.load(tmp_path / f"out{r}.npy") for r in range(ws)])
    assert infos[1]["offset"] == infos[0]["count"]
    assert np.array_equal(got, O.decode_seq(st))
    assert np.array_equal(got[::-1], st.symbols)
