"""One stream split over several ranks (multians_gb300/shard.py), on the CPU:
world-size 2, 3 and 4 gloo process groups run the exchange protocol with a
sequential slice decoder (the reference's per-symbol step,
src/multians_gpu_decoder.cu:131-167, restated here as test infrastructure)
in place of the GPU, and the concatenated outputs must equal the oracle's
sequential decode and the source byte for byte.  A tiny verification prefix
makes the true and guessed starts fail to meet inside it, so the exact
full-slice query is exercised too."""
import json
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class SeqBackend:
    """Decodes a slice's held units one symbol at a time."""

    def __init__(self, units, table, L):
        self.u = [int(x) for x in units]
        self.t = [int(x) for x in table]
        self.L = L

    def _steps(self, state, first_bit, n_units):
        pos, x, u, t, L = 32 - first_bit, state, self.u, self.t, self.L
        while True:
            yield pos, x
            e = t[x - L]
            k = e >> 24
            i = pos >> 5
            w = (u[i] if i < n_units else 0) | ((u[i + 1] if i + 1 < n_units else 0) << 32)
            x = ((e & 0xFFFF) << k) | ((w >> (pos & 31)) & ((1 << k) - 1))
            pos += k

    def query(self, state, first_bit, n_units, positions):
        out, it, cnt = [], self._steps(state, first_bit, n_units), 0
        pos, x = next(it)
        for q in positions:
            while pos < q and cnt < 64 * 32 * n_units + 64:
                pos, x = next(it)
                cnt += 1
            out.append((pos, x, int(pos >= q), cnt))
        return out

    def decode(self, state, first_bit, n_units, n):
        out, it = np.empty(n, dtype=np.uint8), self._steps(state, first_bit, n_units)
        for i in range(n):
            _, x = next(it)
            out[i] = (self.t[x - self.L] >> 16) & 0xFF
        return out


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, outdir, stream_file, prefix_units):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    sys.path.insert(0, ROOT)
    from multians_gb300 import shard
    d = np.load(stream_file)
    units, table = d["units"], d["table"]
    n_units, n, L, fs, fb = (int(x) for x in d["meta"])
    sl = shard.make_slice(n_units, n, L, fs, fb, ws, rank)
    be = SeqBackend(units[sl.u0: sl.u0 + sl.units_held], table, L)
    off, out, info = shard.decode_sharded(be, sl, prefix_units=prefix_units)
    dist.barrier()
    dist.destroy_process_group()
    np.save(os.path.join(outdir, f"out{rank}.npy"), out if out is not None else np.empty(0, np.uint8))
    with open(os.path.join(outdir, f"info{rank}.json"), "w") as f:
        json.dump(dict(info, offset=off), f)


@pytest.mark.parametrize("ws,lam,L,prefix", [(2, 0.05, 1024, None), (3, 1.0, 1024, None),
                                             (2, 0.2, 4096, 2), (4, 2.0, 1024, 3)])
def test_sharded_decode_matches_the_oracle(tmp_path, oracle_lib, ws, lam, L, prefix):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    if not torch.distributed.is_available():
        pytest.skip("torch.distributed is not available")
    O = oracle_lib
    st = O.make_stream(seed=77 + ws, lam=lam, n=40_000, L=L)
    f = str(tmp_path / "stream.npz")
    np.savez(f, units=st.units, table=st.table,
             meta=np.array([st.n_units, st.n, st.L, st.first_state, st.first_bit], np.int64))
    mp.start_processes(_worker, args=(ws, _free_port(), str(tmp_path), f, prefix), nprocs=ws,
                       join=True, start_method="spawn")
    infos = [json.load(open(tmp_path / f"info{r}.json")) for r in range(ws)]
    parts = [np.load(tmp_path / f"out{r}.npy") for r in range(ws)]
    assert [i["offset"] for i in infos] == list(np.cumsum([0] + [p.size for p in parts[:-1]]))
    got = np.concatenate(parts)
    assert np.array_equal(got, O.decode_seq(st))
    assert np.array_equal(got[::-1], st.symbols)
    if prefix is not None:
        assert any(i["full_slice_queries"] for i in infos[1:])


def test_slice_bounds():
    sys.path.insert(0, ROOT)
    from multians_gb300 import shard
    for n_units in (100, 1001, 50_339_428):
        for ws in (1, 2, 3, 8):
            b = [shard.slice_bounds(n_units, ws, r) for r in range(ws)]
            assert b[0][0] == 0 and b[-1][1] == n_units
            assert all(b[i][1] == b[i + 1][0] for i in range(ws - 1))
            assert all(u0 % shard.SLICE_ALIGN == 0 for u0, _ in b)
    with pytest.raises(ValueError):
        shard.make_slice(8, 30, 1024, 1024, 32, 4, 1)
