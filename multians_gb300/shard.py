"""One stream decoded by several GPUs, one process per GPU.

The reference decodes a stream on one GPU: its phase 1 starts every
subsequence from a guessed state, phase 2 repairs the seams on the host
until every subsequence's last codeword matches its successor's
(src/multians_gpu_decoder.cu:195-466, 617-656), and an exclusive scan of the
per-subsequence counts places the output (:658-670).  Here the same method
runs at the granularity of GPUs, with the single-GPU decoder doing the work
inside each slice:

  1. rank r holds units [u0, u1) of the stream (plus a few units of halo
     past u1, which the codewords that straddle the slice end read) and
     decodes its slice from a guessed start (rank 0 from the stream's true
     start): the trajectory query gives its first codeword at or after the
     slice end (the exit: bit offset into the next slice and state) and the
     symbols before it, and where it stands after a prefix of W units;
  2. the ranks exchange their exits (16 bytes each);
  3. rank r > 0 takes its predecessor's exit as the true entry of its slice
     and queries the decode from there at the end of the prefix: when both
     starts stand at the same bit in the same state, they decode alike from
     there on (the fact the whole method rests on), so the slice's true
     symbol count is the true start's count to that point plus the guessed
     start's from there to the exit, and the exit is the guessed start's.
     If they have not met, the true start is queried at the slice end
     itself (exact, one more pass over the slice);
  4. the counts are exchanged and each rank's output offset is their
     exclusive prefix sum (rounds repeat only if some rank's exit changed in
     step 3, at most once per rank);
  5. each rank decodes its slice from the true entry, exactly its count of
     symbols, with the plain decoder: its part of the output in decode order
     (the reference's order), at its offset.

The exchange steps are the only communication: two all-gathers of a few
integers per rank, no decoder data.  Kernels never wait on another rank.
The last rank's count is the stream's symbol count less the others' (the
stream may end in zero-bit codewords at its very end, which no exit counts).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

HALO_UNITS = 4      # codewords read at most 16 bits past the slice end
SLICE_ALIGN = 4     # units: slices start on 16-byte boundaries (TMA copies)


@dataclass
class Slice:
    rank: int
    world: int
    u0: int            # first unit of the slice
    u1: int            # one past its last unit
    n_units: int       # units of the whole stream
    n_out: int         # symbols of the whole stream
    L: int
    first_state: int   # the stream's first state (rank 0's true start, the others' guess)
    first_bit: int

    @property
    def units_held(self) -> int:
        """Units the rank holds: the slice and its halo, within the stream."""
        return min(self.u1 + HALO_UNITS, self.n_units) - self.u0


def slice_bounds(n_units: int, world: int, rank: int) -> tuple[int, int]:
    """Even split of n_units units over `world` ranks, on 4-unit boundaries."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank outside the world")
    edges = [min(n_units, (n_units * i // world) // SLICE_ALIGN * SLICE_ALIGN)
             for i in range(world)] + [n_units]
    return edges[rank], edges[rank + 1]


def make_slice(n_units, n_out, L, first_state, first_bit, world, rank) -> Slice:
    u0, u1 = slice_bounds(n_units, world, rank)
    if u1 - u0 < 2 * SLICE_ALIGN and world > 1:
        raise ValueError("stream too short to split over this many ranks")
    return Slice(rank, world, u0, u1, n_units, n_out, L, first_state, first_bit)


class GpuBackend:
    """Slice decoder on this process's GPU through the C ABI: trajectory
    queries (mans_trajectory_query) and the plain decode (mans_decode_sync).
    units: CUDA int32/uint32 tensor of the slice's held units, 16-byte
    aligned; table: CUDA tensor of the L decoder words."""

    def __init__(self, units, table, L: int, n_out_hint: int = 0):
        from ._lib import lib
        self.units, self.table, self.L = units, table, int(L)
        self.n_out_hint = int(n_out_hint)
        self._lib = lib()
        f = self._lib.mans_trajectory_query
        f.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_uint32,
                      ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_size_t,
                      ctypes.c_void_p,
                      ctypes.c_size_t, ctypes.POINTER(ctypes.c_uint64), ctypes.c_uint32,
                      ctypes.POINTER(Point), ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32)]
        f.restype = ctypes.c_int
        g = self._lib.mans_trajectory_aux_size
        g.argtypes = [ctypes.c_size_t, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_uint32]
        g.restype = ctypes.c_size_t

    def query(self, state: int, first_bit: int, n_units: int, positions, flags: int = 0,
              units=None, table=None):
        import torch

        from ._lib import MansError
        from .decoder import _dev_ptr, _stream_ptr
        units = self.units if units is None else units
        table = self.table if table is None else table
        nq = len(positions)
        need = self._lib.mans_trajectory_aux_size(n_units, self.n_out_hint, self.L, nq)
        aux = torch.empty(need, dtype=torch.uint8, device=units.device)
        q = (ctypes.c_uint64 * nq)(*[int(x) for x in positions])
        out = (Point * nq)()
        st = ctypes.c_uint32(0)
        rc = self._lib.mans_trajectory_query(
            _dev_ptr(units, 4 * n_units, "units"), n_units,
            _dev_ptr(table, 4 * self.L, "table"), self.L, int(state), int(first_bit), int(flags),
            self.n_out_hint, _dev_ptr(aux), need, q, nq, out, _stream_ptr(None),
            ctypes.byref(st))
        if rc:
            raise MansError(rc, f"mans_trajectory_query (device status 0x{st.value:x})")
        return [(p.pos, p.state, p.found, p.count) for p in out]

    def decode(self, state: int, first_bit: int, n_units: int, n_out: int):
        from .decoder import decode
        return decode(self.units, n_units, n_out, self.table, int(state), int(first_bit),
                      L=self.L)


class Point(ctypes.Structure):
    _fields_ = [("pos", ctypes.c_uint64), ("state", ctypes.c_uint32),
                ("found", ctypes.c_uint32), ("count", ctypes.c_uint64)]


def _allgather(vals, group=None):
    """Each rank's list of ints, on every rank (identity without a process
    group).  Host integers travel as one int64 tensor per rank."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return [list(vals)]
    dev = torch.device("cpu")
    if dist.get_backend(group) == "nccl":
        dev = torch.device("cuda", torch.cuda.current_device())
    t = torch.tensor([int(v) for v in vals], dtype=torch.int64, device=dev)
    out = [torch.empty_like(t) for _ in range(dist.get_world_size(group))]
    dist.all_gather(out, t, group=group)
    return [[int(v) for v in x.tolist()] for x in out]


def decode_sharded(backend, sl: Slice, group=None, prefix_units: int | None = None):
    """Runs the protocol above for this rank's slice; returns (offset,
    symbols, info): the rank's part of the stream's decode-order output
    starting at global index `offset`, and what the protocol did."""
    S = sl.u1 - sl.u0
    held = sl.units_held
    end_bit = 32 * S
    W = prefix_units if prefix_units is not None else max(4096, 8 * sl.L)
    W = max(1, min(W, S))
    # 1. the slice from its own start: exit and the prefix point
    if sl.rank == 0:
        own = (sl.first_state, sl.first_bit)
    else:
        own = (sl.first_state, 32)   # guessed state at bit 0 of the slice
    gW, gX = backend.query(own[0], own[1], held, [32 * W, end_bit])
    if not gX[2]:
        raise RuntimeError(f"rank {sl.rank}: the decode does not reach its slice end")

    def exit_of(pt):
        return [pt[0] - end_bit, pt[1]]

    exit_r = exit_of(gX)
    count_r = gX[3]
    entry_used = None
    rounds = 0
    full_queries = 0
    for rounds in range(1, sl.world + 1):
        exits = _allgather(exit_r, group)
        changed = 0
        if sl.rank > 0 and exits[sl.rank - 1] != entry_used:
            entry_used = exits[sl.rank - 1]
            off, state = entry_used
            if not 0 <= off < 32:
                raise RuntimeError(f"rank {sl.rank}: predecessor's exit {off} bits into the slice")
            # 3. the true start of this slice, at the end of the prefix
            # the true start up to the prefix end only: units past it unread
            tW = backend.query(state, 32 - off, min(held, W + HALO_UNITS), [32 * W])[0]
            if tW[2] and (tW[0], tW[1]) == (gW[0], gW[1]):
                new_count, new_exit = tW[3] + gX[3] - gW[3], exit_of(gX)
            else:
                tX = backend.query(state, 32 - off, held, [end_bit])[0]
                full_queries += 1
                if not tX[2]:
                    raise RuntimeError(f"rank {sl.rank}: the decode does not reach its slice end")
                new_count, new_exit = tX[3], exit_of(tX)
            changed = int(new_exit != exit_r)
            count_r, exit_r = new_count, new_exit
        if not any(x[0] for x in _allgather([changed], group)):
            break
    # 4. output offsets
    counts = [x[0] for x in _allgather([count_r], group)]
    offset = sum(counts[: sl.rank])
    n = sl.n_out - offset if sl.rank == sl.world - 1 else count_r
    if n < 0 or offset + n > sl.n_out:
        raise RuntimeError(f"rank {sl.rank}: slice counts exceed the stream ({offset} + {n})")
    # 5. the slice from its true entry
    if sl.rank == 0:
        start = own
    else:
        start = (entry_used[1], 32 - entry_used[0])
    out = backend.decode(start[0], start[1], held, n) if n else None
    info = {"rounds": rounds, "prefix_units": W, "full_slice_queries": full_queries,
            "count": n, "offset": offset}
    return offset, out, info
