"""Multi-table streams: one bitstream whose source segments were each
encoded with their own table, decoded on one GPU.

The reference names multi-table decoding as future work (README.md:11) and
defines no format.  The format here: one unit array (CUHDInputBuffer order)
and the stream's first state and bit, as for a single-table stream; per
segment, in decode order (the source's last segment first), its table (L
states, the same L for all), its symbol count and the bit position of its
first codeword.  The decoder state carries from one segment into the next
(the encoder ran on through the segment end with the next table), so a
segment's start state is not stored: it is where the previous segment's
decode ends.

Decoding keeps the method's parallelism across segments, as the
multi-GPU split does across ranks (multians_gb300/shard.py):

  1. every segment is decoded (sync passes only, trajectory queries) from
     its own start bit with a guessed state (the first segment from the
     stream's true start): its state at its end, and where it stands after a
     prefix of W units;
  2. segment by segment on the host, the true start state of segment j is
     the previous segment's end state; the decode from it is queried at the
     end of the prefix and, where it stands at the same bit in the same
     state as the guessed start, the guessed start's end state is the true
     one (else the true start is queried at the segment end);
  3. one batched decode (mans_decode_batch) writes every segment from its
     true start with its own table, each at its offset in the output.

Segments start at any bit: their units are addressed from the 16-byte
aligned unit at most 3 units before the start (MANS_DECODE_START_OFFSET).
"""
from __future__ import annotations

import numpy as np

from .shard import HALO_UNITS, GpuBackend


def _aligned_view(start_bit: int):
    ua = (start_bit // 32) & ~3
    return ua, start_bit - 32 * ua


def _zero_bit_steps(table, L, state, n, j):
    """The state after n more codewords that read no bits (table words
    {next_state, symbol, bits = 0}: the next state is next_state)."""
    from ._lib import MansError, Status
    if n < 0 or n > 256 * L:
        raise MansError(Status.ERR_SYNC, f"decode_segments: segment {j} count mismatch ({n})")
    for _ in range(n):
        e = int(table[state - L])
        if e >> 24:
            raise MansError(Status.ERR_SYNC, f"decode_segments: segment {j} does not end on "
                                             f"its count")
        state = e & 0xFFFF
    return state


def decode_segments(units, n_units: int, first_state: int, first_bit: int, L: int, tables,
                    counts, starts, prefix_units: int | None = None, stream=None):
    """Decodes a multi-table stream; returns the symbols (CUDA uint8) in
    decode order, every segment's in turn.  units: CUDA tensor of the
    stream's units (16-byte aligned); tables: host uint32 arrays of L words,
    counts: symbols, starts: first-codeword bit positions, all in decode
    order (starts[0] = 32 - first_bit).  Returns (symbols, info)."""
    import torch

    import multians_gb300 as mg
    from . import batch
    from ._lib import DECODE_START_OFFSET, MansError, Status
    n_seg = len(tables)
    if not (len(counts) == len(starts) == n_seg) or n_seg == 0:
        raise ValueError("one table, count and start per segment")
    if int(starts[0]) != 32 - int(first_bit):
        raise ValueError("the first segment starts where the stream does")
    if any(int(b) > int(a) for a, b in zip(starts[1:], starts[:-1])):
        raise ValueError("segment starts must not decrease")
    dev = units.device
    tabs_h = [np.ascontiguousarray(t, dtype=np.uint32) for t in tables]
    for t in tabs_h:
        if t.size != L or mg.table_check(t) < 0:
            raise MansError(Status.ERR_TABLE, "decode_segments: segment table")
    tabs = [torch.from_numpy(t.view(np.int32)).to(dev) for t in tabs_h]
    end_bits = [int(x) for x in starts[1:]] + [32 * n_units]
    W = prefix_units if prefix_units is not None else max(4096, 8 * L)
    be = GpuBackend(units, tabs[0], L)
    views = []
    for j in range(n_seg):
        ua, off = _aligned_view(int(starts[j]))
        held = min((end_bits[j] + 31) // 32 + HALO_UNITS, n_units) - ua
        views.append((ua, off, held, end_bits[j] - 32 * ua))

    def q(j, state, positions, n_units_view):
        ua, off, _, _ = views[j]
        be.n_out_hint = max(1, int(counts[j]))
        return be.query(state, off, n_units_view, positions, flags=DECODE_START_OFFSET,
                        units=units[ua:], table=tabs[j])

    single = [mg.table_check(t) == 1 for t in tabs_h]
    # a single-symbol table's decoder words are zero-bit self loops, while
    # the reference generator's encoder table still moves the state: what
    # follows such a segment in decode order cannot be chained
    if any(single[:-1]):
        raise MansError(Status.ERR_TABLE, "decode_segments: a single-symbol table is allowed "
                                          "only in the last segment (decode order)")
    # 1. every segment but the last from a guessed state (the first from the
    #    true start): where it stands after the prefix and at its end
    guess = [None] * n_seg
    for j in range(n_seg - 1):
        ua, off, held, end_rel = views[j]
        if counts[j] == 0:
            continue
        w = min(end_rel, off + 32 * W)
        guess[j] = (w, *q(j, first_state, [w, end_rel], held))
    # 2. the true start states, segment by segment
    state = int(first_state)
    entry, full = [], 0
    for j in range(n_seg):
        entry.append(state)
        if j == n_seg - 1:
            break
        ua, off, held, end_rel = views[j]
        if counts[j] == 0:
            continue   # an empty segment: the state carries over
        w, gW, gX = guess[j]
        if state == first_state:
            tX, t_end = gX, gX[3]   # the guessed start was the true one
        else:
            # the true start up to the prefix end only: units past it unread
            tW = q(j, state, [w], min(held, (w + 31) // 32 + HALO_UNITS))[0]
            if tW[2] and (tW[0], tW[1]) == (gW[0], gW[1]):
                tX, t_end = gX, tW[3] + gX[3] - gW[3]
            else:
                tX = q(j, state, [end_rel], held)[0]
                t_end, full = tX[3], full + 1
        if not tX[2] or tX[0] != end_rel:
            raise MansError(Status.ERR_SYNC, f"decode_segments: segment {j} does not end "
                                             f"at the next segment's start")
        # the segment may end in zero-bit codewords at the next one's start
        # bit (the split is by symbol count): step them with its own table
        state = _zero_bit_steps(tabs_h[j], L, tX[1], int(counts[j]) - t_end, j)
    # 3. one batched decode, every segment from its true start
    total = int(sum(int(c) for c in counts))
    out = torch.empty(max(1, total), dtype=torch.uint8, device=dev)
    descs, o = [], 0
    for j in range(n_seg):
        ua, off, held, _ = views[j]
        n = int(counts[j])
        if n:
            d = batch.desc(units[ua:], held, out[o: o + n], n, tabs[j], L, entry[j], off)
            d.flags |= DECODE_START_OFFSET
            descs.append(d)
        o += n
    acc, per = batch.decode_batch(descs, stream=stream or torch.cuda.current_stream(dev))
    if acc & ~mg.DEV_DEGENERATE:
        raise MansError(Status.ERR_SYNC, f"decode_segments: device status 0x{acc:x}")
    return out[:total], {"segments": n_seg, "prefix_units": W, "full_segment_queries": full,
                         "entry_states": entry}
