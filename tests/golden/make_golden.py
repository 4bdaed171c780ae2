"""Generates tests/golden/golden.json and the small array fixtures from the
reference's own host code (oracle/_ref, built from the reference sources by
oracle/Makefile).  Run where the reference sources exist:

    python tests/golden/make_golden.py

Each case: symbols from the seeded generator (oracle.gen_symbols), then the
reference table generator + encoder (with the two shims of
oracle/ref_shim.cc) and the reference MulticoreDecoder (S=4, T=4).
Recorded: stream facts and SHA-256 digests of the symbols, units, table,
the decoded output (the source reversed) and the multicore decoder's
output, with a flag telling whether the latter equals the source (it does
not when a thread interval is shorter than the sync distance: a thread can
latch "synchronised" against a start its neighbour rewrites later in the
same pass, multicore_decoder.cc:57-75, 109-111, 232-233).
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402

CASES = [
    # (seed, lambda, n, L)
    (42, 0.05, 16_384, 1024),
    (42, 0.005, 65_536, 1024),
    (43, 0.2, 65_536, 1024),
    (44, 1.0, 65_536, 1024),
    (45, 2.0, 65_536, 1024),
    (46, 0.005, 65_536, 4096),
    (47, 0.05, 65_536, 4096),
    (48, 0.2, 65_536, 4096),
    (49, 1.0, 65_536, 4096),
    (50, 2.0, 65_536, 4096),
    (51, 0.05, 1 << 20, 1024),
    (52, 2.0, 1 << 20, 4096),
    (60, 0.05, 1, 1024),
    (61, 0.05, 2, 1024),
    (62, 2.0, 3, 1024),
    (63, 0.3, 1000, 1024),
]
ARRAY_CASES = [(42, 0.05, 16_384, 1024), (63, 0.3, 1000, 1024), (45, 2.0, 65_536, 1024)]


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def main():
    O.build(ref=True)
    assert O.ref_available()
    out = []
    for seed, lam, n, L in CASES:
        sym = O.gen_symbols(seed, lam, n)
        st = O.ref_encode(sym, L)
        S, T = 4, 4
        nsub = (st.n_units + S - 1) // S
        T = max(1, min(T, nsub))
        seq = O.decode_seq(st)
        single = int(np.unique(sym).size) == 1
        # the reference multicore decoder never returns on a single-symbol
        # table (every state is a zero-bit self loop)
        dec = seq if single else O.ref_multicore_decode(st, S=S, T=T)
        assert np.array_equal(seq[::-1], sym), (seed, lam, n, L)
        out.append({
            "seed": seed, "lambda": lam, "n": n, "L": L,
            "n_units": st.n_units, "first_bit": st.first_bit, "first_state": st.first_state,
            "sha_symbols": sha(sym), "sha_units": sha(st.units), "sha_table": sha(st.table),
            "sha_decoded": sha(seq), "sha_multicore": sha(dec),
            "multicore_matches_source": None if single else bool(np.array_equal(dec[::-1], sym)),
            "multicore_S": S, "multicore_T": T,
        })
        if (seed, lam, n, L) in ARRAY_CASES:
            np.savez_compressed(os.path.join(HERE, f"case_{seed}_{lam}_{n}_{L}.npz"),
                                symbols=sym, units=st.units, table=st.table,
                                decoded=seq, multicore=dec, meta=np.array([st.n_units, st.first_bit,
                                                            st.first_state], dtype=np.int64))
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump({"generator": "oracle.gen_symbols + reference host code (oracle/_ref)",
                   "table_seed": O.TABLE_SEED, "cases": out}, f, indent=1)
    print(f"wrote {len(out)} cases")


if __name__ == "__main__":
    main()
