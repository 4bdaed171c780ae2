"""CPU tests: the library's own table generator and encoder (C++, used by
the benchmark and the serving harness) against the oracle and the golden
fixtures, bit for bit."""
import hashlib
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("L", [256, 1024, 2048, 4096, 8192])
@pytest.mark.parametrize("lam", [0.005, 0.05, 0.2, 1.0, 2.0])
def test_library_encoder_matches_oracle(mg, oracle_lib, L, lam):
    from multians_gb300 import host
    O = oracle_lib
    for n in (1, 2, 3, 1000, 65_537):
        seed = int(lam * 977) + n + L
        a = host.gen_symbols(seed, lam, n)
        b = O.gen_symbols(seed, lam, n)
        assert np.array_equal(a, b)
        x = host.encode(a, L)
        y = O.encode(b, L)
        assert (x.n_units, x.first_bit, x.first_state) == (y.n_units, y.first_bit, y.first_state)
        assert np.array_equal(x.units, y.units)
        assert np.array_equal(x.table, y.table)


def test_library_encoder_matches_golden(mg):
    from multians_gb300 import host
    with open(os.path.join(HERE, "golden", "golden.json")) as f:
        cases = json.load(f)["cases"]
    for c in cases:
        if c["n"] > (1 << 20):
            continue
        sym = host.gen_symbols(c["seed"], c["lambda"], c["n"])
        assert sha(sym) == c["sha_symbols"]
        st = host.encode(sym, c["L"])
        assert (st.n_units, st.first_bit, st.first_state) == (c["n_units"], c["first_bit"], c["first_state"])
        assert sha(st.units) == c["sha_units"]
        assert sha(st.table) == c["sha_table"]


def test_library_encoder_matches_reference_build(mg, oracle_lib):
    O = oracle_lib
    if not O.ref_available():
        pytest.skip("reference sources not built here")
    from multians_gb300 import host
    for lam, L, n in ((0.05, 1024, 300_001), (2.0, 4096, 200_003), (0.005, 4096, 77_777)):
        sym = host.gen_symbols(99, lam, n)
        x = host.encode(sym, L)
        r = O.ref_encode(sym, L)
        assert (x.n_units, x.first_bit, x.first_state) == (r.n_units, r.first_bit, r.first_state)
        assert np.array_equal(x.units, r.units)
        assert np.array_equal(x.table, r.table)
