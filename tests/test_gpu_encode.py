"""GPU encoder parity: units, unit count, first bit and first state equal
the host encoder's (the reference's ANSEncoder restated, pinned to the
reference build) bit for bit, and the streams decode back to the source."""
import hashlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _golden_cases():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return [c for c in json.load(f)["cases"] if c["n"] <= (1 << 22)]


def _check(mg, st, chunk=0):
    from multians_gb300 import encode
    units, n_units, fb, fs, dec = encode.encode(st.symbols, st.L, chunk=chunk)
    assert np.array_equal(dec, st.table)
    assert (n_units, fb, fs) == (st.n_units, st.first_bit, st.first_state)
    got = units.cpu().numpy().view(np.uint32)
    assert np.array_equal(got, st.units), np.nonzero(got != st.units)[0][:10]
    return units


@pytest.mark.parametrize("L", [1024, 4096])
@pytest.mark.parametrize("lam", [0.005, 0.05, 0.5, 2.0])
def test_gpu_encode_matches_host_encoder(mg, L, lam):
    from multians_gb300 import host
    st = host.make_stream(int(lam * 1000) + L, lam, 1_000_003, L)
    units = _check(mg, st)
    got = mg.decode(units, st.n_units, st.n, st.table, st.first_state, st.first_bit, L=L)
    assert np.array_equal(got.cpu().numpy()[::-1], st.symbols)


@pytest.mark.parametrize("n", [1, 2, 3, 15, 16, 17, 255, 256, 257, 4095, 4097, 100_000])
def test_gpu_encode_small(mg, n):
    from multians_gb300 import host
    for lam, L in ((0.05, 1024), (2.0, 4096)):
        _check(mg, host.make_stream(n * 13 + 7, lam, n, L))


@pytest.mark.parametrize("chunk", [256, 768, 2048])
def test_gpu_encode_short_chunks_cross_chunks(mg, chunk):
    """Chunks shorter than the merge distance: walks cross chunks (a
    second cursor replays the next chunk's trajectory)."""
    from multians_gb300 import host
    for lam, L in ((0.5, 1024), (0.05, 4096), (2.0, 1024)):
        st = host.make_stream(int(lam * 77) + chunk, lam, 300_001, L)
        try:
            _check(mg, st, chunk=chunk)
        except mg.MansError as e:   # merges longer than the slots reach
            assert e.code == mg.Status.ERR_SYNC
            _check(mg, st)          # the re-planning entry point still encodes exactly


def test_gpu_encode_matches_reference_encoder(mg, oracle_lib):
    """Against the reference's own encoder (built from its sources)."""
    O = oracle_lib
    if not O.ref_available():
        pytest.skip("reference build not available")
    from multians_gb300 import encode
    for lam, L in ((0.05, 1024), (0.9, 4096)):
        sym = O.gen_symbols(123, lam, 500_000)
        ref = O.ref_encode(sym, L)
        units, n_units, fb, fs, dec = encode.encode(sym, L)
        assert (n_units, fb, fs) == (ref.n_units, ref.first_bit, ref.first_state)
        assert np.array_equal(units.cpu().numpy().view(np.uint32), ref.units)


@pytest.mark.parametrize("case", _golden_cases(),
                         ids=lambda c: f"s{c['seed']}_l{c['lambda']}_n{c['n']}_L{c['L']}")
def test_gpu_encode_matches_reference_goldens(mg, oracle_lib, case):
    """The golden hashes come from the reference's own encoder (built from
    its sources when the fixtures were made): the GPU encoder's units,
    table and stream parameters hash the same."""
    from multians_gb300 import encode
    sym = oracle_lib.gen_symbols(case["seed"], case["lambda"], case["n"])
    units, n_units, fb, fs, dec = encode.encode(sym, case["L"])
    sha = lambda a: hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()
    assert (n_units, fb, fs) == (case["n_units"], case["first_bit"], case["first_state"])
    assert sha(units.cpu().numpy().view(np.uint32)) == case["sha_units"]
    assert sha(dec) == case["sha_table"]
