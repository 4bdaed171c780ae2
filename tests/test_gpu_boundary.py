"""GPU tests of the boundary calls that manage memory for the caller:
mans_aux_alloc / mans_aux_free, mans_table_upload / mans_table_free and the
one-call batch decode mans_decode_batch."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int32)).to("cuda")


def test_aux_alloc_and_table_upload(mg, oracle_lib):
    import torch

    from multians_gb300._lib import Cfg, check
    O = oracle_lib
    lib = mg.lib()
    for lam in (0.05, 2.0):
        st = O.make_stream(seed=8100 + int(lam * 10), lam=lam, n=250_000, L=1024)
        tab = np.ascontiguousarray(st.table, dtype=np.uint32)
        d_tab = ctypes.c_void_p()
        check(lib.mans_table_upload(tab.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                    st.L, ctypes.byref(d_tab)), "mans_table_upload")
        aux = ctypes.c_void_p()
        nbytes = ctypes.c_size_t()
        check(lib.mans_aux_alloc(st.n_units, st.n, st.L, None, ctypes.byref(aux),
                                 ctypes.byref(nbytes)), "mans_aux_alloc")
        plan = mg.plan(st.n_units, st.n, st.L)
        assert nbytes.value == mg.aux_size(st.n_units, plan)
        units = _dev(st.units)
        out = torch.full((st.n,), 0xAB, dtype=torch.uint8, device="cuda")
        stream = torch.cuda.current_stream()
        check(lib.mans_decode(units.data_ptr(), st.n_units, out.data_ptr(), st.n, d_tab.value,
                              st.L, st.first_state, st.first_bit, aux.value, nbytes.value,
                              ctypes.byref(Cfg(**plan)), ctypes.c_void_p(stream.cuda_stream)),
              "mans_decode")
        s = ctypes.c_uint32()
        check(lib.mans_aux_status(aux.value, ctypes.c_void_p(stream.cuda_stream),
                                  ctypes.byref(s)), "mans_aux_status")
        assert s.value == 0
        assert np.array_equal(out.cpu().numpy()[::-1], st.symbols)
        assert lib.mans_aux_free(aux.value) == 0
        assert lib.mans_table_free(d_tab.value) == 0


def test_decode_batch_one_call(mg, oracle_lib):
    import torch

    from multians_gb300 import batch
    O = oracle_lib
    sts = [O.make_stream(seed=8200 + i, lam=lam, n=n, L=L)
           for i, (lam, n, L) in enumerate([(0.05, 120_000, 1024), (2.0, 80_000, 4096),
                                            (0.2, 3_000, 1024), (0.005, 50_000, 1024)])]
    keep, descs = [], []
    for i, st in enumerate(sts):
        u, t = _dev(st.units), _dev(st.table)
        o = torch.full((st.n,), 0xAB, dtype=torch.uint8, device="cuda")
        keep.append((u, t, o))
        descs.append(batch.desc(u, st.n_units, o, st.n, t, st.L, st.first_state, st.first_bit,
                                source_order=bool(i & 1)))
    acc, per = batch.decode_batch(descs, stream=torch.cuda.current_stream())
    assert acc == 0 and per == [0] * len(sts)
    for i, (st, (_, _, o)) in enumerate(zip(sts, keep)):
        got = o.cpu().numpy()
        assert np.array_equal(got if i & 1 else got[::-1], st.symbols), i
