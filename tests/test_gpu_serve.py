"""GPU tests of the serving loop (mans_server_*): every result is identical
whether its request is decoded alone or batched with others, under memory
pressure (admission waits, blocks reused), with staggered arrivals, and for
device-resident, pageable and failing requests."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pool(n, seed, max_sym=300_000):
    from multians_gb300 import host
    rng = np.random.default_rng(seed)
    pool = []
    for i in range(n):
        size = int(np.exp(rng.uniform(np.log(1_000), np.log(max_sym))))
        lam = float(rng.uniform(0.005, 2.0))
        L = 1024 if i % 2 else 4096
        pool.append(host.make_stream(seed * 1000 + i, lam, size, L))
    return pool


def _pinned(arr_u32_or_u8):
    import torch
    t = torch.from_numpy(arr_u32_or_u8.view(np.int32) if arr_u32_or_u8.dtype == np.uint32
                         else arr_u32_or_u8)
    return t.pin_memory()


def _setup(srv, pool):
    import torch
    items = []
    for st in pool:
        tid = srv.add_table(st.table)
        units = _pinned(st.units)
        out = torch.empty(st.n, dtype=torch.uint8).pin_memory()
        items.append((st, tid, units, out))
    return items


def _req(serve, item, tag, arrival_ns=0):
    st, tid, units, out = item
    return serve.request(units, st.n_units, out, st.n, tid, st.first_state, st.first_bit,
                         tag=tag, arrival_ns=arrival_ns)


def test_identical_alone_and_in_the_mix(mg):
    from multians_gb300 import serve
    pool = _pool(40, seed=3)
    with serve.Server(budget_bytes=2 << 30) as srv:
        items = _setup(srv, pool)
        alone = []
        for i, it in enumerate(items):
            it[3].fill_(0xCD)
            srv.submit([_req(serve, it, i)])
            (c,) = srv.wait(1)
            assert c.tag == i and c.status == 0, c
            alone.append(it[3].numpy().copy())
            assert np.array_equal(alone[-1][::-1], it[0].symbols), i
        single_batches = srv.stats()["batches"]
        assert single_batches == len(items)

        order = np.random.default_rng(9).permutation(len(items))
        for it in items:
            it[3].fill_(0xCD)
        srv.submit([_req(serve, items[i], int(i)) for i in order])
        done = srv.wait(len(items))
        assert sorted(c.tag for c in done) == list(range(len(items)))
        assert all(c.status == 0 for c in done), [c for c in done if c.status]
        for i, it in enumerate(items):
            assert np.array_equal(it[3].numpy(), alone[i]), i
        st = srv.stats()
        assert st["batches"] - single_batches < len(items)   # requests shared launches
        assert st["largest_batch"] > 1
        assert st["failed"] == 0 and st["range_in_use"] > 0   # tables stay resident


def test_small_budget_admission_and_reuse(mg):
    """Only a few requests fit at once: the rest wait in arrival order, blocks
    are reused, and a request larger than the whole range fails alone."""
    import torch

    from multians_gb300 import serve
    pool = _pool(24, seed=5, max_sym=2_000_000)
    budget = 40 << 20
    with serve.Server(budget_bytes=budget, max_inflight=2) as srv:
        items = _setup(srv, pool)
        reqs = [_req(serve, it, i) for i, it in enumerate(items)]
        big = np.zeros(30_000_000, dtype=np.uint32)     # 120 MB of units: never fits
        big_t = torch.from_numpy(big.view(np.int32)).pin_memory()
        big_out = torch.empty(50_000_000, dtype=torch.uint8).pin_memory()
        st0, tid0 = items[0][0], items[0][1]
        reqs.insert(5, serve.request(big_t, big.size, big_out, big_out.numel(), tid0,
                                     st0.first_state, st0.first_bit, tag=999))
        srv.submit(reqs)
        done = {c.tag: c for c in srv.wait(len(reqs), timeout_s=120)}
        assert done[999].status == mg.Status.ERR_NOMEM
        for i, it in enumerate(items):
            assert done[i].status == 0, (i, done[i])
            assert np.array_equal(it[3].numpy()[::-1], it[0].symbols), i
        s = srv.stats()
        assert s["admission_waits"] > 0
        assert s["range_peak"] <= s["range_bytes"] == budget


def test_staggered_arrivals_join_later_launches(mg):
    import time

    from multians_gb300 import serve
    pool = _pool(30, seed=11, max_sym=400_000)
    with serve.Server(budget_bytes=1 << 30) as srv:
        items = _setup(srv, pool)
        for k in range(0, len(items), 5):
            t0 = serve.now_ns()
            srv.submit([_req(serve, items[i], i, arrival_ns=t0)
                        for i in range(k, min(k + 5, len(items)))])
            time.sleep(0.002)
        done = srv.wait(len(items))
        for c in done:
            assert c.status == 0 and c.done_ns >= c.admit_ns >= c.arrival_ns > 0, c
        for st, _, _, out in items:
            assert np.array_equal(out.numpy()[::-1], st.symbols)
        assert srv.stats()["batches"] >= 2


def test_small_requests_batched_apart(mg):
    """Requests of at most small_bytes output go to the small-request slot's
    batches, larger ones to the other slots: submitted together, the two
    classes share no launch; without the small-request slot they share one.
    Requests of one class only still use every slot."""
    from multians_gb300 import serve
    rng = np.random.default_rng(23)
    from multians_gb300 import host
    small = [host.make_stream(2300 + i, float(rng.uniform(0.01, 1.0)), int(rng.integers(2_000, 200_000)),
                              1024) for i in range(8)]
    large = [host.make_stream(2400 + i, float(rng.uniform(0.01, 1.0)), int(rng.integers(1_200_000, 2_500_000)),
                              1024 if i % 2 else 4096) for i in range(4)]
    threshold = 1 << 20
    for small_bytes, apart in ((threshold, True), (serve.SMALL_OFF, False)):
        with serve.Server(budget_bytes=1 << 30, small_bytes=small_bytes) as srv:
            items = _setup(srv, small + large)
            for it in items:
                it[3].fill_(0xCD)
            srv.submit([_req(serve, it, i) for i, it in enumerate(items)])
            done = {c.tag: c for c in srv.wait(len(items))}
            assert all(c.status == 0 for c in done.values()), done
            for st, _, _, out in items:
                assert np.array_equal(out.numpy()[::-1], st.symbols)
            sb = {done[i].batch for i in range(len(small))}
            lb = {done[i].batch for i in range(len(small), len(items))}
            if apart:
                assert sb.isdisjoint(lb), (sb, lb)
                assert len(sb) == 1 and len(lb) == 1   # one launch per class
            else:
                assert sb == lb and len(sb) == 1
            # small requests only, arriving while a batch of them runs: the
            # other slots take them too
            srv.submit([_req(serve, items[i], 100 + i) for i in range(len(small))])
            srv.submit([_req(serve, items[i], 200 + i) for i in range(len(small))])
            again = srv.wait(2 * len(small))
            assert all(c.status == 0 for c in again), again
            for st, _, _, out in items[: len(small)]:
                assert np.array_equal(out.numpy()[::-1], st.symbols)


def test_device_io_pageable_and_errors(mg):
    import torch

    from multians_gb300 import serve
    pool = _pool(3, seed=17, max_sym=200_000)
    with serve.Server(budget_bytes=256 << 20) as srv:
        tids = [srv.add_table(st.table) for st in pool]
        # device-resident request
        st = pool[0]
        du = torch.from_numpy(st.units.view(np.int32)).cuda()
        do = torch.full((st.n,), 0xCD, dtype=torch.uint8, device="cuda")
        r0 = serve.request(du, st.n_units, do, st.n, tids[0], st.first_state, st.first_bit,
                           tag=0, device_io=True)
        # pageable host request (numpy buffers)
        st1 = pool[1]
        hu = np.ascontiguousarray(st1.units)
        ho = np.full(st1.n, 0xCD, dtype=np.uint8)
        r1 = serve.request(hu.ctypes.data, st1.n_units, ho.ctypes.data, st1.n, tids[1],
                           st1.first_state, st1.first_bit, tag=1)
        # unknown table, bad first_state, empty output
        r2 = serve.request(hu.ctypes.data, st1.n_units, ho.ctypes.data, st1.n, 77,
                           st1.first_state, st1.first_bit, tag=2)
        r3 = serve.request(hu.ctypes.data, st1.n_units, ho.ctypes.data, st1.n, tids[1],
                           5, st1.first_bit, tag=3)
        r4 = serve.request(hu.ctypes.data, st1.n_units, ho.ctypes.data, 0, tids[1],
                           st1.first_state, st1.first_bit, tag=4)
        srv.submit([r0, r1, r2, r3, r4])
        done = {c.tag: c for c in srv.wait(5)}
        assert done[0].status == 0 and done[1].status == 0 and done[4].status == 0
        assert done[2].status == mg.Status.ERR_ARG and done[3].status == mg.Status.ERR_ARG
        torch.cuda.synchronize()
        assert np.array_equal(do.cpu().numpy()[::-1], st.symbols)
        assert np.array_equal(ho[::-1], st1.symbols)
        bad = pool[2].table.copy()
        bad[3] = (bad[3] & 0x00FFFFFF) | (20 << 24)
        with pytest.raises(mg.MansError):
            srv.add_table(bad)


def test_source_order_requests(mg):
    """A request can ask for its output in source order; others in the same
    launch keep decode order."""
    from multians_gb300 import serve
    pool = _pool(6, seed=23, max_sym=300_000)
    with serve.Server(budget_bytes=512 << 20) as srv:
        items = _setup(srv, pool)
        reqs = []
        for i, (st, tid, units, out) in enumerate(items):
            reqs.append(serve.request(units, st.n_units, out, st.n, tid, st.first_state,
                                      st.first_bit, tag=i, source_order=bool(i % 2)))
        srv.submit(reqs)
        done = srv.wait(len(reqs))
        assert all(c.status == 0 for c in done)
        for i, (st, _, _, out) in enumerate(items):
            got = out.numpy()
            assert np.array_equal(got if i % 2 else got[::-1], st.symbols), i


def test_container_requests_share_resident_tables(mg):
    """Requests given as containers: the server reads the stream parameters
    from the header and adds each distinct table once."""
    import torch

    from multians_gb300 import container, host, serve
    a = host.make_stream(71, 0.05, 150_000, 1024)
    b = host.encode(host.gen_symbols(72, 0.05, 90_000), 1024)
    with serve.Server(budget_bytes=256 << 20) as srv:
        outs, bufs = [], []
        for i, st in enumerate((a, a, b)):
            c = torch.from_numpy(container.pack_encoded(st)).pin_memory()
            o = torch.full((st.n + 5,), 0xCD, dtype=torch.uint8).pin_memory()
            bufs.append(c)
            outs.append(o)
            srv.submit([serve.request_container(c, o, tag=i, source_order=(i == 2))])
            (done,) = srv.wait(1)
            assert done.status == 0, done
        base = srv.stats()["range_in_use"]
        assert np.array_equal(outs[0].numpy()[: a.n][::-1], a.symbols)
        assert np.array_equal(outs[1].numpy()[: a.n][::-1], a.symbols)
        assert np.array_equal(outs[2].numpy()[: b.n], b.symbols)
        assert (outs[0].numpy()[a.n:] == 0xCD).all()
        # the same table again adds nothing resident
        srv.submit([serve.request_container(bufs[0], outs[0], tag=9)])
        assert srv.wait(1)[0].status == 0
        assert srv.stats()["range_in_use"] == base
