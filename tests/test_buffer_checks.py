"""Buffer checks of the Python mirror (no GPU).  The C calls see only
addresses, so a tensor shorter than the sizes passed, on the wrong side of
the host/device split, or not contiguous is refused in Python before any C
call is made.  Stand-in tensors are used: every case here raises before an
address could be used."""
import pytest


class _Dev:
    index = None


class Fake:
    """Duck-typed tensor of `nbytes` bytes (never dereferenced)."""

    def __init__(self, nbytes, cuda=True, contiguous=True):
        self._n = nbytes
        self.is_cuda = cuda
        self._contiguous = contiguous
        self.device = _Dev()

    def numel(self):
        return self._n

    def element_size(self):
        return 1

    def is_contiguous(self):
        return self._contiguous

    def data_ptr(self):
        return 0x10000


N_UNITS, N_OUT, L = 1000, 5000, 1024


@pytest.mark.parametrize("bad,what", [
    ({"units": Fake(4 * N_UNITS - 1)}, "units"),
    ({"out": Fake(N_OUT - 1)}, "out"),
    ({"table": Fake(4 * L - 4)}, "table"),
    ({"units": Fake(4 * N_UNITS, cuda=False)}, "CUDA"),
    ({"out": Fake(N_OUT, contiguous=False)}, "contiguous"),
])
def test_decode_async_refuses_bad_buffers(mg, bad, what):
    from multians_gb300.decoder import decode_async
    args = {"units": Fake(4 * N_UNITS), "out": Fake(N_OUT), "table": Fake(4 * L)}
    args.update(bad)
    with pytest.raises(ValueError, match=what):
        decode_async(args["units"], N_UNITS, args["out"], N_OUT, args["table"], L, L, 7,
                     Fake(1 << 20))


@pytest.mark.parametrize("bad,what", [
    ({"units": Fake(4 * N_UNITS - 4)}, "units"),
    ({"out": Fake(N_OUT - 1)}, "out"),
    ({"table": Fake(4 * L - 1)}, "table"),
])
def test_batch_desc_refuses_short_buffers(mg, bad, what):
    from multians_gb300 import batch
    args = {"units": Fake(4 * N_UNITS), "out": Fake(N_OUT), "table": Fake(4 * L)}
    args.update(bad)
    with pytest.raises(ValueError, match=what):
        batch.desc(args["units"], N_UNITS, args["out"], N_OUT, args["table"], L, L, 7)


def test_batch_desc_sizing_only_and_exact_sizes(mg):
    from multians_gb300 import batch
    d = batch.desc(None, N_UNITS, None, N_OUT, None, L, L, 7)
    assert (d.d_units, d.n_units, d.n_out, d.L) == (None, N_UNITS, N_OUT, L)
    d = batch.desc(Fake(4 * N_UNITS), N_UNITS, Fake(N_OUT), N_OUT, Fake(4 * L), L, L, 7)
    assert d.d_units == d.d_out == d.d_table == 0x10000
    d = batch.desc(Fake(4 * N_UNITS), N_UNITS, Fake(0), 0, Fake(4 * L), L, L, 7)
    assert d.n_out == 0


def test_server_request_checks(mg):
    from multians_gb300 import serve
    host_u, host_o = Fake(4 * N_UNITS, cuda=False), Fake(N_OUT, cuda=False)
    r = serve.request(host_u, N_UNITS, host_o, N_OUT, 0, L, 7)
    assert (r.units, r.n_units, r.n_out, r.flags) == (0x10000, N_UNITS, N_OUT, 0)
    r = serve.request(Fake(4 * N_UNITS), N_UNITS, Fake(N_OUT), N_OUT, 0, L, 7, device_io=True)
    assert r.flags & serve.REQ_DEVICE_IO
    r = serve.request(0x2000, N_UNITS, 0x3000, N_OUT, 0, L, 7)   # raw addresses pass as is
    assert (r.units, r.out) == (0x2000, 0x3000)
    with pytest.raises(ValueError, match="units"):
        serve.request(Fake(4 * N_UNITS - 1, cuda=False), N_UNITS, host_o, N_OUT, 0, L, 7)
    with pytest.raises(ValueError, match="out"):
        serve.request(host_u, N_UNITS, Fake(N_OUT - 1, cuda=False), N_OUT, 0, L, 7)
    with pytest.raises(ValueError, match="host"):
        serve.request(Fake(4 * N_UNITS), N_UNITS, host_o, N_OUT, 0, L, 7)
    with pytest.raises(ValueError, match="CUDA"):
        serve.request(host_u, N_UNITS, host_o, N_OUT, 0, L, 7, device_io=True)
    with pytest.raises(ValueError, match="host"):
        serve.request_container(Fake(4096), host_o)
    r = serve.request_container(Fake(4096, cuda=False), host_o, tag=3)
    assert (r.n_units, r.n_out, r.flags, r.tag) == (4096, N_OUT, serve.REQ_CONTAINER, 3)
