"""State transfer through the C ABI: a state upload from inside a page-locked buffer
from ebb_host_alloc (16-byte aligned) is read by the device directly, with no
staging copy; any other upload, and every download, goes through a staging array.
Both give the same bits, in the caller's cell order, for the whole arena and for one
instance of a batch."""
import ctypes as C

import numpy as np
import pytest

import ebbcfd_gb300 as E
from ebbcfd_gb300 import _lib
from tests.cases import case

pytestmark = pytest.mark.gpu


class Pinned:
    def __init__(self, n_doubles):
        self.L = _lib.load()
        self.p = C.c_void_p()
        assert self.L.ebb_host_alloc(8 * n_doubles, C.byref(self.p)) == 0
        self.a = np.ctypeslib.as_array((C.c_double * n_doubles).from_address(self.p.value))

    def ptr(self, offset=0):
        return C.cast(self.p.value + 8 * offset, C.POINTER(C.c_double))

    def close(self):
        self.L.ebb_host_free(self.p)


@pytest.mark.parametrize("precision,off", [("fp64", 8), ("split", 8), ("fp64", 7)])
def test_pinned_state_round_trip(precision, off):
    """off = 8 doubles: a 16-byte aligned interior pointer, read directly; off = 7:
    not 16-byte aligned, so the upload stages through device memory."""
    c = case("bump_roe_tvd")
    m = c.product_mesh()
    cfg = E.load_config(c.text)
    s = E.UfvmSolver(m, cfg, precision)
    L = _lib.load()
    n = 4 * s.n_cells
    rng = np.random.default_rng(5)
    q = s.state * (1 + 0.01 * rng.uniform(-1, 1, (s.n_cells, 4)))
    buf = Pinned(n + 12)
    buf.a[off:off + n] = q.reshape(-1)
    assert L.ebb_set_state(s.h, buf.ptr(off)) == 0
    assert np.array_equal(s.state, q)  # read back through the staging path
    s.run(3, records=False)
    want = s.state
    buf.a[:] = -1.0
    assert L.ebb_get_state(s.h, buf.ptr(off)) == 0
    assert np.array_equal(buf.a[off:off + n].reshape(-1, 4), want)
    assert (buf.a[:off] == -1.0).all() and (buf.a[off + n:] == -1.0).all()
    # the same run from the staged path gives the same bits
    s2 = E.UfvmSolver(m, cfg, precision)
    s2.set_state(q)
    s2.run(3, records=False)
    assert np.array_equal(s2.state, want)
    s2.close()
    s.close()
    buf.close()


def test_pinned_instance_state_of_a_batch():
    c = case("bump_roe_tvd")
    m = c.product_mesh()
    cfg = E.load_config(c.text)
    b = E.UfvmBatch([m, m, m], [cfg, cfg, cfg], "split")
    L = _lib.load()
    nc = m.n_cells
    q = b.instance_state(1) * 1.01
    buf = Pinned(4 * nc)
    buf.a[:] = q.reshape(-1)
    assert L.ebb_batch_set_state(b.h, 1, buf.ptr()) == 0
    assert np.array_equal(b.instance_state(1), q)
    assert np.array_equal(b.instance_state(0), b.instance_state(2))
    b.run(2, records=False)
    buf.a[:] = 0.0
    assert L.ebb_batch_get_state(b.h, 1, buf.ptr()) == 0
    assert np.array_equal(buf.a.reshape(-1, 4), b.instance_state(1))
    b.close()
    buf.close()
