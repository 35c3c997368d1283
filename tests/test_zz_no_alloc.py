"""The allocation-free flux entry point (ebb_flux_noalloc) against ebb_flux (GPU).

Callers that cannot allocate device memory when they call (a process sharing the GPU
with running solves, where cudaFree would synchronise the device and stall them; a
serving process whose device memory is all reserved) use ebb_flux_noalloc, which
stages through a fixed array compiled into the library instead of allocating.  This
file is collected last
so that a run stopping at the first failure has already run every other test; it
also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from ebbcfd_gb300 import _lib

pytestmark = pytest.mark.gpu


def _states(rng, n):
    rho = rng.uniform(0.2, 3, (n, 2))
    u = rng.uniform(-3, 3, (n, 2))
    v = rng.uniform(-3, 3, (n, 2))
    p = rng.uniform(0.1, 5, (n, 2))
    q = np.stack([rho, rho * u, rho * v, p / 0.4 + 0.5 * rho * (u * u + v * v)], axis=-1)
    th = rng.uniform(0, 2 * np.pi, n)
    return (np.ascontiguousarray(q[:, 0]), np.ascontiguousarray(q[:, 1]),
            np.ascontiguousarray(np.column_stack([np.cos(th), np.sin(th)])))


def _call(fn, kind, qL, qR, nrm):
    n = len(qL)
    F = np.full((n, 4), np.nan)
    s = np.full(n, np.nan)
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    code = fn(kind, n, dp(qL), dp(qR), dp(nrm), dp(F), dp(s))
    return code, F, s


@pytest.mark.parametrize("kind", [1, 0])
def test_noalloc_matches_allocating_entry_point_on_two_calls(kind):
    L = _lib.load()
    rng = np.random.default_rng(100 + kind)
    # two calls in a row with different inputs and sizes; the second fills the array
    for n in (5000, _lib.FLUX_NOALLOC_MAX):
        qL, qR, nrm = _states(rng, n)
        c0, F0, s0 = _call(L.ebb_flux, kind, qL, qR, nrm)
        c1, F1, s1 = _call(L.ebb_flux_noalloc, kind, qL, qR, nrm)
        assert c0 == 0 and c1 == 0
        # the same kernel arithmetic (no fused multiply-adds): bitwise equal
        assert np.array_equal(F1, F0) and np.array_equal(s1, s0)


def test_noalloc_rejects_sizes_beyond_its_limit():
    L = _lib.load()
    n = _lib.FLUX_NOALLOC_MAX + 1
    qL = np.ones((n, 4))
    nrm = np.tile([1.0, 0.0], (n, 1))
    code, F, s = _call(L.ebb_flux_noalloc, 1, qL, qL, nrm)
    assert code == 12  # EBB_ERR_LIMIT
    assert np.isnan(F).all() and np.isnan(s).all()


def test_noalloc_call_leaves_free_device_memory_unchanged():
    """After the first call on the device (its set-up), a call of the largest size
    takes no device memory: the free memory the driver reports is the same before and
    after it."""
    torch = pytest.importorskip("torch")
    L = _lib.load()
    rng = np.random.default_rng(7)
    n = _lib.FLUX_NOALLOC_MAX
    qL, qR, nrm = _states(rng, n)
    code, F0, s0 = _call(L.ebb_flux_noalloc, 1, qL, qR, nrm)  # set-up call
    assert code == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    code, F1, s1 = _call(L.ebb_flux_noalloc, 1, qL, qR, nrm)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert code == 0 and free1 == free0
    assert np.array_equal(F1, F0) and np.array_equal(s1, s0)
