"""pq_gather_elements_noalloc: amplitude readout without device allocation.

For hosts that own every device allocation themselves (for example a Julia
process whose CUDA.jl pool must account for all device memory, or an
application under a fixed device-memory budget), the library offers a
gather that stages indices and values in a fixed static device array instead
of allocating per call.  This file checks, through the C ABI, that it returns
what pq_gather_elements returns, on two calls in a row, and that requests
beyond its 65536-index limit are refused.  It is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_ELEMS = 65536


def _gather(be, fn, label, idx, dtype):
    from pqgb300 import _lib as L

    idx = np.ascontiguousarray(idx, dtype=np.int64)
    out = np.empty(idx.size, dtype=dtype)
    dt = L.PQ_C64 if np.dtype(dtype) == np.complex64 else L.PQ_C128
    rc = getattr(be.lib, fn)(be.ctx, be.id_of(label), idx.ctypes.data_as(L.i64p), idx.size,
                             out.ctypes.data_as(C.c_void_p), dt)
    L.check(rc, be.ctx, fn)
    return out


@pytest.mark.parametrize("precision,tol", [(0, 1e-12), (1, 2e-6)], ids=["c128", "c64"])
def test_noalloc_gather_matches_allocating_gather(pq, precision, tol):
    be = pq.GB300Backend(precision)
    rng = np.random.default_rng(precision)
    # a state large enough to be stored as complex64 in the mixed modes
    psi = rng.standard_normal(1 << 17) + 1j * rng.standard_normal(1 << 17)
    be.save_tensor_data("psi", psi.reshape((2,) * 17, order="F"))
    for call, n in enumerate((1024, MAX_ELEMS)):  # two calls in a row
        idx = rng.integers(0, psi.size, n)
        for dtype in (np.complex128, np.complex64):
            ref = _gather(be, "pq_gather_elements", "psi", idx, dtype)
            got = _gather(be, "pq_gather_elements_noalloc", "psi", idx, dtype)
            scale = np.max(np.abs(ref))
            assert np.max(np.abs(got - ref)) <= tol * scale, (call, dtype)
            assert np.max(np.abs(got - psi[idx])) <= 2e-6 * scale
    be.close()


def test_noalloc_gather_rejects_oversize_request(pq):
    from pqgb300 import _lib as L

    be = pq.GB300Backend(pq.PREC_C128)
    be.save_tensor_data("v", np.ones(8))
    with pytest.raises(L.PQError) as e:
        _gather(be, "pq_gather_elements_noalloc", "v", np.zeros(MAX_ELEMS + 1, np.int64), np.complex128)
    assert e.value.code == L.PQ_ERR_INVALID
    assert "65536" in str(e.value)
    # still usable afterwards
    assert np.array_equal(_gather(be, "pq_gather_elements_noalloc", "v", [0, 7], np.complex128), [1, 1])
    be.close()


def test_noalloc_gather_allocates_nothing(pq):
    """The property the entry point exists for: the context's device memory
    in use is the same before and after each call, and with the context's
    memory cap set to exactly what is in use (so any further allocation
    fails) the allocating gather is refused with PQ_ERR_OOM while the
    allocation-free one still returns the right values, twice in a row."""
    from pqgb300 import _lib as L

    be = pq.GB300Backend(pq.PREC_C64)
    rng = np.random.default_rng(11)
    psi = rng.standard_normal(1 << 18) + 1j * rng.standard_normal(1 << 18)
    be.save_tensor_data("psi", psi.reshape((2,) * 18, order="F"))
    used = be.mem_in_use()
    assert used > 0
    for n in (4096, MAX_ELEMS):
        idx = rng.integers(0, psi.size, n)
        got = _gather(be, "pq_gather_elements_noalloc", "psi", idx, np.complex128)
        assert be.mem_in_use() == used
        assert np.max(np.abs(got - psi[idx])) <= 2e-6 * np.max(np.abs(psi))
    be.set_mem_cap(used)
    idx = rng.integers(0, psi.size, 1000)
    with pytest.raises(L.PQError) as e:
        _gather(be, "pq_gather_elements", "psi", idx, np.complex128)
    assert e.value.code == L.PQ_ERR_OOM
    for _ in range(2):
        got = _gather(be, "pq_gather_elements_noalloc", "psi", idx, np.complex64)
        assert be.mem_in_use() == used
        assert np.max(np.abs(got - psi[idx])) <= 2e-6 * np.max(np.abs(psi))
    be.set_mem_cap(0)
    be.close()
