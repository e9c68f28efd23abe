"""Device-side failure reporting, exercised without a GPU fault.

The tensor-core kernels bound every mbarrier wait; an expired wait is
written to the context's status word and surfaces as PQ_ERR_DEVICE at the
next synchronising call, after which the context must keep working (the
reference raises an error and carries on, src/backends/interactive.jl:44-49).
``pq_selftest_wait_expiry`` runs one wait that nobody completes, with a short
poll limit and nothing else in flight, through the same reporting helper.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATUS_TC_TIMEOUT = 0x7C01


def _expire(be, polls):
    flag = C.c_int(-1)
    rc = be.lib.pq_selftest_wait_expiry(be.ctx, polls, C.byref(flag))
    return rc, flag.value


@pytest.mark.parametrize("precision", [5, 0], ids=["ozaki", "c128"])
def test_expired_wait_reports_device_error_then_recovers(pq, O, precision):
    from pqgb300 import _lib as L

    be = pq.GB300Backend(precision)
    rc, expired = _expire(be, 1024)
    assert rc == L.PQ_OK and expired == 1
    with pytest.raises(L.PQError) as e:
        be.sync()
    assert e.value.code == L.PQ_ERR_DEVICE
    assert str(STATUS_TC_TIMEOUT) in str(e.value)
    be.sync()  # reported once, then cleared
    # the context still contracts correctly, on the tensor-core class too
    rng = np.random.default_rng(3)
    A = (rng.standard_normal((512, 64)) + 1j * rng.standard_normal((512, 64))).astype(np.complex64)
    B = rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64))
    be.save_tensor_data("a", A)
    be.save_tensor_data("b", B)
    be.contract_tensors("a", [-1, 1], "b", [1, -2], "c")
    got = np.asarray(be.load_tensor_data("c"))
    ref = O.contract_tensors_arrays(np.asarray(A, dtype=np.complex128), [-1, 1], B, [1, -2])
    tol = 1e-12 if precision == 0 else 1e-6
    assert np.max(np.abs(got - ref)) <= tol * np.max(np.abs(ref))
    be.close()


def test_expired_wait_surfaces_through_a_plan_run(pq):
    """The status word is checked by every synchronising call, not only
    pq_ctx_sync: a plan execution after an expiry reports it, and the next
    one succeeds with the right result."""
    from pqgb300 import _lib as L

    be = pq.GB300Backend(pq.PREC_C128)
    gates = pq.random_grid_gates(2, 2, 3, seed=1)
    net = pq.build_network(4, gates, backend=be)
    pq.add_input(net, "0000")
    plan = pq.NetworkPlan(net, planner="wavefunction")
    plan.execute()
    ref = np.asarray(plan.result()).copy()
    _expire(be, 64)
    with pytest.raises(L.PQError) as e:
        plan.execute()
        plan.result()
    assert e.value.code == L.PQ_ERR_DEVICE
    plan.execute()
    assert np.allclose(plan.result(), ref, rtol=0, atol=1e-13)
    plan.close()
    be.close()


def test_selftest_rejects_bad_poll_limits(pq):
    from pqgb300 import _lib as L

    be = pq.GB300Backend(pq.PREC_C128)
    for polls in (0, (1 << 20) + 1):
        rc, _ = _expire(be, polls)
        assert rc == L.PQ_ERR_INVALID
    be.sync()
    be.close()
