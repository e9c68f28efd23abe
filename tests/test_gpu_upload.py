"""Batched uploads (pq_save_tensors) against one-by-one uploads."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_save_tensors_matches_single_uploads(pq):
    rng = np.random.default_rng(0)
    items = []
    for i, shape in enumerate([(2, 2), (2, 2, 2), (3,), (5, 7, 3), (300, 400), (1,)]):
        a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
        items.append((f"t{i}", a.astype(np.complex64) if i % 2 else a))
    be = pq.GB300Backend(pq.PREC_OZAKI)  # (300, 400) is stored as complex64
    be.save_tensors(items)
    n0 = be.launch_count()
    for lab, a in items:
        got = be.load_tensor_data(lab)
        assert got.shape == a.shape
        tol = 0 if a.size <= 65536 or a.dtype == np.complex64 else 1e-6 * np.abs(a).max()
        assert np.max(np.abs(got - a.astype(np.complex128))) <= tol
    # replacing with the same extents reuses storage; other extents reallocate
    items2 = [(lab, 2 * a) for lab, a in items[:3]] + [("t3", np.ones((4, 4), np.complex128))]
    be.save_tensors(items2)
    for lab, a in items2:
        np.testing.assert_array_equal(be.load_tensor_data(lab), np.asarray(a, np.complex128))
    assert be.launch_count() - n0 == 1  # one scatter launch per batch
    with pytest.raises(pq.PQError):
        be.save_tensors([("x", np.ones(2)), ("x", np.ones(2))])
    be.close()


def test_save_tensors_feeds_a_plan(pq, O):
    """A compiled plan reads leaves re-uploaded by batches."""
    gates = pq.random_grid_gates(2, 3, 4, seed=2)
    be = pq.GB300Backend(pq.PREC_C128)
    net = pq.build_network(6, gates, backend=be)
    pq.add_input(net, "0" * 6)
    plan = pq.NetworkPlan(net, planner="greedy")
    leaves = [(net.nodes[nl].data_label, be.load_tensor_data(net.nodes[nl].data_label)) for nl in plan.leaves]
    for _ in range(3):
        be.save_tensors(leaves)
        plan.execute()
        out = np.asarray(plan.result()).reshape(-1, order="F")
        assert np.max(np.abs(out - O.statevector(6, gates))) < 1e-12
    plan.close()
    be.close()


def test_prepared_uploads_follow_the_arrays(pq):
    """prepare_tensors builds the argument arrays once; save_prepared uploads
    whatever the host arrays hold at that moment (values rewritten in place
    between uploads), and refuses arrays it cannot upload without a copy."""
    rng = np.random.default_rng(3)
    arrs = [np.asfortranarray(rng.standard_normal(s) + 1j * rng.standard_normal(s)).astype(dt)
            for s, dt in (((2, 2), np.complex128), ((2, 2, 2), np.complex64), ((5,), np.complex128))]
    be = pq.GB300Backend(pq.PREC_C64)
    prep = be.prepare_tensors([(f"p{i}", a) for i, a in enumerate(arrs)])
    for step in range(3):
        for a in arrs:
            a[...] = (step + 1) * (rng.standard_normal(a.shape) + 1j * rng.standard_normal(a.shape))
        be.save_prepared(prep)
        for i, a in enumerate(arrs):
            np.testing.assert_array_equal(be.load_tensor_data(f"p{i}"), a.astype(np.complex128))
    with pytest.raises(ValueError):
        be.prepare_tensors([("c", np.ones((3, 4), np.complex128))])  # C-ordered
    with pytest.raises(ValueError):
        be.prepare_tensors([("r", np.ones((2, 2)))])  # real
    be.close()
