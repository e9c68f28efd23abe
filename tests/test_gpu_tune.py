"""The autotuner: every kernel choice it can install computes the same
contraction (against the FP64 oracle), the tuned choice is never slower
than the fixed rule's, and the persisted table is keyed by GPU and kernels.

Tolerances (max-abs error over max |C|): 1e-6 for the exact-accumulation
tensor-core class and the FP32 SIMT kernels on complex64 storage.
"""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (A dims, A labels, B dims, B labels): the headline's boundary x gate-column
# shape at reduced height, the same with A contiguous along K, a 16-wide
# gate column, and a two-qubit gate on a state vector (skinny class)
SHAPES = [
    ([1 << 12, 16, 16], [-1, 1, 2], [16, 16, 256], [1, 2, -2]),
    ([16, 16, 1 << 12], [1, 2, -1], [16, 16, 256], [1, 2, -2]),
    ([1 << 14, 256], [-1, 1], [256, 16], [1, -2]),
    ([2] * 16, [-(i + 1) for i in range(3)] + [1, 2] + [-(i + 4) for i in range(11)], [2, 2, 2, 2], [1, 2, -15, -16]),
]


def _rand(rng, dims, dtype):
    return (rng.standard_normal(dims) + 1j * rng.standard_normal(dims)).astype(dtype)


def _to_pair(la, lb):
    """ncon labels -> positive integer labels for the tuner (shared label
    values kept equal)."""
    m = {}
    for x in list(la) + list(lb):
        m.setdefault(x, len(m))
    return [m[x] for x in la], [m[x] for x in lb]


@pytest.mark.parametrize("shape", range(len(SHAPES)))
def test_every_tuning_choice_matches_oracle(pq, O, shape):
    from pqgb300 import autotune as AT

    da, ia, db, ib = SHAPES[shape]
    be = pq.GB300Backend(pq.PREC_OZAKI)
    t = AT.Tuner(be)
    pa, pb = _to_pair(ia, ib)
    key, cands = t.classify(pa, da, pb, db)
    assert len(cands) >= 2
    rng = np.random.default_rng(shape)
    A = _rand(rng, da, np.complex64)
    B = rng.standard_normal(db) + 1j * rng.standard_normal(db)
    ref = O.contract_tensors_arrays(np.asarray(A, dtype=np.complex128), ia, B, ib)
    for c in cands:
        t.install({key: c})
        be.save_tensor_data("a", A)
        be.save_tensor_data("b", B)
        be.contract_tensors("a", ia, "b", ib, "c")
        got = np.asarray(be.load_tensor_data("c"))
        err = float(np.max(np.abs(got - ref)) / np.max(np.abs(ref)))
        assert err <= 1e-6, (AT.choice_name(c), err)
    be.close()


def test_tuned_choice_not_slower_than_default(pq):
    from pqgb300 import autotune as AT

    be = pq.GB300Backend(pq.PREC_OZAKI)
    t = AT.Tuner(be)
    for da, ia, db, ib in SHAPES:
        pa, pb = _to_pair(ia, ib)
        key = t.tune_pair(pa, da, pb, db, reps=5)
        e = t.entries[key]
        shape = (np.array([len(pa)], np.int32), np.array([len(pb)], np.int32), np.array(pa + pb, np.int32),
                 np.array(list(da) + list(db), np.int64))
        best, default = tuple(e["choice"]), tuple(e["default"])
        tb, td = [], []
        for _ in range(3):  # interleaved re-measurement
            tb.append(t._time(key, best, shape, 5))
            td.append(t._time(key, default, shape, 5))
        assert min(tb) <= 1.10 * min(td), (AT.choice_name(best), tb, AT.choice_name(default), td)
    t.install()
    assert be.tuning_size() == len(t.entries) == len(SHAPES)
    be.close()


def test_tuning_cache_keyed_by_gpu_and_sources(pq, tmp_path):
    from pqgb300 import autotune as AT

    be = pq.GB300Backend(pq.PREC_OZAKI)
    t = AT.Tuner(be)
    da, ia, db, ib = SHAPES[2]
    pa, pb = _to_pair(ia, ib)
    key = t.tune_pair(pa, da, pb, db, reps=2)
    path = t.save(tmp_path / "cache.json")
    t2 = AT.Tuner(be)
    assert t2.load(path) and t2.entries[key]["choice"] == t.entries[key]["choice"]
    data = json.loads(path.read_text())
    assert data["gpu"] == AT.device_name(0) and data["source_hash"] == AT.source_hash()
    data["source_hash"] = "0" * 16  # tuned for other kernels: ignored
    path.write_text(json.dumps(data))
    assert not AT.Tuner(be).load(path)
    be.close()


def test_tuned_plan_same_amplitude(pq, O):
    """A sliced amplitude contracted with a plan compiled under the tuned
    table equals the one under the fixed rules and the oracle's."""
    from pqgb300 import autotune as AT

    rows, cols, depth = 4, 4, 10
    n = rows * cols
    gates = pq.random_grid_gates(rows, cols, depth, seed=3)
    bits = pq.random_bitstrings(n, 1, seed=4)[0]
    amps = []
    for tuned in (False, True):
        be = pq.GB300Backend(pq.PREC_OZAKI)
        net = pq.build_network(n, gates, decompose=True, backend=be)
        pq.add_input(net, "0" * n)
        pq.add_output(net, bits)
        steps, _, _, _ = pq.planning.best_flop_plan(net, out_edges=[], candidates=("sweep",))
        if tuned:
            p0 = pq.NetworkPlan(net, steps=steps, out_edges=[])
            AT.ensure_tuned(be, [p0], reps=2, save=False)
            p0.close()
        plan = pq.NetworkPlan(net, steps=steps, out_edges=[])
        sl = plan.choose_slices(max_sliced=4, log2_target=0.0)
        amps.append(plan.run_sliced(sl, batch=16))
        plan.close()
        be.close()
    ref = O.statevector(n, O.random_grid_gates(rows, cols, depth, seed=3))[O.amplitude_index(bits)]
    for a in amps:
        assert abs(a - ref) <= 2e-6 * abs(ref) + 1e-9 * 2.0 ** (-n / 2)
