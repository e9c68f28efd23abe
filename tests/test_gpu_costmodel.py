"""Learned cost model: the library's MLP kernels against the FP64 oracle
(gradients, forward, bf16 inference), GPU training, the pair-timing
harness, and the learned planner (amplitudes equal across plans)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def be(pq):
    b = pq.GB300Backend(pq.PREC_C64)
    yield b
    b.close()


def test_mlp_gradients_match_oracle(pq, be):
    import mlp_oracle as MO
    from pqgb300.costmodel import CostModel

    m = CostModel(be, hidden=32, layers=3, seed=3)
    rng = np.random.default_rng(0)
    X = rng.standard_normal((257, 5)).astype(np.float32)
    y = rng.standard_normal(257).astype(np.float32)
    g, loss = m.gradients(X, y)
    lo, go = MO.loss_and_grad(m.params.astype(np.float64), X, y, 5, 32, 3)
    assert abs(loss - lo) <= 1e-5 * max(1.0, abs(lo))
    # fp32 kernels vs FP64 oracle
    assert np.max(np.abs(g - go)) <= 1e-4 * max(1.0, np.max(np.abs(go)))
    m.close()


def test_mlp_forward_fp32_and_bf16(pq, be):
    import mlp_oracle as MO
    from pqgb300.costmodel import CostModel

    m = CostModel(be, hidden=128, layers=3, seed=1)
    rng = np.random.default_rng(1)
    X = rng.standard_normal((1000, 5)).astype(np.float32)
    ref = MO.forward(m.params, X, 5, 128, 3)[-1][:, 0]
    f32 = m.predict(X, bf16=False)
    b16 = m.predict(X, bf16=True)
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(f32 - ref)) <= 1e-4 * scale
    assert np.max(np.abs(b16 - ref)) <= 5e-2 * scale  # bf16 weights and activations
    m.close()


def test_mlp_training_reduces_loss(pq, be):
    from pqgb300.costmodel import CostModel

    rng = np.random.default_rng(2)
    X = rng.uniform(0, 1.5, (8192, 5)).astype(np.float32)
    y = (np.log1p(np.exp(4 * X[:, 0] - 2)) + 0.5 * X[:, 1] * X[:, 2] - X[:, 3]).astype(np.float32)
    m = CostModel(be, seed=0)
    _, l0 = m.gradients(X, y)
    l1 = m.train(X, y, epochs=30, batch=256, lr=2e-3, seed=0)
    _, l2 = m.gradients(X, y)
    assert l2 < 0.05 * l0 and l2 < 0.05, (l0, l1, l2)
    m.close()


def test_measure_pairs(pq, be):
    from pqgb300 import costmodel as CM

    shapes = CM.random_pair_shapes(64, seed=5, max_log2=18)
    ms, feats = CM.measure_pairs(be, shapes, reps=2)
    assert np.all(ms > 0) and np.all(np.isfinite(ms))
    a_r, b_r, lab, dims = shapes
    pos = 0
    for p in range(len(a_r)):
        da = dims[pos:pos + a_r[p]]
        pos += a_r[p]
        db = dims[pos:pos + b_r[p]]
        pos += b_r[p]
        assert abs(feats[p, 0] - np.log2(np.prod(da))) < 1e-9
        assert abs(feats[p, 1] - np.log2(np.prod(db))) < 1e-9
    X = CM.model_inputs(feats)
    assert X.shape == (64, 5) and np.all(np.isfinite(X))


def test_learned_plan_amplitudes_agree_with_flop_plan(pq, O, be):
    from pqgb300 import costmodel as CM

    # a quickly trained model is enough to exercise ranking + execution
    shapes = CM.random_pair_shapes(2000, seed=7, max_log2=18)
    ms, feats = CM.measure_pairs(be, shapes, reps=1)
    model = CM.CostModel(be, seed=0)
    model.train(CM.model_inputs(feats), np.log(np.maximum(ms, 1e-4) * 1e3), epochs=20, batch=256)
    r, c, d = 3, 4, 8
    bits = "011010011100"
    g = pq.random_grid_gates(r, c, d, seed=12)
    net = pq.build_network(r * c, g, backend=be, decompose=True)
    pq.add_input(net, "0" * (r * c))
    pq.add_output(net, bits)
    chosen, best_flop, cands = CM.learned_plan(net, model, out_edges=[], n_random=6)
    assert chosen["cmacs"] <= 8.0 * best_flop["cmacs"]
    ref = O.statevector(r * c, g)[O.amplitude_index(bits)]
    for plan_d in (chosen, best_flop):
        p = pq.NetworkPlan(net, steps=plan_d["steps"], out_edges=[])
        p.execute()
        amp = complex(np.asarray(p.result()).reshape(-1)[0])
        assert abs(amp - ref) / 2.0 ** -6 < 1e-6
        p.close()
    model.close()


def test_sliced_features_and_slicing_set_ranking(pq, O, be):
    """Sliced step features: with no slicing they are the plan's own; with
    slicing the per-amplitude work they imply (runs x |C| K) equals the
    unbatched steps once plus the batched ones per batch.  Ranking slicing
    sets with the trained model picks a set whose sliced amplitude is the
    state-vector amplitude."""
    from pqgb300 import costmodel as CM

    if not CM.WEIGHTS_FILE.exists():
        pytest.skip("no trained weights committed yet")
    r, c, d = 3, 4, 8
    bits = "100110101100"
    g = pq.random_grid_gates(r, c, d, seed=21)
    net = pq.build_network(r * c, g, backend=be, decompose=True)
    pq.add_input(net, "0" * (r * c))
    pq.add_output(net, bits)
    steps, cm, mx, _ = pq.planning.best_flop_plan(net, out_edges=[], candidates=("sweep",))
    p = pq.NetworkPlan(net, steps=steps, out_edges=[])
    f0, reps0 = p.sliced_features([], 4)
    np.testing.assert_allclose(f0[:, :4], p.features()[:, :4])
    assert np.all(reps0 == 1)
    sl = p.choose_slices(max_sliced=4, log2_target=0)
    f1, reps1 = p.sliced_features(sl, 4)
    sizes = p.sliced_sizes(sl)
    assert all((rp > 1) == b for rp, (_, b) in zip(reps1, sizes))
    np.testing.assert_allclose(f1[:, 2], [sz + (2.0 if b else 0.0) for sz, b in sizes])
    p.close()
    model = CM.CostModel.load(be)
    chosen, best_flop, cands = CM.learned_plan(net, model, out_edges=[], n_random=4, slice_targets=(6, 4))
    model.close()
    assert "sliced" in chosen and np.isfinite(chosen["pred_us"])
    pc = pq.NetworkPlan(net, steps=chosen["steps"], out_edges=[])
    if chosen["sliced"]:
        amp = pc.run_sliced(chosen["sliced"], batch=4)
    else:
        pc.execute()
        amp = complex(np.asarray(pc.result()).reshape(-1)[0])
    pc.close()
    ref = O.statevector(r * c, g)[O.amplitude_index(bits)]
    assert abs(amp - ref) / 2.0 ** -6 < 1e-6


def test_trained_weights_file_loads(pq, be):
    from pqgb300 import costmodel as CM

    if not CM.WEIGHTS_FILE.exists():
        pytest.skip("no trained weights committed yet")
    m = CM.CostModel.load(be)
    X = CM.model_inputs(np.array([[20, 16, 20, 8, 3, 4, 1, 1e7]], dtype=np.float64))
    assert np.isfinite(m.predict(X)).all()
    m.close()


def test_learned_plan_gains_over_flop_plan(pq, O):
    """What the trained network gains over the method without it: on the
    4x5 depth-12 open-output network the cost model ranks a Boltzmann-greedy
    draw first, while the flop-count planner (the judge and fallback) picks
    the reference's full-wavefunction order with fewer multiply-adds.  Both
    plans run as CUDA graphs, timed interleaved; the learned pick must not be
    slower (it ran 1.14x faster when the model was trained, 1.64x with the
    grouped small-step launches), and both give
    the oracle's state."""
    from pqgb300 import costmodel as CM
    from pqgb300.train_costmodel import time_plan

    be = pq.GB300Backend(pq.PREC_OZAKI)
    gates = pq.random_grid_gates(4, 5, 12, seed=2024)
    net = pq.build_network(20, gates, backend=be)
    pq.add_input(net, "0" * 20)
    model = CM.CostModel.load(be)
    chosen, best_flop, cands = CM.learned_plan(net, model, out_edges=None, n_random=16)
    model.close()
    assert chosen["name"] != best_flop["name"] and chosen["cmacs"] > best_flop["cmacs"]
    oe = pq.open_output_edges(net)
    tl, tf = [], []
    for _ in range(3):
        t, r_l = time_plan(pq, net, chosen["steps"], oe, reps=10)
        tl.append(t)
        t, r_f = time_plan(pq, net, best_flop["steps"], oe, reps=10)
        tf.append(t)
    assert min(tl) <= min(tf), (chosen["name"], tl, best_flop["name"], tf)
    sv = O.statevector(20, O.random_grid_gates(4, 5, 12, seed=2024))
    for r in (r_l, r_f):
        v = np.asarray(r).reshape(-1, order="F")
        assert np.max(np.abs(v - sv)) <= 1e-6 * np.max(np.abs(sv))
    be.close()
