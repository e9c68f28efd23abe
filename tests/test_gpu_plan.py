"""Compiled plans (NetworkPlan): wavefunction / greedy / sweep plans, CUDA
graph replay, many amplitudes, and sliced single amplitudes with the FP64
compensated slice sum, all against the FP64 oracle.

Tolerances: complex128 1e-12 relative, complex64 1e-6 relative (max-abs error
over the largest reference magnitude; for single amplitudes the error is
relative to the amplitude's magnitude scale 2^-n/2).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {0: 1e-12, 1: 1e-6}


def rel(a, b):
    a = np.asarray(a).reshape(-1)
    b = np.asarray(b).reshape(-1)
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.fixture(params=[0, 1], ids=["c128", "c64"])
def prec(request):
    return request.param


def open_net(pq, be, r, c, d, seed, decompose=False):
    n = r * c
    g = pq.random_grid_gates(r, c, d, seed=seed)
    net = pq.build_network(n, g, backend=be, decompose=decompose)
    pq.add_input(net, "0" * n)
    return net, g


@pytest.mark.parametrize("planner", ["wavefunction", "greedy"])
def test_plan_state_vector(pq, O, prec, planner):
    be = pq.GB300Backend(prec)
    net, g = open_net(pq, be, 3, 4, 8, seed=21)
    plan = pq.NetworkPlan(net, planner=planner, trials=4)
    info = plan.info()
    assert info["steps"] == len(net.nodes) - 1 and info["arena_bytes"] > 0
    plan.execute()
    got = plan.result().reshape(-1, order="F")
    ref = O.statevector(12, g)
    assert rel(got, ref) < TOL[prec]
    # graph capture, replayed twice, gives the same result
    plan.capture()
    plan.execute()
    got2 = plan.result().reshape(-1, order="F")
    assert rel(got2, ref) < TOL[prec]
    assert np.array_equal(got, got2)
    # the leaves were not consumed: the interactive path still works
    pq.full_wavefunction_contraction(net, "vector")
    assert rel(pq.load_tensor_data(net, "result"), ref) < TOL[prec]
    plan.close()
    be.close()


def test_plan_profile_and_features(pq, prec):
    be = pq.GB300Backend(prec)
    net, _ = open_net(pq, be, 2, 3, 4, seed=3)
    plan = pq.NetworkPlan(net, planner="greedy", trials=2)
    ms = plan.profile()
    f = plan.features()
    n = len(net.nodes) - 1
    assert ms.shape == (n,) and np.all(ms >= 0)
    assert f.shape == (n, 8) and np.all(np.isfinite(f))
    plan.close()
    be.close()


def test_many_amplitudes_small(pq, O, prec):
    be = pq.GB300Backend(prec)
    net, g = open_net(pq, be, 3, 4, 8, seed=5)
    bits = pq.random_bitstrings(12, 256, seed=1)
    plan = pq.NetworkPlan(net, planner="wavefunction")
    plan.capture()
    amps = plan.amplitudes(bits)
    sv = O.statevector(12, g)
    ref = sv[[O.amplitude_index(b) for b in bits]]
    assert np.max(np.abs(amps - ref)) / np.max(np.abs(sv)) < TOL[prec]
    plan.close()
    be.close()


def test_config2_grid_4x5_depth12_1024_amplitudes(pq, O, prec):
    """4x5 grid, depth 12, 1024 seeded bitstrings (config 2), c64 and c128."""
    be = pq.GB300Backend(prec)
    net, g = open_net(pq, be, 4, 5, 12, seed=2024)
    bits = pq.random_bitstrings(20, 1024, seed=7)
    steps, cm, mx, name = pq.planning.best_flop_plan(net, trials=4)
    plan = pq.NetworkPlan(net, steps=steps)
    plan.capture()
    amps = plan.amplitudes(bits)
    sv = O.statevector(20, g)
    ref = sv[[O.amplitude_index(b) for b in bits]]
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(amps - ref)) / scale < TOL[prec]
    plan.close()
    be.close()


def single_amp_net(pq, be, r, c, d, seed, bits):
    n = r * c
    g = pq.random_grid_gates(r, c, d, seed=seed)
    net = pq.build_network(n, g, backend=be, decompose=True)
    pq.add_input(net, "0" * n)
    pq.add_output(net, bits)
    return net, g


@pytest.mark.parametrize("batch", [1, 7, 64])
def test_sliced_single_amplitude(pq, O, prec, batch):
    r, c, d = 3, 4, 8
    bits = "011010011100"
    be = pq.GB300Backend(prec)
    net, g = single_amp_net(pq, be, r, c, d, 99, bits)
    steps, cm, mx, name = pq.planning.best_flop_plan(net, out_edges=[], candidates=("sweep",))
    plan = pq.NetworkPlan(net, steps=steps, out_edges=[])
    sliced = plan.choose_slices(max_sliced=5, log2_target=0)
    assert 1 <= len(sliced) <= 5
    amp = plan.run_sliced(sliced, batch=batch)
    plan.execute()
    unsliced = complex(np.asarray(plan.result()).reshape(-1)[0])
    ref = O.statevector(r * c, g)[O.amplitude_index(bits)]
    scale = 2.0 ** (-(r * c) / 2)
    assert abs(amp - ref) / scale < TOL[prec]
    assert abs(unsliced - ref) / scale < TOL[prec]
    # partial ranges accumulate to the same sum
    total = 2 ** len(sliced)
    half = total // 2
    plan.run_sliced(sliced, batch=batch, begin=0, end=half, reset=True)
    amp2 = plan.run_sliced(sliced, batch=batch, begin=half, end=total, reset=False)
    assert abs(amp2 - amp) / scale < 10 * TOL[prec]
    plan.close()
    be.close()


def test_sliced_run_graph_replay(pq, O, prec):
    """Repeated identical sliced runs: the second is captured as a CUDA graph
    and later ones replay it; results stay the same, the launch count per
    run stays the same, new leaf data in the same storage is picked up, and a
    changed range runs directly again."""
    r, c, d = 3, 4, 8
    bits = "110100101101"
    be = pq.GB300Backend(prec)
    net, g = single_amp_net(pq, be, r, c, d, 7, bits)
    steps, _, _, _ = pq.planning.best_flop_plan(net, out_edges=[], candidates=("sweep",))
    plan = pq.NetworkPlan(net, steps=steps, out_edges=[])
    sliced = plan.choose_slices(max_sliced=4, log2_target=0)
    amps, counts = [], []
    for _ in range(4):
        n0 = be.launch_count()
        amps.append(plan.run_sliced(sliced, batch=4))
        counts.append(be.launch_count() - n0)
    assert len(set(counts)) == 1
    assert max(abs(a - amps[0]) for a in amps) <= 1e-12 * abs(amps[0])
    ref = O.statevector(r * c, g)[O.amplitude_index(bits)]
    assert abs(amps[0] - ref) / 2.0 ** (-(r * c) / 2) < TOL[prec]
    # scale one leaf in place (same extents: batched upload keeps its storage)
    lab = net.nodes[plan.leaves[0]].data_label
    data = be.load_tensor_data(lab)
    be.save_tensors([(lab, 2 * data)])
    assert abs(plan.run_sliced(sliced, batch=4) - 2 * amps[0]) <= 1e-9 * abs(amps[0])
    # another range
    total = 2 ** len(sliced)
    part = plan.run_sliced(sliced, batch=4, begin=0, end=total // 2)
    assert np.isfinite(part)
    plan.close()
    be.close()


def test_config3_scaled_sliced(pq, O, prec):
    """Config 3 in miniature: 4x4 grid, depth 10, CZ split into bond-2
    virtual edges, 6 sliced bonds (64 identical-shape slices) summed in FP64."""
    bits = "0110100111001010"
    be = pq.GB300Backend(prec)
    net, g = single_amp_net(pq, be, 4, 4, 10, 3, bits)
    steps, cm, mx, name = pq.planning.best_flop_plan(net, out_edges=[], candidates=("sweep", "greedy"))
    plan = pq.NetworkPlan(net, steps=steps, out_edges=[])
    sliced = plan.choose_slices(max_sliced=6, log2_target=0)
    amp = plan.run_sliced(sliced, batch=16)
    ref = O.statevector(16, g)[O.amplitude_index(bits)]
    assert abs(amp - ref) / 2.0 ** -8 < TOL[prec]
    plan.close()
    be.close()


def test_plan_rejects_bad_input(pq):
    from pqgb300 import _lib as L

    be = pq.GB300Backend(pq.PREC_C64)
    net, _ = open_net(pq, be, 2, 2, 2, seed=1)
    plan = pq.NetworkPlan(net, planner="greedy")
    bad = list(plan.steps)
    bad[0] = bad[1]
    with pytest.raises(L.PQError):
        pq.NetworkPlan(net, steps=bad)
    # a leaf replaced by a tensor of the wrong size
    first = net.nodes[plan.leaves[0]].data_label
    be.save_tensor_data(first, np.ones((3,)))
    with pytest.raises(L.PQError) as e:
        plan.execute()
    assert e.value.code == L.PQ_ERR_INVALID
    plan.close()
    be.close()


@pytest.mark.parametrize("prec", [0, 5], ids=["c128", "ozaki"])
def test_small_steps_launch_in_groups(pq, O, prec):
    """The qubit-sweep plan of a 4x4 depth-10 single amplitude: its per-qubit
    chains are runs of small complex128 steps, launched level by level in
    groups (fewer launches than steps, counted both at compile time and by
    the context); the amplitude matches the state vector, directly, replayed
    from a CUDA graph, and through the sliced path."""
    be = pq.GB300Backend(prec)
    n, bits = 16, "0110100111001010"
    g = pq.random_grid_gates(4, 4, 10, seed=31)
    net = pq.build_network(n, g, backend=be, decompose=True)
    pq.add_input(net, "0" * n)
    pq.add_output(net, bits)
    steps, _, _, _ = pq.planning.best_flop_plan(net, out_edges=[], candidates=("sweep",))
    plan = pq.NetworkPlan(net, steps=steps, out_edges=[])
    info = plan.info()
    assert info["launches"] < info["steps"] // 2
    n0 = be.launch_count()
    plan.execute()
    assert be.launch_count() - n0 == info["launches"]
    ref = O.statevector(n, g)[O.amplitude_index(bits)]
    tol = 1e-12 if prec == 0 else 1e-6
    amp = complex(np.asarray(plan.result()).reshape(-1)[0])
    assert abs(amp - ref) / 2.0 ** (-n / 2) < tol
    plan.capture()
    plan.execute()
    assert complex(np.asarray(plan.result()).reshape(-1)[0]) == amp
    sliced = plan.choose_slices(max_sliced=3, log2_target=8)
    for batch in (1, 8):
        a2 = plan.run_sliced(sliced, batch=batch)
        assert abs(a2 - ref) / 2.0 ** (-n / 2) < tol
    plan.close()
    be.close()


@pytest.mark.parametrize("prec", [0, 1], ids=["c128", "c64"])
def test_small_step_groups_chunked(pq, prec):
    """65 independent 4 x 4 matrix products on the first level (one group of
    64 and a single step), then a chain of 64 dependent products: the plan
    result is the product of all 130 matrices."""
    import ctypes as C

    from pqgb300 import _lib as L

    rng = np.random.default_rng(41)
    npairs = 65
    be = pq.GB300Backend(prec)
    # labels: x_i = i (0..65), k_i = 66 + i
    ranks, flat, ids, mats = [], [], [], []
    for i in range(npairs):
        A = rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))
        B = rng.standard_normal((4, 4)) + 1j * rng.standard_normal((4, 4))
        for nm, M, lab in ((f"a{i}", A, [i, 66 + i]), (f"b{i}", B, [66 + i, i + 1])):
            be.save_tensor_data(nm, M)
            ranks.append(2)
            flat += lab
            ids.append(be.id_of(nm))
        mats.append(A @ B)
    dims = [4] * (66 + npairs)
    steps = []
    for i in range(npairs):
        steps += [2 * i, 2 * i + 1]  # value 2*npairs + i = A_i B_i
    v = 2 * npairs
    nxt = 3 * npairs
    for i in range(1, npairs):
        steps += [v, 2 * npairs + i]
        v = nxt
        nxt += 1
    h = C.c_void_p()
    L.check(be.lib.pq_plan_create(be.ctx, len(ranks), L.arr(C.c_int32, ranks), L.arr(C.c_int32, flat), len(dims),
                                  L.arr(C.c_int64, dims), len(steps) // 2, L.arr(C.c_int32, steps), 2,
                                  L.arr(C.c_int32, [0, npairs]), C.byref(h)), be.ctx, "plan_create")
    cm, mx, ar, la = C.c_double(), C.c_int64(), C.c_int64(), C.c_int64()
    L.check(be.lib.pq_plan_info(h, C.byref(cm), C.byref(mx), C.byref(ar), C.byref(la)), be.ctx, "info")
    assert la.value == 2 + (npairs - 1)  # the first level in two launches, then the chain
    L.check(be.lib.pq_plan_execute(h, L.arr(C.c_int64, ids), be.id_of("r")), be.ctx, "execute")
    got = be.load_tensor_data("r")
    be.lib.pq_plan_destroy(h)
    be.close()
    ref = mats[0]
    for M in mats[1:]:
        ref = ref @ M
    assert rel(got, ref) < TOL[prec]


@pytest.mark.parametrize("prec", [0, 1], ids=["c128", "c64"])
def test_small_step_groups_mixed_extents(pq, O, prec):
    """Independent small steps with extents 3, 5, 6 and 7 (the grouped
    kernel's division decode), three chains advancing together, then joined:
    the plan result is the oracle's contraction."""
    import ctypes as C

    from pqgb300 import _lib as L

    rng = np.random.default_rng(43)
    ext = [3, 5, 6, 7, 2, 3, 5, 7, 6]
    # chains c = 0, 1, 2: T_c0 [a_c, k_c] x T_c1 [k_c, m_c] x T_c2 [m_c, b_c]; then joined over b_c -> a_c's open
    labels = {}
    def lab(name, d):
        if name not in labels:
            labels[name] = (len(labels), d)
        return labels[name][0]
    leaves, ranks, flat, ids = [], [], [], []
    be = pq.GB300Backend(prec)
    for c in range(3):
        a, k, m, b = ext[3 * c], ext[3 * c + 1], ext[3 * c + 2], 4
        shapes = [((a, k), [f"a{c}", f"k{c}"]), ((k, m), [f"k{c}", f"m{c}"]), ((m, b), [f"m{c}", "b"])]
        for t, (shp, names) in enumerate(shapes):
            T = rng.standard_normal(shp) + 1j * rng.standard_normal(shp)
            nm = f"t{c}{t}"
            be.save_tensor_data(nm, T)
            leaves.append((T, names))
            ranks.append(2)
            flat += [lab(x, d) for x, d in zip(names, shp)]
            ids.append(be.id_of(nm))
    dims = [d for _, d in sorted(labels.values())]
    # chain steps first (level 0: t_c0 t_c1 for each c; level 1: with t_c2), then the joins over "b"
    steps = []
    for c in range(3):
        steps += [3 * c, 3 * c + 1]          # value 9 + c
    for c in range(3):
        steps += [9 + c, 3 * c + 2]          # value 12 + c: [a_c, b]
    steps += [12, 13, 15, 14]                # value 15: [a0, b, a1] (b still open for chain 2), value 16
    out = [labels["a0"][0], labels["a1"][0], labels["a2"][0]]
    h = C.c_void_p()
    L.check(be.lib.pq_plan_create(be.ctx, len(ranks), L.arr(C.c_int32, ranks), L.arr(C.c_int32, flat), len(dims),
                                  L.arr(C.c_int64, dims), len(steps) // 2, L.arr(C.c_int32, steps), len(out),
                                  L.arr(C.c_int32, out), C.byref(h)), be.ctx, "plan_create")
    L.check(be.lib.pq_plan_execute(h, L.arr(C.c_int64, ids), be.id_of("r")), be.ctx, "execute")
    got = be.load_tensor_data("r")
    be.lib.pq_plan_destroy(h)
    be.close()
    T = [x[0] for x in leaves]
    ref = np.einsum("ak,km,mb,cl,ln,nb,dp,pq,qb->acd", *T)
    assert rel(got, ref) < TOL[prec]


def test_grid7x7_d14_amplitude_vs_oracle(pq, O):
    """A single amplitude of the 7x7 depth-14 random circuit (49 qubits, the
    learned-planning workload's size) on the exact-accumulation path, along
    the flop-count planner's sweep plan (2^36.5 complex multiply-adds,
    intermediates up to 2^26 elements), unsliced and with the heavy subtree
    sliced (ten bonds chosen for a 2^22-element target: per-slice
    intermediates of at most 2^24 elements, part of the work repeated per
    slice), against the FP64 oracle's contraction of the same network
    along the same plan: relative error <= 1e-6 both ways."""
    import bench

    rows, cols, depth = 7, 7, 14
    n = rows * cols
    gates = pq.random_grid_gates(rows, cols, depth, seed=2026)
    bits = pq.random_bitstrings(n, 1, seed=2027)[0]
    be = pq.GB300Backend(pq.PREC_OZAKI)
    net = pq.build_network(n, gates, decompose=True, backend=be)
    pq.add_input(net, "0" * n)
    pq.add_output(net, bits)
    steps, cm, mx, _ = pq.planning.best_flop_plan(net, out_edges=[], candidates=("sweep",))
    nodes = list(net.nodes)
    rec = {"rows": rows, "cols": cols, "depth": depth, "circuit_seed": 2026, "bitstring": bits, "leaves": nodes,
           "leaf_indices": [list(net.nodes[x].indices) for x in nodes], "steps": steps}
    ref, _ = bench.oracle_amplitude(O, rec)
    plan = pq.NetworkPlan(net, steps=steps, out_edges=[])
    plan.execute()
    amp = complex(np.asarray(plan.result()).reshape(-1)[0])
    assert abs(amp - ref) <= 1e-6 * abs(ref), (amp, ref)
    sl = plan.choose_slices(max_sliced=10, log2_target=22.0)
    assert len(sl) >= 4
    sizes = plan.sliced_sizes(sl)
    assert max(x for x, _ in sizes) <= np.log2(mx) - 2
    amp_s = plan.run_sliced(sl, batch=plan.auto_batch(sl))
    assert abs(amp_s - ref) <= 1e-6 * abs(ref), (amp_s, ref, sizes)
    plan.close()
    be.close()


@pytest.mark.parametrize("rows,cols,depth", [(5, 5, 12), (7, 7, 14)])
def test_plan_cost_batch_matches_host(pq, rows, cols, depth):
    """Candidate scoring on the device (one warp per plan) gives the host
    pass's complex multiply-adds and largest intermediate for seeded greedy
    draws and qubit-sweep orders of a decomposed random circuit, and the
    sweep planner picks the same plan with device scoring; a plan that is not
    SSA over the leaves is refused."""
    from pqgb300 import _lib as L
    from pqgb300 import planning as PL

    n = rows * cols
    be = pq.GB300Backend(pq.PREC_C64)
    net = pq.build_network(n, pq.random_grid_gates(rows, cols, depth, seed=8), decompose=True, backend=be)
    pq.add_input(net, "0" * n)
    pq.add_output(net, pq.random_bitstrings(n, 1, seed=9)[0])
    nodes, ranks, flat, dims, label_of = PL._leaf_arrays(net, [])
    cands = [s for s, _, _ in PL.greedy_draws(ranks, flat, dims, [], 24, seed=3)]
    cands += [s for s, _, _ in PL.sweep_steps(net, nodes, [], label_of, ranks, flat, dims, all_orders=True,
                                              random_orders=16, seed=1)]
    got = PL.plan_cost_batch(be, ranks, flat, dims, cands, [])
    for st, (cm, mx) in zip(cands, got):
        hc, hm = PL.plan_cost(ranks, flat, dims, st, [])
        assert abs(cm - hc) <= 1e-9 * hc and abs(mx - hm) <= 1e-9 * hm
    host = PL.sweep_steps(net, nodes, [], label_of, ranks, flat, dims, random_orders=16, seed=1)
    dev = PL.sweep_steps(net, nodes, [], label_of, ranks, flat, dims, random_orders=16, seed=1, cost_backend=be)
    assert dev[0] == host[0] and abs(dev[1] - host[1]) <= 1e-9 * host[1]
    bad = list(cands[0])
    bad[0] = len(nodes) + 5  # an operand that does not exist yet
    with pytest.raises(L.PQError):
        PL.plan_cost_batch(be, ranks, flat, dims, [cands[1], bad], [])
    be.close()
