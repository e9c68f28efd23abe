"""Host-side logic on CPU: the C ABI loads and exports every declared symbol,
the native planners produce valid plans, and the product's graph layer (run
over a numpy test backend) reproduces the oracle's bookkeeping."""
import re
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "pqgb300.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*|void)\s+(pq_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(pq):
    from pqgb300 import _lib as L

    lib = L.lib()
    syms = declared_symbols()
    assert len(syms) >= 30
    for s in syms:
        assert hasattr(lib, s), f"libpqgb300.so does not export {s}"
    bound = {name for name, _, _ in L.SIGNATURES}
    assert set(syms) <= bound | L.OPTIONAL, set(syms) - bound


def test_null_handles_are_rejected(pq):
    from pqgb300 import _lib as L

    lib = L.lib()
    assert lib.pq_ctx_destroy(None) == L.PQ_ERR_INVALID
    assert lib.pq_plan_destroy(None) == L.PQ_ERR_INVALID
    assert lib.pq_ctx_sync(None) == L.PQ_ERR_INVALID
    assert lib.pq_last_error(None) == b"null context"


def _ssa_valid(steps, n):
    live = set(range(n))
    for i in range(len(steps) // 2):
        a, b = steps[2 * i], steps[2 * i + 1]
        assert a in live and b in live and a != b
        live -= {a, b}
        live.add(n + i)
    assert live == {2 * n - 2}


def _leaves(pq, net):
    return pq.planning._leaf_arrays(net, pq.open_output_edges(net))


@pytest.mark.parametrize("rows,cols,depth", [(2, 2, 3), (2, 3, 5), (3, 3, 6)])
def test_greedy_plan_valid_and_cost_consistent(pq, O, host_backend, rows, cols, depth):
    n = rows * cols
    gates = pq.random_grid_gates(rows, cols, depth, seed=3)
    net = pq.build_network(n, gates, backend=host_backend)
    pq.add_input(net, "0" * n)
    nodes, ranks, flat, dims, label_of = _leaves(pq, net)
    outl = [label_of[e] for e in pq.open_output_edges(net)]
    steps, cm, mx = pq.greedy_steps(ranks, flat, dims, outl, 1.0, 1.0, 6, 1)
    _ssa_valid(steps, len(ranks))
    c2, m2 = pq.planning.plan_cost(ranks, flat, dims, steps, outl)
    assert abs(cm - c2) <= 1e-9 * c2 and m2 == mx
    # executing the plan with the oracle backend gives the state vector
    plan = pq.steps_to_pairs(net, steps, nodes)
    pq.contract_network(net, plan)
    out = pq.load_tensor_data(net, "result").reshape(-1, order="F")
    assert np.max(np.abs(out - O.statevector(n, gates))) < 1e-12


def test_sweep_plan_single_amplitude(pq, O, host_backend):
    gates = pq.random_grid_gates(3, 3, 6, seed=5)
    bits = "101100110"
    net = pq.build_network(9, gates, backend=host_backend, decompose=True)
    pq.add_input(net, "0" * 9)
    pq.add_output(net, bits)
    steps, cm, mx, name = pq.planning.best_flop_plan(net, out_edges=[], candidates=("sweep",))
    _ssa_valid(steps, len(net.nodes))
    pq.contract_network(net, pq.steps_to_pairs(net, steps))
    amp = pq.load_tensor_data(net, "result")
    ref = O.statevector(9, gates)[O.amplitude_index(bits)]
    assert abs(complex(np.asarray(amp).reshape(-1)[0]) - ref) < 1e-13


def test_slice_chooser_reduces_size(pq, host_backend):
    gates = pq.random_grid_gates(4, 4, 8, seed=9)
    net = pq.build_network(16, gates, backend=host_backend, decompose=True)
    pq.add_input(net, "0" * 16)
    pq.add_output(net, "0" * 16)
    nodes, ranks, flat, dims, label_of = pq.planning._leaf_arrays(net, [])
    steps, cm, mx, _ = pq.planning.best_flop_plan(net, out_edges=[], candidates=("sweep",))
    lib_steps = pq.planning
    from pqgb300 import _lib as L
    import ctypes as C

    out = (C.c_int32 * 8)()
    ns = C.c_int()
    rc = L.lib().pq_plan_choose_slices(len(ranks), L.arr(C.c_int32, ranks), L.arr(C.c_int32, flat), len(dims),
                                       L.arr(C.c_int64, dims), len(steps) // 2, L.arr(C.c_int32, steps), 0,
                                       L.arr(C.c_int32, []), 4, 0.0, out, C.byref(ns))
    assert rc == 0 and ns.value >= 1
    chosen = set(out[: ns.value])
    # recompute the largest intermediate with those labels fixed
    sliced_dims = [1 if i in chosen else d for i, d in enumerate(dims)]
    _, mx2 = lib_steps.plan_cost(ranks, flat, sliced_dims, steps, [])
    assert mx2 < mx


def test_product_graph_matches_oracle_metrics(pq, host_backend):
    # the reference's 8/44/124 golden through the product's L2 code
    net = pq.build_network(3, [(pq.H, [1]), (pq.CX, [1, 2]), (pq.CX, [1, 2]), (pq.CX, [1, 3])],
                           backend=host_backend)
    pq.add_input(net, "000")
    pq.full_wavefunction_contraction(net, "vector")
    m = host_backend.metrics
    assert (m.max_tensor_size, m.total_space_allocated, m.flops) == (8, 44, 124)


def test_product_generators_match_oracle(pq, O):
    a = pq.random_grid_gates(3, 4, 5, seed=17)
    b = O.random_grid_gates(3, 4, 5, 17)
    assert len(a) == len(b)
    for (ua, qa), (ub, qb) in zip(a, b):
        assert qa == qb and np.array_equal(ua, ub)
    for (ua, qa), (ub, qb) in zip(pq.qft_gates(6), O.qft_gates(6)):
        assert qa == qb and np.allclose(ua, ub, atol=0, rtol=0)
    for U, _ in pq.random_grid_gates(2, 2, 3, seed=1):
        if U.shape == (2, 2):
            assert np.allclose(U @ U.conj().T, np.eye(2), atol=1e-14)
            assert abs(np.linalg.det(U) - 1) < 1e-14


def test_product_slicing_host_logic(pq, O, host_backend):
    n = 4
    circ = O.simple_preparation_gates(n, 2, np.random.default_rng(2)) + O.qft_gates(n)
    full = O.statevector(n, circ)
    tot = 0
    for p in range(1, 5):
        be = type(host_backend)()
        net = pq.build_network(n, circ, decompose=True, backend=be)
        pq.add_input(net, "0" * n)
        bl, bv = pq.partition_network_on_virtual_bonds(net, 4, p)
        pq.slice_tensor_network(net, bl, bv)
        pq.full_wavefunction_contraction(net, "vector")
        tot = tot + pq.load_tensor_data(net, "result")
    assert np.max(np.abs(tot - full)) < 1e-13


def test_wavefunction_steps_match_reference_order(pq, O, host_backend):
    gates = pq.random_grid_gates(2, 3, 4, seed=2)
    net = pq.build_network(6, gates, backend=host_backend)
    pq.add_input(net, "0" * 6)
    steps = pq.wavefunction_steps(net)
    _ssa_valid(steps, len(net.nodes))
    pq.contract_network(net, pq.steps_to_pairs(net, steps))
    out = pq.load_tensor_data(net, "result").reshape(-1, order="F")
    assert np.max(np.abs(out - O.statevector(6, gates))) < 1e-13


def test_fused_gates_statevector_order(pq, O, host_backend):
    """Single-qubit gates folded into two-qubit gates, applied gate by gate
    to the state: the state vector of the original circuit."""
    from pqgb300 import circuits as CI

    gates = pq.random_grid_gates(2, 3, 5, seed=4)
    fused = CI.fuse_single_qubit_gates(gates)
    assert len(fused) < len(gates) // 2
    net = pq.build_network(6, fused, backend=host_backend)
    pq.add_input(net, "0" * 6)
    steps = pq.planning.statevector_steps(net)
    _ssa_valid(steps, len(net.nodes))
    pq.contract_network(net, pq.steps_to_pairs(net, steps))
    out = pq.load_tensor_data(net, "result").reshape(-1, order="F")
    assert np.max(np.abs(out - O.statevector(6, gates))) < 1e-13


@pytest.mark.parametrize("max_qubits", [2, 3, 4])
def test_block_fused_gates(pq, O, host_backend, max_qubits):
    """Gates fused into blocks of at most 2, 3 or 4 qubits (open blocks merged
    when a gate joins them): exact, fewer blocks than gates, and the block
    circuit contracted gate by gate on the host backend gives the original
    circuit's state vector."""
    from pqgb300 import circuits as CI

    gates = pq.random_grid_gates(3, 3, 8, seed=11)
    blocks = CI.fuse_gates(gates, max_qubits)
    assert max(len(q) for _, q in blocks) <= max_qubits
    assert len(blocks) < len(CI.fuse_single_qubit_gates(gates)) or max_qubits == 2
    ref = O.statevector(9, gates)
    assert np.max(np.abs(O.statevector(9, blocks) - ref)) < 1e-12
    net = pq.build_network(9, blocks, backend=host_backend)
    pq.add_input(net, "0" * 9)
    pq.contract_network(net, pq.steps_to_pairs(net, pq.planning.statevector_steps(net)))
    out = pq.load_tensor_data(net, "result").reshape(-1, order="F")
    assert np.max(np.abs(out - ref)) < 1e-12


def test_block_fusion_keeps_order_of_random_gates(pq, O):
    """Random gates of one to three qubits on arbitrary qubits: blocks of up
    to four qubits reproduce the state vector (only commuting blocks move)."""
    from pqgb300 import circuits as CI

    rng = np.random.default_rng(3)
    for _ in range(10):
        gates = []
        for _ in range(40):
            k = int(rng.integers(1, 4))
            qs = [int(q) for q in rng.choice(np.arange(1, 8), k, replace=False)]
            z = rng.standard_normal((2 ** k, 2 ** k)) + 1j * rng.standard_normal((2 ** k, 2 ** k))
            gates.append((np.linalg.qr(z)[0], qs))
        ref = O.statevector(7, gates)
        for m in (3, 4):
            assert np.max(np.abs(O.statevector(7, CI.fuse_gates(gates, m)) - ref)) < 1e-12


def test_batched_output_amplitudes(pq, O, host_backend):
    """Output tensors sharing one bitstring-batch index: one contraction of
    the sweep order gives the amplitudes of all bitstrings."""
    import bench

    gates = pq.random_grid_gates(2, 3, 4, seed=6)
    bits = pq.random_bitstrings(6, 5, seed=7)
    net = pq.build_network(6, gates, backend=host_backend, decompose=True)
    pq.add_input(net, "0" * 6)
    bench.batched_outputs(pq, net, bits)
    nodes, ranks, flat, dims, label_of = pq.planning._leaf_arrays(net, [bench.AMP_INDEX])
    out = [label_of[bench.AMP_INDEX]]
    steps, cm, mx = pq.planning.sweep_steps(net, nodes, out, label_of, ranks, flat, dims)
    _ssa_valid(steps, len(nodes))
    leaves = [host_backend.tensors[net.nodes[nl].data_label] for nl in nodes]
    labs, pos = [], 0
    for r in ranks:
        labs.append(flat[pos:pos + r])
        pos += r
    amps = O.execute_ssa_plan(leaves, labs, steps, out)
    sv = O.statevector(6, gates)
    ref = np.array([sv[O.amplitude_index(b)] for b in bits])
    assert np.max(np.abs(np.asarray(amps).reshape(-1) - ref)) < 1e-13


def test_greedy_draws_parallel_deterministic(pq, host_backend):
    """Parallel planner draws: valid SSA plans whose costs match the host
    cost function; draw 0 is the plain greedy order; results do not depend
    on the thread count; the Boltzmann draws vary."""
    gates = pq.random_grid_gates(3, 3, 6, seed=3)
    net = pq.build_network(9, gates, backend=host_backend, decompose=True)
    pq.add_input(net, "0" * 9)
    pq.add_output(net, "010011010")
    nodes, ranks, flat, dims, label_of = pq.planning._leaf_arrays(net, [])
    d1 = pq.planning.greedy_draws(ranks, flat, dims, [], 12, seed=5, threads=1)
    d4 = pq.planning.greedy_draws(ranks, flat, dims, [], 12, seed=5, threads=4)
    assert [x[0] for x in d1] == [x[0] for x in d4]
    for s, cm, mx in d1:
        _ssa_valid(s, len(ranks))
        c2, m2 = pq.planning.plan_cost(ranks, flat, dims, s, [])
        assert abs(cm - c2) <= 1e-9 * c2 and m2 == mx
    s0, _, _ = pq.greedy_steps(ranks, flat, dims, [], 1.0, 1.0, 1, 5)
    assert d1[0][0] == s0
    assert len({tuple(x[0]) for x in d1}) > 1


def test_network_json_round_trip(pq, O, host_backend):
    """src/layer3.jl:579-707: to_json / network_from_json keep the graph (and
    the reference's value formats); the round-tripped network contracts to
    the same GHZ-3 amplitude (test/layer1_tests.jl:34-39)."""
    import json

    net = pq.build_network(3, pq.ghz_gates(3), backend=host_backend, decompose=True)
    pq.add_input(net, "000")
    pq.add_output(net, "000")
    s = pq.to_json(net, 2)
    d = json.loads(s)
    assert list(d) == ["number_qubits", "edges", "nodes", "input_qubits", "output_qubits", "qubit_ordering",
                       "node_layers"]
    assert all(isinstance(x, str) for v in d["nodes"].values() for x in v["dims"])
    net2 = pq.network_from_json(s, host_backend)
    assert pq.to_dict(net2) == pq.to_dict(net)
    assert net2.counters["node"] == max(int(k.split("_")[-1]) for k in net.nodes)
    # a new node continues the numbering
    assert pq.network.new_label(net2, "node") not in net.nodes
    pq.contract_network(net2, pq.random_contraction_plan(net2, np.random.default_rng(0)))
    amp = complex(np.asarray(pq.load_tensor_data(net2, "result")).reshape(-1)[0])
    assert abs(amp - 1 / np.sqrt(2)) < 1e-12


def _cost_restated(ranks, flat, dims, steps, out_labels):
    """The executor's label rule restated in Python: a label is summed once
    no other live tensor and no output carries it."""
    labs, pos, cnt = [], 0, {}
    for r in ranks:
        lab = list(flat[pos:pos + r])
        pos += r
        labs.append(lab)
        for x in lab:
            cnt[x] = cnt.get(x, 0) + 1
    for x in out_labels:
        cnt[x] = cnt.get(x, 0) + 1
    l2 = [float(np.log2(d)) for d in dims]
    cost, mx = 0.0, 0.0
    for i in range(len(steps) // 2):
        a, b = labs[steps[2 * i]], labs[steps[2 * i + 1]]
        for x in a + b:
            cnt[x] -= 1
        union = list(dict.fromkeys(a + b))
        keep = [x for x in union if cnt[x] > 0]
        for x in keep:
            cnt[x] += 1
        labs.append(keep)
        cost += 2.0 ** sum(l2[x] for x in union)
        mx = max(mx, sum(l2[x] for x in keep))
    return cost, 2.0 ** mx


def test_native_plan_cost_matches_label_rule(pq, host_backend):
    """pq_plan_cost against the restated rule: every candidate plan of a 3x4
    depth-8 single amplitude (exact), and random networks with extents 1..6,
    repeated and open labels (to 1e-12)."""
    from pqgb300 import costmodel as CM
    from pqgb300 import planning as PL

    gates = pq.random_grid_gates(3, 4, 8, seed=2)
    net = pq.build_network(12, gates, decompose=True, backend=host_backend)
    pq.add_input(net, "0" * 12)
    pq.add_output(net, "010011010110")
    nodes, ranks, flat, dims, _ = CM._leaf_arrays(net, [])
    cands, _ = CM.candidate_plans(net, [], 8, 0)
    for c in cands:
        assert PL.plan_cost(ranks, flat, dims, c["steps"], []) == _cost_restated(ranks, flat, dims, c["steps"], [])
    rng = np.random.default_rng(0)
    for _ in range(40):
        nl, nlab = int(rng.integers(2, 12)), int(rng.integers(3, 14))
        dims = [int(x) for x in rng.integers(1, 7, nlab)]
        ranks = [int(x) for x in rng.integers(1, 4, nl)]
        flat = [int(x) for x in rng.integers(0, nlab, sum(ranks))]
        out = [int(x) for x in rng.choice(nlab, int(rng.integers(0, 3)), replace=False)]
        live, steps, nxt = list(range(nl)), [], nl
        while len(live) > 1:
            i, j = rng.choice(len(live), 2, replace=False)
            x, y = live[i], live[j]
            steps += [x, y]
            live = [v for v in live if v not in (x, y)] + [nxt]
            nxt += 1
        got, ref = PL.plan_cost(ranks, flat, dims, steps, out), _cost_restated(ranks, flat, dims, steps, out)
        assert np.allclose(got, ref, rtol=1e-12, atol=0)


def test_flop_planner_statevector_candidate_on_fused_circuit(pq, O, host_backend):
    """The flop-count planner with the gate-by-gate state-vector order among
    its candidates, on a circuit fused into blocks of up to four qubits: the
    chosen plan, contracted on the host backend, gives the state vector of the
    unfused circuit; the state-vector order itself is valid and exact too."""
    from pqgb300 import circuits as CI

    gates = pq.random_grid_gates(3, 4, 10, seed=5)
    for cands in (("sweep", "greedy", "wavefunction", "statevector"), ("statevector",)):
        be = type(host_backend)()
        net = pq.build_network(12, CI.fuse_gates(gates, 4), backend=be)
        pq.add_input(net, "0" * 12)
        steps, cm, mx, name = pq.planning.best_flop_plan(net, trials=2, candidates=cands)
        assert name in cands and cm > 0 and mx >= 2 ** 12
        _ssa_valid(steps, len(net.nodes))
        pq.contract_network(net, pq.steps_to_pairs(net, steps))
        out = pq.load_tensor_data(net, "result").reshape(-1, order="F")
        assert np.max(np.abs(out - O.statevector(12, gates))) < 1e-12


def test_randomized_sweep_orders(pq, O, host_backend):
    """Seeded randomized qubit-sweep orders: valid SSA plans, reproducible for
    a seed, never costlier than the deterministic sweeps (the cheapest is
    kept), and the chosen plan contracted on the host backend gives the
    state vector's amplitude."""
    from pqgb300 import costmodel as CM
    from pqgb300 import planning as PL

    n, bits = 12, "011010011100"
    gates = pq.random_grid_gates(3, 4, 10, seed=7)
    net = pq.build_network(n, gates, decompose=True, backend=host_backend)
    pq.add_input(net, "0" * n)
    pq.add_output(net, bits)
    nodes, ranks, flat, dims, label_of = CM._leaf_arrays(net, [])
    det = PL.sweep_steps(net, nodes, [], label_of, ranks, flat, dims)
    rnd = PL.sweep_steps(net, nodes, [], label_of, ranks, flat, dims, random_orders=32, seed=3)
    again = PL.sweep_steps(net, nodes, [], label_of, ranks, flat, dims, random_orders=32, seed=3)
    assert rnd[0] == again[0] and rnd[1] <= det[1]
    allo = PL.sweep_steps(net, nodes, [], label_of, ranks, flat, dims, all_orders=True, random_orders=32, seed=3,
                          keep_random=4)
    assert 7 <= len(allo) <= 7 + 4 and min(c for _, c, _ in allo) == rnd[1]
    for steps, cm, mx in allo:
        _ssa_valid(steps, len(nodes))
        assert PL.plan_cost(ranks, flat, dims, steps, []) == (cm, mx)
    pq.contract_network(net, pq.steps_to_pairs(net, rnd[0]))
    amp = complex(np.asarray(pq.load_tensor_data(net, "result")).reshape(-1)[0])
    assert abs(amp - O.statevector(n, gates)[O.amplitude_index(bits)]) < 1e-12


def test_bench_roofline_classes():
    """The bench's roofline assembly over per-step timings: every kernel class
    (generic, SIMT GEMM, tcgen05, copy, skinny) is named, shares add up, each
    step's lower bound is max(bytes / HBM, flops / peak), and the dominant
    class's bound is the side with the larger summed lower bound (HBM for a
    skinny class and for a shallow tensor-core pair, tensor for a deep one)."""
    import bench

    peaks = {"hbm_gbs": 6757.5, "bf16_tflops": 1871.0, "bf16_tflops_sustained": 1683.9}

    def feats(kc, lc, lk, nbytes):
        return [10.0, 10.0, lc, lk, 1.0, 1.0, float(kc), nbytes]

    steps = [(0.2, False, feats(0, 10, 2, 1e6)), (3.0, False, feats(4, 28, 4, 4e9)),
             (0.1, True, feats(3, 12, 0, 1e5)), (0.5, False, feats(1, 20, 8, 1e8))]
    ms, batched, fs = zip(*steps)
    roof, info, overall = bench.roofline_from_profile(ms, batched, fs, peaks, "measured", 4, "ozaki", 5.0)
    assert set(info) == {"generic", "skinny", "copy", "gemm_simt"}
    assert abs(sum(d["share"] for d in info.values()) - 1.0) < 1e-12
    assert roof["bound"] == "hbm" and roof["kernel"] == "skinny" and roof["unit"] == "GB/s"
    assert abs(roof["achieved"] - 4e9 / 3e-3 / 1e9) < 1e-6 and roof["frac"] == roof["achieved"] / 6757.5
    assert abs(info["skinny"]["lower_bound_ms"] - 1e3 * 4e9 / 6757.5e9) < 1e-9
    assert overall["wall_ms"] == 5.0 and 0 < overall["frac_of_wall"] < 1
    # a shallow tensor-core pair (K = 2^8): its bytes bound it
    steps.append((9.0, False, feats(2, 28, 8, 5e9)))
    ms, batched, fs = zip(*steps)
    roof, info, _ = bench.roofline_from_profile(ms, batched, fs, peaks, "measured", 4, "ozaki", 13.0)
    assert roof["bound"] == "hbm" and roof["tensor_ops_per_algorithmic_flop"] == 15.0
    assert abs(roof["achieved"] - 5e9 / 9e-3 / 1e9) < 1e-6
    assert abs(roof["algorithmic_tflops"] - 8.0 * 2 ** 28 * 2 ** 8 / 9e-3 / 1e12) < 1e-9
    # a deep one (K = 2^12): its flops bound it
    steps[-1] = (9.0, False, feats(2, 28, 12, 5e9))
    ms, batched, fs = zip(*steps)
    roof, info, _ = bench.roofline_from_profile(ms, batched, fs, peaks, "measured", 4, "ozaki", 13.0)
    assert roof["bound"] == "tensor" and roof["unit"] == "TFLOP/s"
    assert abs(roof["achieved"] - 8.0 * 2 ** 28 * 2 ** 12 / 9e-3 / 1e12) < 1e-9
    lb = 1e3 * 8.0 * 2 ** 40 / 1683.9e12
    assert abs(info["tcgen05"]["lower_bound_ms"] - lb) < 1e-9


def test_reference_arm_loads_no_product_library():
    """bench.py's CPU reference arm runs the FP64 oracle only: in a fresh
    process it neither imports the product package nor maps its library."""
    import json
    import subprocess
    import sys

    code = ("import sys; sys.argv = ['bench.py', '--impl', 'reference', '--workload', 'grid4x5_d12_amps', "
            "'--steps', '1']; import bench; bench.main(); "
            "maps = open('/proc/self/maps').read(); "
            "print('LOADED', int('libpqgb300' in maps), int('pqgb300' in sys.modules), int('torch' in sys.modules))")
    r = subprocess.run([sys.executable, "-c", code], cwd=str(ROOT), capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.strip().splitlines()
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0 and line["cpu_baseline"]["sample"].startswith("timed")
    assert lines[-1] == "LOADED 0 0 0"


def test_recorded_plan_matches_oracle_network():
    """The committed 6x6 depth-16 plan record applies to the network the
    oracle builds itself (same leaves, same index names, in order), and its
    steps form one whole contraction of it."""
    import json

    import bench

    sys.path.insert(0, str(ROOT / "oracle"))
    import tn_oracle as O

    rec = json.loads(bench.PLAN_FILE.read_text())
    net = bench.oracle_network(O, rec)
    assert len(rec["steps"]) == 2 * (len(net.nodes) - 1)
    assert 39.0 < rec["log2_cmacs"] < 40.0 and rec["log2_max_elems"] <= 28.0
    seen = set()
    for i, s in enumerate(rec["steps"]):
        assert s < len(net.nodes) + i // 2 and s not in seen
        seen.add(s)


def test_oracle_amplitude_along_plan_record(pq, O):
    """The bench's oracle pin on a small circuit: a plan record made from the
    product's planner, replayed on the oracle's own network, gives the
    state-vector amplitude."""
    import bench

    rows, cols, depth = 3, 3, 8
    n = rows * cols
    gates = pq.random_grid_gates(rows, cols, depth, seed=2026)
    bits = pq.random_bitstrings(n, 1, seed=2027)[0]
    net = pq.build_network(n, gates, decompose=True, backend=bench._HostStore())
    pq.add_input(net, "0" * n)
    pq.add_output(net, bits)
    steps, cm, mx, name = pq.planning.best_flop_plan(net, out_edges=[], candidates=("sweep",))
    nodes = list(net.nodes.keys())
    rec = {"rows": rows, "cols": cols, "depth": depth, "circuit_seed": 2026, "bitstring": bits, "leaves": nodes,
           "leaf_indices": [list(net.nodes[x].indices) for x in nodes], "steps": steps}
    amp, secs = bench.oracle_amplitude(O, rec)
    ref = O.statevector(n, O.random_grid_gates(rows, cols, depth, seed=2026))[O.amplitude_index(bits)]
    assert abs(amp - ref) < 1e-12 * max(1.0, abs(ref)) and secs >= 0
    rec["leaves"] = nodes[1:] + nodes[:1]
    with pytest.raises(RuntimeError):
        bench.oracle_network(O, rec)


def test_autotune_plan_pairs_and_names(pq):
    """The tuner's view of a plan: each step's operand labels and extents
    under the executor's label rule, steps keeping a shared label skipped;
    and readable choice names."""
    from pqgb300 import autotune as AT

    class Plan:
        ranks = [2, 2, 2, 1]
        flat = [0, 1, 1, 2, 2, 3, 3]
        out_labels = [0]
        steps = [0, 1, 4, 2, 5, 3]
        dims = [4, 8, 3, 5]

    pairs = AT.plan_pairs(Plan)
    assert pairs[0] == ([0, 1], [4, 8], [1, 2], [8, 3])
    assert pairs[1] == ([0, 2], [4, 3], [2, 3], [3, 5])
    assert pairs[2] == ([0, 3], [4, 5], [3], [5])

    class Hyper:  # label 1 is carried by three leaves: the first step keeps it
        ranks = [2, 1, 1]
        flat = [0, 1, 1, 1]
        out_labels = [0]
        steps = [0, 1, 3, 2]
        dims = [2, 3]

    assert AT.plan_pairs(Hyper) == [([0, 1], [2, 3], [1], [3])]
    assert AT.choice_name((2, 64, 2)) == "tcgen05/tn64/swapped" and AT.choice_name((4, 0, 0)) == "skinny"
    assert len(AT.source_hash()) == 16


def test_backend_rejects_unknown_svd_mode(pq):
    """The bond-split location is "host" or "device"; anything else is
    refused before the library is touched."""
    with pytest.raises(ValueError):
        pq.GB300Backend(pq.PREC_C64, svd="gpu")
