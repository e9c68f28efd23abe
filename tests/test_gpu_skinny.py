"""Skinny pairs (a large tensor against a small one: K <= 16 contracted, the
small side's free extent <= 16, at least 4096 rows) on the row-per-thread
SIMT kernel vs the FP64 oracle: gates of one to four qubits applied to a
state vector at any qubit positions (the unit-stride qubit contracted or
not), either operand order, complex64 and complex128 storage."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KC_SKINNY = 4


def rand(rng, dims):
    return rng.standard_normal(dims) + 1j * rng.standard_normal(dims)


def rel_err(a, b):
    a, b = np.asarray(a).reshape(-1), np.asarray(b).reshape(-1)
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def step_class(be, A, ia, B, ib):
    """Kernel class of the single step of a two-leaf plan C = A x B (labels in
    ncon form: positive contracted, negative open)."""
    from pqgb300 import _lib as L

    labels, dims = {}, []

    def lab(x, d):
        if x not in labels:
            labels[x] = len(dims)
            dims.append(d)
        return labels[x]

    fa = [lab(x, d) for x, d in zip(ia, A.shape)]
    fb = [lab(x, d) for x, d in zip(ib, B.shape)]
    out = [labels[x] for x in sorted((x for x in labels if x < 0), reverse=True)]
    be.save_tensor_data("pa", A)
    be.save_tensor_data("pb", B)
    h = C.c_void_p()
    L.check(be.lib.pq_plan_create(be.ctx, 2, L.arr(C.c_int32, [len(fa), len(fb)]), L.arr(C.c_int32, fa + fb),
                                  len(dims), L.arr(C.c_int64, dims), 1, L.arr(C.c_int32, [0, 1]), len(out),
                                  L.arr(C.c_int32, out), C.byref(h)), be.ctx, "plan_create")
    f = (C.c_double * 8)()
    L.check(be.lib.pq_plan_step_features(h, f), be.ctx, "features")
    be.lib.pq_plan_destroy(h)
    be.delete_tensor("pa")
    be.delete_tensor("pb")
    return int(f[6])


def gate_labels(n, qubits):
    """ncon labels of an n-qubit state (mode i = qubit i) and of a gate on
    `qubits` (inputs contracted with the state, outputs open)."""
    ia = [-(i + 1) for i in range(n)]
    for j, q in enumerate(qubits):
        ia[q] = j + 1
    ib = [j + 1 for j in range(len(qubits))] + [-(n + 1 + j) for j in range(len(qubits))]
    return ia, ib


@pytest.mark.parametrize("qubits", [[0], [5], [0, 1], [3, 9], [0, 7, 15], [2, 4, 6, 8], [0, 1, 2, 3], [12, 13, 14, 15]],
                         ids=lambda q: "q" + "-".join(map(str, q)))
@pytest.mark.parametrize("prec", [1, 0], ids=["c64", "c128"])
def test_gate_on_state(pq, O, qubits, prec):
    n = 16
    rng = np.random.default_rng(len(qubits) * 31 + qubits[0])
    psi = rand(rng, [2] * n)
    G = rand(rng, [2] * (2 * len(qubits)))
    ia, ib = gate_labels(n, qubits)
    be = pq.GB300Backend(prec)
    assert step_class(be, psi, ia, G, ib) == KC_SKINNY
    be.save_tensor_data("psi", psi)
    be.save_tensor_data("g", G)
    n0 = be.launch_count()
    be.contract_tensors("psi", ia, "g", ib, "out")
    assert be.launch_count() - n0 == 1
    got = be.load_tensor_data("out")
    be.close()
    ref = O.contract_tensors_arrays(psi, ia, G, ib)
    assert rel_err(got, ref) < (2e-6 if prec == 1 else 1e-13)


@pytest.mark.parametrize("prec", [1, 0], ids=["c64", "c128"])
def test_gate_first_operand(pq, O, prec):
    """The small operand first: the kernel takes its rows from B."""
    n = 14
    rng = np.random.default_rng(3)
    psi = rand(rng, [2] * n)
    G = rand(rng, [2] * 4)
    ia, ib = gate_labels(n, [1, 6])
    be = pq.GB300Backend(prec)
    assert step_class(be, G, ib, psi, ia) == KC_SKINNY
    be.save_tensor_data("psi", psi)
    be.save_tensor_data("g", G)
    be.contract_tensors("g", ib, "psi", ia, "out")
    got = be.load_tensor_data("out")
    be.close()
    ref = O.contract_tensors_arrays(G, ib, psi, ia)
    assert rel_err(got, ref) < (2e-6 if prec == 1 else 1e-13)


@pytest.mark.parametrize("k,n", [(1, 16), (16, 1), (16, 16), (8, 12), (3, 5)])
def test_matrix_shapes_and_mixed_storage(pq, O, k, n):
    """Plain matrices (rows 9000: ragged, not a power of two), an outer
    product (K = 1), non-power-of-two K and N; the small operand kept in
    complex128 beside a complex64 large one (the mixed default)."""
    m = 9000
    rng = np.random.default_rng(k * 17 + n)
    A = rand(rng, (m, k)).astype(np.complex64)
    B = rand(rng, (k, n))
    be = pq.GB300Backend(1)
    ia, ib = [-1, 1], [1, -2]
    assert step_class(be, A, ia, B, ib) == KC_SKINNY
    be.save_tensor_data("a", A)
    be.save_tensor_data("b", B)
    be.contract_tensors("a", ia, "b", ib, "c")
    got = be.load_tensor_data("c")
    be.close()
    ref = A.astype(np.complex128) @ B
    assert rel_err(got, ref) < 2e-6


def test_batch_modes_stay_on_other_kernels(pq, O):
    """A label shared by both operands and the result (a batch mode) is not a
    skinny pair; the result is still right."""
    rng = np.random.default_rng(9)
    A = rand(rng, (5000, 4, 3))
    B = rand(rng, (4, 4, 3))
    be = pq.GB300Backend(0)
    from pqgb300 import _lib as L

    be.save_tensor_data("a", A)
    be.save_tensor_data("b", B)
    h = C.c_void_p()
    L.check(be.lib.pq_plan_create(be.ctx, 2, L.arr(C.c_int32, [3, 3]), L.arr(C.c_int32, [0, 1, 3, 1, 2, 3]), 4,
                                  L.arr(C.c_int64, [5000, 4, 4, 3]), 1, L.arr(C.c_int32, [0, 1]), 3,
                                  L.arr(C.c_int32, [0, 2, 3]), C.byref(h)), be.ctx, "plan_create")
    f = (C.c_double * 8)()
    L.check(be.lib.pq_plan_step_features(h, f), be.ctx, "features")
    assert int(f[6]) != KC_SKINNY
    ids = L.arr(C.c_int64, [be.id_of("a"), be.id_of("b")])
    L.check(be.lib.pq_plan_execute(h, ids, be.id_of("r")), be.ctx, "execute")
    got = be.load_tensor_data("r")
    be.lib.pq_plan_destroy(h)
    be.close()
    assert rel_err(got, np.einsum("mkz,knz->mnz", A, B)) < 1e-13


def test_statevector_circuit_amplitudes(pq, O):
    """A 14-qubit circuit contracted gate by gate (every step a skinny pair
    once the state is large) matches the oracle's state vector."""
    n = 14
    gates = pq.random_grid_gates(2, 7, 6, seed=21)
    be = pq.GB300Backend(1)
    net = pq.build_network(n, gates, backend=be)
    pq.add_input(net, "0" * n)
    plan = pq.NetworkPlan(net, steps=pq.planning.statevector_steps(net))
    assert np.sum(plan.features()[:, 6] == KC_SKINNY) > 0
    plan.execute()
    got = plan.result().reshape(-1, order="F")
    plan.close()
    be.close()
    assert rel_err(got, O.statevector(n, gates)) < 2e-6


def test_block_fused_statevector(pq, O):
    """A 16-qubit circuit fused into blocks of at most four qubits, applied
    block by block (16 x 16 skinny pairs), matches the oracle's state vector
    of the unfused circuit."""
    from pqgb300 import circuits as CI

    n = 16
    gates = pq.random_grid_gates(4, 4, 10, seed=23)
    blocks = CI.fuse_gates(gates, 4)
    be = pq.GB300Backend(1)
    net = pq.build_network(n, blocks, backend=be)
    pq.add_input(net, "0" * n)
    plan = pq.NetworkPlan(net, steps=pq.planning.statevector_steps(net))
    f = plan.features()
    assert np.sum((f[:, 6] == KC_SKINNY) & (f[:, 3] == 4.0)) > 0  # 4-qubit blocks: K = 16
    plan.execute()
    got = plan.result().reshape(-1, order="F")
    plan.close()
    be.close()
    assert rel_err(got, O.statevector(n, gates)) < 2e-6


@pytest.mark.parametrize("prec", [1, 0], ids=["c64", "c128"])
def test_block_fused_amplitudes_4x5(pq, O, prec):
    """The 4x5 depth-12 circuit fused into blocks of up to four qubits, the
    flop-count planner choosing among sweep, greedy, full-wavefunction and
    state-vector orders: 1024 amplitudes gathered from the open-output result
    match the oracle's state vector of the unfused circuit."""
    from pqgb300 import circuits as CI

    n = 20
    gates = pq.random_grid_gates(4, 5, 12, seed=2024)
    be = pq.GB300Backend(prec)
    net = pq.build_network(n, CI.fuse_gates(gates, 4), backend=be)
    pq.add_input(net, "0" * n)
    steps, _, _, name = pq.planning.best_flop_plan(
        net, trials=2, candidates=("sweep", "greedy", "wavefunction", "statevector"))
    plan = pq.NetworkPlan(net, steps=steps)
    bits = pq.random_bitstrings(n, 1024, seed=7)
    got = np.asarray(plan.amplitudes(bits))
    plan.close()
    be.close()
    ref = O.statevector(n, gates)[[O.amplitude_index(b) for b in bits]]
    scale = np.sqrt(np.mean(np.abs(ref) ** 2))
    assert np.max(np.abs(got - ref)) / scale < (2e-5 if prec == 1 else 1e-11)
