"""Pin the FP64 oracle against the reference's own known-answer tests."""
import math
from pathlib import Path

import numpy as np
import pytest


def test_ghz3_single_amplitude(O):
    # test/layer1_tests.jl:11-46: <000|GHZ> = 1/sqrt(2) with a random edge plan
    for seed in range(4):
        net = O.build_network(3, O.ghz_gates(3))
        O.add_input(net, "000")
        O.add_output(net, "000")
        O.contract_network(net, O.random_contraction_plan(net, np.random.default_rng(seed)))
        assert abs(net.backend.load_tensor_data("result") - 1 / math.sqrt(2)) < 1e-15


def test_hadamard_pair_disjoint(O):
    # test/layer2_tests.jl:69-103: disjoint network, vector output, real(result)[1] = 1/2
    net = O.build_network(2, [(O.GATES["H"], [1]), (O.GATES["H"], [2])])
    O.add_input(net, "00")
    O.contract_network(net, O.random_contraction_plan(net, np.random.default_rng(0)), "vector")
    assert len(net.nodes) == 1
    r = net.backend.load_tensor_data("result")
    assert r.ndim == 1 and abs(r.real[0] - 0.5) < 1e-15


def test_metrics_golden(O):
    # test/layer2_tests.jl:106-143: h; cx01; cx01; cx02 on |000>, full wavefunction
    net = O.build_network(3, [(O.GATES["H"], [1]), (O.CX, [1, 2]), (O.CX, [1, 2]), (O.CX, [1, 3])])
    O.add_input(net, "000")
    O.full_wavefunction_contraction(net, "vector")
    m = net.backend.metrics
    assert (m.max_tensor_size, m.total_space_allocated, m.flops) == (8, 44, 124)
    assert len(net.nodes) == 1


def test_qft10_closed_form(O):
    # QFT on |0..0> gives the uniform state 1/32 (config 1)
    net = O.build_network(10, O.qft_gates(10))
    O.add_input(net, "0" * 10)
    O.full_wavefunction_contraction(net, "vector")
    r = net.backend.load_tensor_data("result")
    assert r.shape == (1024,)
    assert np.max(np.abs(r - 1 / 32)) < 1e-15


@pytest.mark.parametrize("n", [3, 8])
def test_qft_is_normalised_ifft(O, n):
    # test/algorithms_tests.jl:39-82 with the endianness switch of test/test_utils.jl:12-17
    prep = O.simple_preparation_gates(n, 3, np.random.default_rng(43))
    inp = O.statevector(n, prep)
    net = O.build_network(n, prep + O.qft_gates(n))
    O.add_input(net, "0" * n)
    O.full_wavefunction_contraction(net, "vector")
    out = net.backend.load_tensor_data("result")

    def big_endian(v):
        return v.reshape((2,) * n).transpose().reshape(-1)

    ref = np.fft.ifft(big_endian(inp))
    ref /= np.linalg.norm(ref)
    assert abs(abs(np.vdot(big_endian(out), ref)) - 1) < 1e-12


def test_slices_sum_to_unsliced(O):
    # test/layer2_tests.jl:419-455: 4 qubits, decompose, 4 partitions
    n = 4
    circ = O.simple_preparation_gates(n, 2, np.random.default_rng(2)) + O.qft_gates(n)
    net = O.build_network(n, circ, decompose=True)
    O.add_input(net, "0" * n)
    O.full_wavefunction_contraction(net, "vector")
    wf = net.backend.load_tensor_data("result")
    tot = 0
    for p in range(1, 5):
        net = O.build_network(n, circ, decompose=True)
        O.add_input(net, "0" * n)
        bl, bv = O.partition_network_on_virtual_bonds(net, 4, p)
        O.slice_tensor_network(net, bl, bv)
        O.full_wavefunction_contraction(net, "vector")
        tot = tot + net.backend.load_tensor_data("result")
    assert np.max(np.abs(tot - wf)) < 1e-14
    assert np.max(np.abs(wf - O.statevector(n, circ))) < 1e-13


def test_decompose_round_trip(O):
    # test/layer3_tests.jl:57-71
    rng = np.random.default_rng(7)
    gd = rng.random((2, 2, 2, 2)) + 1j * rng.random((2, 2, 2, 2))
    net = O.TensorNetworkCircuit(2)
    labs = O.add_gate(net, gd, [1, 2], decompose=True)
    r = O.contract_pair(net, *labs)
    assert np.max(np.abs(O.permute_array(net.backend.tensors[r], [1, 3, 2, 4]) - gd)) < 1e-13


def test_structure_counts(O):
    # test/layer3_tests.jl:154-171, 189-203, 221-240
    net = O.TensorNetworkCircuit(3)
    O.add_gate(net, O.operator_to_tensor(O.GATES["H"]), [1])
    assert len(net.nodes) == 1 and len(net.edges) == 4
    net = O.build_network(3, [(O.GATES["H"], [1]), (O.CX, [1, 2]), (O.CX, [2, 3])], decompose=True)
    assert len(net.nodes) == 5
    net = O.TensorNetworkCircuit(3)
    O.add_input(net, "000")
    assert len(net.nodes) == 3
    O.add_output(net, "000")
    assert len(net.nodes) == 6
    O.add_input(net, "000")
    O.add_output(net, "000")
    assert len(net.nodes) == 6


def test_bgreedy_plan_contracts(O):
    # test/layer2_tests.jl:175-203
    net = O.build_network(3, [(O.GATES["H"], [1]), (O.CX, [1, 2]), (O.CX, [1, 3])])
    O.add_input(net, "000")
    O.add_output(net, "000")
    plan, cost = O.bgreedy(net, 1, 1, 10, np.random.default_rng(0))
    O.contract_network(net, plan)
    assert len(net.nodes) == 1
    assert abs(net.backend.load_tensor_data("result") - 1 / math.sqrt(2)) < 1e-15


def test_random_circuits_match_statevector(O):
    for seed, (r, c, d) in enumerate([(2, 2, 4), (2, 3, 5), (3, 3, 4)]):
        g = O.random_grid_gates(r, c, d, seed)
        for dec in (False, True):
            net = O.build_network(r * c, g, decompose=dec)
            O.add_input(net, "0" * (r * c))
            O.full_wavefunction_contraction(net, "vector")
            assert np.max(np.abs(net.backend.load_tensor_data("result") - O.statevector(r * c, g))) < 1e-13


def test_multi_index_partition(O):
    # column-major CartesianIndices, slicing.jl:12-26
    assert O.multi_index_partition((2, 2, 2), 4, 1) == (1, 1)
    assert O.multi_index_partition((2, 2, 2), 4, 2) == (2, 1)
    assert O.multi_index_partition((2, 2, 2), 4, 3) == (1, 2)
    assert O.multi_index_partition((2, 3, 2), 6, 6) == (2, 3)


GOLDEN = Path(__file__).resolve().parent / "golden" / "reference_examples"


@pytest.mark.parametrize("name,n", [("qft_2", 2), ("qft_3", 3), ("qft_5", 5), ("qft_10", 10), ("ghz_3", 3)])
def test_reference_qasm_fixtures(O, name, n):
    # examples/*.qasm of the reference (copies in tests/golden): transpiled QFT /
    # GHZ circuits; on |0..0> the QFT gives the uniform state and GHZ gives
    # (|0..0> + |1..1>)/sqrt(2).
    gates = O.parse_qasm((GOLDEN / f"{name}.qasm").read_text())
    net = O.build_network(n, gates)
    O.add_input(net, "0" * n)
    O.full_wavefunction_contraction(net, "vector")
    out = net.backend.load_tensor_data("result")
    sv = O.statevector(n, gates)
    assert np.max(np.abs(out - sv)) < 1e-13
    if name.startswith("qft"):
        assert np.max(np.abs(np.abs(out) - 2 ** (-n / 2))) < 1e-12
    else:
        ref = np.zeros(2**n)
        ref[0] = ref[-1] = 1 / math.sqrt(2)
        assert np.max(np.abs(np.abs(out) - ref)) < 1e-12


def test_reference_edge_plan_golden(O):
    """examples/ghz_3.json contracted along examples/ghz_3_plan.json (edges
    index_4 then index_6, one contract_pair! each) gives the network the
    reference wrote to examples/ghz_3_contracted.json: the node name
    (node_5), its index order (symdiff of the operands' indices,
    src/layer1.jl:89) and its data."""
    import json

    net = O.network_from_dict(json.loads((GOLDEN / "ghz_3.json").read_text()))
    plan = json.loads((GOLDEN / "ghz_3_plan.json").read_text())
    for e in plan:
        O.contract_pair(net, e)
    want = json.loads((GOLDEN / "ghz_3_contracted.json").read_text())
    assert list(net.nodes) == list(want["nodes"]) == ["node_5"]
    assert list(net.edges) == list(want["edges"])
    for k, e in want["edges"].items():
        assert (net.edges[k].src, net.edges[k].dst) == (e["src"], e["dst"])
    w = want["nodes"]["node_5"]
    assert net.nodes["node_5"].indices == w["indices"] and net.nodes["node_5"].dims == w["data_dims"]
    got = np.asarray(net.backend.load_tensor_data("node_5")).reshape(-1, order="F")
    ref = np.asarray(w["data_re"]) + 1j * np.asarray(w["data_im"])
    assert np.max(np.abs(got - ref)) < 1e-15


def test_mlp_oracle_gradient_finite_differences():
    # pins the MLP oracle used to check the GPU training kernels
    import mlp_oracle as MO

    rng = np.random.default_rng(0)
    n_in, hidden, layers = 5, 7, 3
    npar = sum(a * b + b for a, b in MO.layer_shapes(n_in, hidden, layers))
    p = rng.standard_normal(npar)
    X = rng.standard_normal((11, n_in))
    y = rng.standard_normal(11)
    loss, g = MO.loss_and_grad(p, X, y, n_in, hidden, layers)
    eps = 1e-6
    for i in rng.choice(npar, 25, replace=False):
        q = p.copy()
        q[i] += eps
        lp, _ = MO.loss_and_grad(q, X, y, n_in, hidden, layers)
        q[i] -= 2 * eps
        lm, _ = MO.loss_and_grad(q, X, y, n_in, hidden, layers)
        assert abs((lp - lm) / (2 * eps) - g[i]) < 1e-6 * max(1.0, abs(g[i]))
