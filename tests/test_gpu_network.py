"""The reference's known answers and circuit workloads through GB300Backend.

Tolerances: complex128 1e-12 (config 1 asks for 1e-12), complex64 1e-6
relative (max-abs error over the largest reference magnitude).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = np.asarray(a).reshape(-1)
    b = np.asarray(b).reshape(-1)
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.fixture(params=[0, 1], ids=["c128", "c64"])
def prec(request):
    return request.param


TOL = {0: 1e-12, 1: 1e-6}


def test_ghz3_amplitude(pq, O, prec):
    for seed in range(3):
        be = pq.GB300Backend(prec)
        net = pq.build_network(3, pq.ghz_gates(3), backend=be)
        pq.add_input(net, "000")
        pq.add_output(net, "000")
        pq.contract_network(net, pq.random_contraction_plan(net, np.random.default_rng(seed)))
        assert len(net.nodes) == 1
        assert abs(pq.load_tensor_data(net, "result") - 1 / math.sqrt(2)) < TOL[prec]
        be.close()


def test_hadamard_pair_vector(pq, prec):
    be = pq.GB300Backend(prec)
    net = pq.build_network(2, [(pq.H, [1]), (pq.H, [2])], backend=be)
    pq.add_input(net, "00")
    pq.contract_network(net, pq.random_contraction_plan(net, np.random.default_rng(0)), "vector")
    r = pq.load_tensor_data(net, "result")
    assert r.ndim == 1 and abs(r.real[0] - 0.5) < TOL[prec]
    be.close()


def test_metrics_golden(pq, prec):
    be = pq.GB300Backend(prec)
    net = pq.build_network(3, [(pq.H, [1]), (pq.CX, [1, 2]), (pq.CX, [1, 2]), (pq.CX, [1, 3])], backend=be)
    pq.add_input(net, "000")
    pq.full_wavefunction_contraction(net, "vector")
    m = be.metrics
    assert (m.max_tensor_size, m.total_space_allocated, m.flops) == (8, 44, 124)
    ref = np.zeros(8)
    ref[0] = ref[5] = 1 / math.sqrt(2)  # |000> + |101>
    assert rel(pq.load_tensor_data(net, "result"), ref) < TOL[prec]
    be.close()


def test_config1_qft10_full_wavefunction(pq, O):
    # 10-qubit QFT on |0..0>, reference default plan, complex128, within 1e-12
    be = pq.GB300Backend(pq.PREC_C128)
    net = pq.build_network(10, pq.qft_gates(10), backend=be)
    pq.add_input(net, "0" * 10)
    pq.full_wavefunction_contraction(net, "vector")
    got = pq.load_tensor_data(net, "result")
    onet = O.build_network(10, O.qft_gates(10))
    O.add_input(onet, "0" * 10)
    O.full_wavefunction_contraction(onet, "vector")
    ref = onet.backend.load_tensor_data("result")
    assert got.shape == (1024,)
    assert np.max(np.abs(got - ref)) < 1e-12
    assert np.max(np.abs(got - 1 / 32)) < 1e-12
    be.close()


@pytest.mark.parametrize("n", [3, 8])
def test_qft_is_normalised_ifft(pq, O, prec, n):
    prep = O.simple_preparation_gates(n, 3, np.random.default_rng(43))
    inp = O.statevector(n, prep)
    be = pq.GB300Backend(prec)
    net = pq.build_network(n, prep + pq.qft_gates(n), backend=be)
    pq.add_input(net, "0" * n)
    pq.full_wavefunction_contraction(net, "vector")
    out = pq.load_tensor_data(net, "result")

    def big(v):
        return v.reshape((2,) * n).transpose().reshape(-1)

    ref = np.fft.ifft(big(inp))
    ref /= np.linalg.norm(ref)
    assert abs(abs(np.vdot(big(out), ref)) - 1) < 10 * TOL[prec]
    be.close()


def test_slices_sum_to_unsliced(pq, O, prec):
    n = 4
    circ = O.simple_preparation_gates(n, 2, np.random.default_rng(2)) + pq.qft_gates(n)
    full = O.statevector(n, circ)
    tot = 0
    for p in range(1, 5):
        be = pq.GB300Backend(prec)
        net = pq.build_network(n, circ, decompose=True, backend=be)
        pq.add_input(net, "0" * n)
        bl, bv = pq.partition_network_on_virtual_bonds(net, 4, p)
        pq.slice_tensor_network(net, bl, bv)
        pq.full_wavefunction_contraction(net, "vector")
        tot = tot + pq.load_tensor_data(net, "result")
        be.close()
    assert rel(tot, full) < TOL[prec]


def test_decompose_round_trip(pq, O, prec):
    rng = np.random.default_rng(7)
    gd = rng.random((2, 2, 2, 2)) + 1j * rng.random((2, 2, 2, 2))
    be = pq.GB300Backend(prec)
    net = pq.TensorNetworkCircuit(2, be)
    labs = pq.add_gate(net, gd, [1, 2], decompose=True)
    r = pq.contract_pair(net, *labs)
    got = O.permute_array(pq.load_tensor_data(net, r), [1, 3, 2, 4])
    assert rel(got, gd) < 10 * TOL[prec]
    be.close()


@pytest.mark.parametrize("shape", [(2, 3, 6), (3, 3, 8), (3, 4, 10)])
def test_random_grid_full_wavefunction(pq, O, prec, shape):
    r, c, d = shape
    n = r * c
    g = pq.random_grid_gates(r, c, d, seed=n + d)
    be = pq.GB300Backend(prec)
    net = pq.build_network(n, g, backend=be)
    pq.add_input(net, "0" * n)
    pq.full_wavefunction_contraction(net, "vector")
    assert rel(pq.load_tensor_data(net, "result"), O.statevector(n, g)) < TOL[prec]
    be.close()


GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden" / "reference_examples"


def test_reference_json_network_edge_plan(pq, prec):
    """A network produced by the reference (examples/ghz_3.json, copied in
    tests/golden), loaded through network_from_json onto the GB300 backend
    and contracted along the reference's edge plan (ghz_3_plan.json), gives
    the reference's own contracted network (ghz_3_contracted.json): node
    name, index order and data."""
    import json

    be = pq.GB300Backend(prec)
    net = pq.network_from_json((GOLDEN / "ghz_3.json").read_text(), be)
    for e in json.loads((GOLDEN / "ghz_3_plan.json").read_text()):
        pq.contract_pair(net, e)
    want = json.loads((GOLDEN / "ghz_3_contracted.json").read_text())
    assert list(net.nodes) == ["node_5"] and list(net.edges) == list(want["edges"])
    w = want["nodes"]["node_5"]
    assert net.nodes["node_5"].indices == w["indices"]
    got = np.asarray(be.load_tensor_data("node_5")).reshape(-1, order="F")
    ref = np.asarray(w["data_re"]) + 1j * np.asarray(w["data_im"])
    assert np.max(np.abs(got - ref)) <= TOL[prec]
    be.close()


def test_json_round_trip_contracts_on_gpu(pq, O, prec):
    """A random circuit's network written with its data (to_json with
    with_data=True), read back onto a fresh GB300 backend and contracted by
    a compiled plan, gives the oracle's amplitude of the original circuit."""
    n = 12
    gates = pq.random_grid_gates(3, 4, 8, seed=5)
    bits = pq.random_bitstrings(n, 1, seed=6)[0]
    be0 = pq.GB300Backend(pq.PREC_C128)
    net0 = pq.build_network(n, gates, decompose=True, backend=be0)
    pq.add_input(net0, "0" * n)
    pq.add_output(net0, bits)
    text = pq.to_json(net0, with_data=True)
    be0.close()
    be = pq.GB300Backend(prec)
    net = pq.network_from_json(text, be)
    steps, _, _, _ = pq.planning.best_flop_plan(net, out_edges=[])
    plan = pq.NetworkPlan(net, steps=steps, out_edges=[])
    plan.execute()
    amp = complex(np.asarray(plan.result()).reshape(-1)[0])
    plan.close()
    ref = O.statevector(n, O.random_grid_gates(3, 4, 8, seed=5))[O.amplitude_index(bits)]
    assert abs(amp - ref) <= TOL[prec] * 2.0 ** (-n / 2) * 8
    be.close()
