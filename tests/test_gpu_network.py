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
