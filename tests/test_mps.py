"""The compressed (MPS) contraction path, after the reference's MPS tests
(test/layer2_tests.jl:204-240, :330-350)."""
import numpy as np
import pytest


def _prep_gates(pq, n, seed):
    rng = np.random.default_rng(seed)
    g = [(pq.haar_su2(rng), [q]) for q in range(1, n + 1)]
    g += [(pq.CX, [q, q + 1]) for q in range(1, n)]
    g += [(pq.haar_su2(rng), [q]) for q in range(1, n + 1)]
    return g + pq.ghz_gates(n)


def _mps_vs_full(pq, backend_factory, n=3, seed=0):
    gates = _prep_gates(pq, n, seed)
    be1 = backend_factory()
    tn = pq.build_network(n, gates, backend=be1, decompose=True)
    pq.add_input(tn, "0" * n)
    pq.full_wavefunction_contraction(tn, "vector")
    full = np.asarray(pq.load_tensor_data(tn, "result")).reshape(-1)
    be2 = backend_factory()
    tn = pq.build_network(n, gates, backend=be2, decompose=True)
    pq.add_input(tn, "0" * n)
    mps = pq.contract_mps_tensor_network_circuit(tn)
    pq.calculate_mps_amplitudes(tn, mps)
    mps_wf = np.asarray(pq.load_tensor_data(tn, "result")).reshape(-1)
    return full, mps_wf, gates


def test_mps_matches_full_wavefunction(pq, O):
    full, mps_wf, gates = _mps_vs_full(pq, O.OracleBackend)
    assert np.max(np.abs(full - mps_wf)) < 1e-12
    assert np.max(np.abs(full - O.statevector(3, gates))) < 1e-12


def test_mps_state_ghz5_amplitudes(pq, O):
    be = O.OracleBackend()
    tn = pq.build_network(5, pq.ghz_gates(5), backend=be, decompose=True)
    pq.add_input(tn, "0" * 5)
    mps = pq.contract_mps_tensor_network_circuit(tn)
    st = pq.MPSState(tn, mps)
    assert st.size() == (2,) * 5 and len(st) == 32
    assert abs(st["11111"] - 1 / np.sqrt(2)) < 1e-12 and abs(st["00000"] - 1 / np.sqrt(2)) < 1e-12
    assert abs(st["10101"]) < 1e-12
    assert abs(st[(2, 2, 2, 2, 2)] - st["11111"]) < 1e-15


def test_compression_max_rank_truncates(pq, O):
    """With max_rank 1 the bonds keep one singular value: a product state."""
    be = O.OracleBackend()
    tn = pq.build_network(4, pq.ghz_gates(4), backend=be, decompose=True)
    pq.add_input(tn, "0" * 4)
    mps = pq.contract_mps_tensor_network_circuit(tn, max_rank=1)
    assert all(d == 1 for nl in mps for idx, d in zip(tn.nodes[nl].indices, tn.nodes[nl].dims)
               if tn.edges[idx].virtual)


@pytest.mark.gpu
def test_mps_on_gpu_backend(pq, O):
    full, mps_wf, gates = _mps_vs_full(pq, lambda: pq.GB300Backend(pq.PREC_C128), n=4, seed=3)
    ref = O.statevector(4, gates)
    assert np.max(np.abs(full - ref)) < 1e-12
    assert np.max(np.abs(mps_wf - ref)) < 1e-12
