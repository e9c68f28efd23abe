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


def test_mps_state_ghz5_amplitudes(pq, host_backend):
    be = host_backend
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


@pytest.mark.gpu
def test_mps_state_on_gpu_backend(pq, O):
    """MPSState amplitudes from device copies of the MPS tensors, contracted
    on the device, against the oracle's state vector (every bitstring of a
    5-qubit random circuit)."""
    n = 5
    gates = _prep_gates(pq, n, 7)
    for prec, tol in ((pq.PREC_C128, 1e-12), (pq.PREC_C64, 2e-6)):
        be = pq.GB300Backend(prec)
        tn = pq.build_network(n, gates, backend=be, decompose=True)
        pq.add_input(tn, "0" * n)
        mps = pq.contract_mps_tensor_network_circuit(tn)
        st = pq.MPSState(tn, mps)
        sv = O.statevector(n, gates)
        for k in range(2 ** n):
            bits = "".join("1" if (k >> i) & 1 else "0" for i in range(n))
            assert abs(st[bits] - sv[O.amplitude_index(bits)]) < tol
        used = be.mem_in_use()
        st.close()
        assert be.mem_in_use() < used
        be.close()


def _compress_chain_cases(pq, be):
    """test/layer2_tests.jl:240-305 restated: (a) two input vectors
    compressed as a chain stay two nodes; (b) H then three CX on two qubits,
    the gates split by decompose_tensor, every non-virtual closed edge
    contracted, then the chain [node_18, node_19] compressed: the three
    parallel bonds collapse to one of extent 2 (index_14)."""
    tn = pq.TensorNetworkCircuit(2, be)
    pq.add_input(tn, "00")
    pq.compress_tensor_chain(tn, list(tn.nodes))
    assert len(tn.nodes) == 2
    from pqgb300.mps import decompose_tensor

    tn = pq.build_network(2, [(pq.H, [1]), (pq.CX, [1, 2]), (pq.CX, [1, 2]), (pq.CX, [1, 2])], backend=be)
    pq.add_input(tn, "00")
    decompose_tensor(tn, "node_2", ["index_3", "index_4"], ["index_2", "index_5"])
    decompose_tensor(tn, "node_3", ["index_4", "index_6"], ["index_5", "index_7"])
    decompose_tensor(tn, "node_4", ["index_6", "index_8"], ["index_7", "index_9"])
    plan = [k for k, v in tn.edges.items() if not v.virtual and v.src is not None and v.dst is not None]
    for e in plan:
        pq.contract_pair(tn, e)
    pq.compress_tensor_chain(tn, ["node_18", "node_19"])
    idx = tn.nodes["node_18"].indices.index("index_14")
    assert np.asarray(be.load_tensor_data("node_18")).shape[idx] == 2
    return tn


def test_compress_tensor_chain_reference_cases(pq, host_backend):
    _compress_chain_cases(pq, host_backend)


def _inorder_vs_statevector(pq, O, be, n=5, seed=9, tol=1e-12):
    """inorder_contraction (src/layer2.jl:78-112) absorbs every gate into its
    qubit's line, leaving one node per qubit joined by virtual bonds, each
    pair of nodes by at most one bond (merge_common_bonds; the two CZs on
    qubits 1-2 at the end share a layer pair); contracting those nodes then
    gives the state."""
    rng = np.random.default_rng(seed)
    gates = []
    for layer in range(4):
        gates += [(pq.haar_su2(rng), [q]) for q in range(1, n + 1)]
        gates += [(pq.CZ, [q, q + 1]) for q in range(1 + layer % 2, n, 2)]
    gates += [(pq.CZ, [1, 2]), (pq.CZ, [1, 2])]
    tn = pq.build_network(n, gates, backend=be, decompose=True)
    pq.add_input(tn, "0" * n)
    pq.inorder_contraction(tn)
    assert len(tn.nodes) == n
    labels = list(tn.nodes)
    for i, x in enumerate(labels):
        for y in labels[i + 1:]:
            assert len(set(tn.nodes[x].indices) & set(tn.nodes[y].indices)) <= 1
    cur = labels[0]
    for y in labels[1:]:
        cur = pq.contract_pair(tn, cur, y)
    node = tn.nodes[cur]
    outs = [tn.output_qubits[q - 1] for q in tn.qubit_ordering]
    data = np.asarray(be.load_tensor_data(node.data_label))
    vec = np.transpose(data, [node.indices.index(x) for x in outs]).reshape(-1, order="F")
    sv = O.statevector(n, gates)
    assert np.max(np.abs(vec - sv)) < tol
    return tn


def test_inorder_contraction_matches_statevector(pq, O, host_backend):
    _inorder_vs_statevector(pq, O, host_backend)


def test_merge_common_bonds_merges_parallel_bonds(pq, host_backend):
    """Two nodes joined by three bonds (held in different orders) end joined
    by one new virtual bond of the product extent, and contracting over it
    gives the contraction over the three bonds."""
    be = host_backend
    tn = pq.TensorNetworkCircuit(1, be)
    rng = np.random.default_rng(2)
    a = rng.standard_normal((2, 3, 2, 4)) + 0j
    b = rng.standard_normal((4, 3, 5, 2)) + 0j
    tn.nodes["node_1"] = pq.Node(["index_2", "index_3", "index_4", "index_5"], [2, 3, 2, 4], "node_1")
    tn.nodes["node_2"] = pq.Node(["index_5", "index_3", "index_6", "index_4"], [4, 3, 5, 2], "node_2")
    for e in ("index_3", "index_4", "index_5"):
        tn.edges[e] = pq.Edge("node_1", "node_2", None, True)
    tn.edges["index_2"] = pq.Edge(None, "node_1", None, False)
    tn.edges["index_6"] = pq.Edge("node_2", None, None, False)
    tn.counters["index"] = 6
    tn.counters["node"] = 2
    be.save_tensor_data("node_1", a)
    be.save_tensor_data("node_2", b)
    pq.merge_common_bonds(tn, "node_1", "node_2")
    assert tn.nodes["node_1"].indices == ["index_2", "index_7"] and tn.nodes["node_1"].dims == [2, 24]
    assert tn.nodes["node_2"].indices == ["index_6", "index_7"] and tn.nodes["node_2"].dims == [5, 24]
    assert "index_3" not in tn.edges and tn.edges["index_7"].virtual
    ref = np.einsum("ajkl,ljbk->ab", a, b)
    got = np.asarray(be.load_tensor_data("node_1")) @ np.asarray(be.load_tensor_data("node_2")).T
    assert np.max(np.abs(got - ref)) < 1e-12


@pytest.mark.gpu
def test_compression_and_inorder_on_gpu_backend(pq, O):
    for prec, tol in ((pq.PREC_C128, 1e-12), (pq.PREC_C64, 2e-6)):
        be = pq.GB300Backend(prec)
        _compress_chain_cases(pq, be)
        be.close()
        be = pq.GB300Backend(prec)
        _inorder_vs_statevector(pq, O, be, tol=tol)
        be.close()
