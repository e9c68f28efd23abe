"""FP64 CPU oracle for the tensor-network contraction path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product package imports this
module; only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py`` use it, and only as the checker / the timed CPU baseline.

This is a plain numpy restatement (complex128 everywhere) of PicoQuant.jl's
contraction semantics, written from the reference's behaviour:

* circuit -> graph bookkeeping            src/layer3.jl:93-118, 145-313
* 2-qubit gate SVD split (``decompose``)  src/layer3.jl:715-739
* pairwise contraction ``contract_pair!`` src/layer2.jl:346-405
* index classification / ncon labels      src/layer2.jl:209-240
* full-wavefunction order                 src/layer2.jl:132-195
* plan execution (pair plan / edge plan)  src/layer2.jl:250-321
* cost metrics                            src/backends.jl:8-57
* InteractiveBackend storage semantics    src/backends/interactive.jl:10-172
* L1 array kernels (tensorcontract etc.)  src/layer1.jl:85-125, 191-194
* slicing on virtual bonds                src/layer2/slicing.jl:12-110
* Boltzmann-greedy planner                src/layer2/bgreedy_contraction.jl:17-131
* circuit generators (QFT, GHZ, prep)     src/algorithms.jl:14-89

Arrays follow the reference's (Julia) index semantics: a tensor with dims
``(d1, ..., dr)`` is a numpy array of that shape indexed the same way; any
flattening uses column-major order (``order='F'``), matching Julia.

The third-party arithmetic behind ``tensorcontract`` (TensorOperations.jl 3.x
-> BLAS) is restated with ``numpy.tensordot`` (-> BLAS zgemm): contract the
shared labels, output modes in ``symdiff(ia, ib)`` order.

Parity status: pinned against the reference's own known-answer tests
(test/layer1_tests.jl:34-39, test/layer2_tests.jl:97-100, :127-132,
:419-455, test/layer3_tests.jl:57-71, test/algorithms_tests.jl:39-82) and
against an independent state-vector simulator in this module; the reference
itself (Julia) cannot run in this environment.
"""
from __future__ import annotations

import math
from collections import OrderedDict
from dataclasses import dataclass, field

import numpy as np

CDT = np.complex128

# --------------------------------------------------------------------------
# Metrics (src/backends.jl:8-57)
# --------------------------------------------------------------------------


@dataclass
class Metrics:
    max_tensor_size: int = 0
    total_space_allocated: int = 0
    flops: int = 0


def record_compute_costs(metrics: Metrics, open_dims, contracted_dims):
    """src/backends.jl:30-41: space += prod(open); flops += prod(open)*prod(contracted)."""
    space = int(np.prod(open_dims, dtype=np.int64)) if len(open_dims) else 1
    record_memory_costs(metrics, space)
    fl = space * (int(np.prod(contracted_dims, dtype=np.int64)) if len(contracted_dims) else 1)
    metrics.flops += fl
    return fl, space


def record_memory_costs(metrics: Metrics, mem: int):
    """src/backends.jl:50-57."""
    metrics.total_space_allocated += mem
    if mem > metrics.max_tensor_size:
        metrics.max_tensor_size = mem


# --------------------------------------------------------------------------
# L1 array kernels (src/layer1.jl:85-125, 191-194)
# --------------------------------------------------------------------------


def symdiff(a, b):
    """Julia ``symdiff`` on index tuples: a∖b (a order) then b∖a (b order)."""
    out = [x for x in a if x not in b]
    seen = set(out)
    for x in b:
        if x not in a and x not in seen:
            out.append(x)
    return out


def contract_tensors_arrays(A, ia, B, ib):
    """src/layer1.jl:85-92: ``tensorcontract(A, ia, B, ib, symdiff(ia, ib))``.

    Labels present in both are summed; output modes are A's remaining labels
    (A order) followed by B's remaining labels (B order).
    """
    ia, ib = list(ia), list(ib)
    common = [x for x in ia if x in ib]
    pa = [ia.index(x) for x in common]
    pb = [ib.index(x) for x in common]
    C = np.tensordot(A, B, axes=(pa, pb))
    # tensordot already yields A-free then B-free in their original orders,
    # which is symdiff order.
    return C


def permute_array(A, perm1):
    """src/layer1.jl:111-114 (permutedims); ``perm1`` is 1-based."""
    return np.transpose(A, [p - 1 for p in perm1]).copy()


def reshape_array(A, dims):
    """src/layer1.jl:100-103 (column-major reshape)."""
    return np.reshape(A, tuple(int(d) for d in dims), order="F")


def tensor_view_array(A, bond_idx1, lo1, hi1):
    """src/layer1.jl:191-194: copy with mode ``bond_idx`` narrowed to lo:hi (1-based)."""
    sl = [slice(None)] * A.ndim
    sl[bond_idx1 - 1] = slice(lo1 - 1, hi1)
    return A[tuple(sl)].copy()


# --------------------------------------------------------------------------
# Interactive (numpy, FP64) backend (src/backends/interactive.jl)
# --------------------------------------------------------------------------


class OracleBackend:
    """InteractiveBackend{Array{ComplexF64}} restated with numpy."""

    def __init__(self):
        self.tensors: dict[str, np.ndarray] = {}
        self.metrics = Metrics()

    def save_tensor_data(self, label, data):
        self.tensors[label] = np.array(data, dtype=CDT)

    def load_tensor_data(self, label):
        return self.tensors.get(label)

    def contract_tensors(self, A, ia, B, ib, C):
        """src/backends/interactive.jl:60-75 (A and B are consumed)."""
        self.tensors[C] = contract_tensors_arrays(self.tensors[A], ia, self.tensors[B], ib)
        del self.tensors[A]
        del self.tensors[B]

    def save_output(self, node, name="result"):
        self.tensors[name] = self.tensors[node]

    def reshape_tensor(self, t, groups):
        dims = self.tensors[t].shape
        self.tensors[t] = reshape_array(self.tensors[t], [int(np.prod([dims[i - 1] for i in g])) for g in groups])

    def permute_tensor(self, t, perm1):
        self.tensors[t] = permute_array(self.tensors[t], perm1)

    def delete_tensor(self, t):
        self.tensors.pop(t, None)

    def view_tensor(self, view, node, bond_idx1, lo1, hi1):
        self.tensors[view] = tensor_view_array(self.tensors[node], bond_idx1, lo1, hi1)

    def decompose_tensor(self, tensor, left_positions, right_positions, threshold=1e-13, max_rank=0,
                         left_label=None, right_label=None):
        """src/backends/interactive.jl:124-151 -> src/layer1.jl:146-184: SVD
        across (left | right) positions (1-based); singular values kept while
        s / ||s|| exceeds max(threshold, sqrt(eps)); returns the bond extent."""
        t = self.tensors[tensor]
        ld = [t.shape[x - 1] for x in left_positions]
        rd = [t.shape[x - 1] for x in right_positions]
        A = np.transpose(t, [x - 1 for x in list(left_positions) + list(right_positions)])
        A = np.reshape(A, (int(np.prod(ld)), int(np.prod(rd))), order="F")
        U, S, Vh = np.linalg.svd(A, full_matrices=False)
        thr = max(threshold, float(np.sqrt(np.finfo(np.float64).eps)))
        norm = float(np.sqrt(np.sum(S ** 2)))
        chi = int(np.sum(S / norm > thr)) if norm > 0 else 0
        if max_rank > 0:
            chi = min(chi, max_rank)
        sq = np.sqrt(S[:chi])
        self.tensors[left_label] = np.reshape(U[:, :chi] * sq[None, :], tuple(ld) + (chi,), order="F")
        self.tensors[right_label] = np.reshape(sq[:, None] * Vh[:chi, :], (chi,) + tuple(rd), order="F")
        del self.tensors[tensor]
        return chi


# --------------------------------------------------------------------------
# L3: tensor network circuit (src/layer3.jl)
# --------------------------------------------------------------------------


@dataclass
class Node:
    indices: list
    dims: list
    data_label: str


@dataclass
class Edge:
    src: str | None
    dst: str | None
    qubit: int | None
    virtual: bool = False


class TensorNetworkCircuit:
    """src/layer3.jl:56-118."""

    def __init__(self, qubits: int, backend=None):
        self.backend = backend if backend is not None else OracleBackend()
        self.number_qubits = qubits
        labels = [f"index_{i}" for i in range(1, qubits + 1)]
        self.edges: OrderedDict[str, Edge] = OrderedDict()
        for i in range(1, qubits + 1):
            self.edges[labels[i - 1]] = Edge(None, None, i, False)
        self.input_qubits = list(labels)
        self.output_qubits = list(labels)
        self.nodes: OrderedDict[str, Node] = OrderedDict()
        self.qubit_ordering = list(range(1, qubits + 1))
        self.counters = {"index": qubits, "node": 0, "layer": 0}
        self.node_layers: dict[str, int] = {}

    def new_label(self, s):
        """src/layer3.jl:145-148."""
        self.counters[s] += 1
        return f"{s}_{self.counters[s]}"


def network_from_dict(d, backend=None):
    """src/layer3.jl:654-681 (``network_from_dict``): edges and nodes in the
    file's order, label counters continued after the largest numbers
    present.  Also reads the older form of the reference's example networks
    (examples/ghz_3.json), whose nodes embed their tensor (``data_re``,
    ``data_im`` flattened column-major, ``data_dims``; the node name is its
    data label) and whose edges carry only src/dst."""
    net = TensorNetworkCircuit(int(d["number_qubits"]), backend)
    net.edges = OrderedDict()
    index = 0
    for k, v in d["edges"].items():
        index = max(index, int(k.split("_")[-1]))
        net.edges[k] = Edge(v["src"], v["dst"], v.get("qubit"), bool(v.get("virtual", False)))
    net.nodes = OrderedDict()
    node = 0
    for k, v in d["nodes"].items():
        node = max(node, int(k.split("_")[-1]))
        if "data_re" in v:
            dims = [int(x) for x in v["data_dims"]]
            data = (np.asarray(v["data_re"], dtype=np.float64) + 1j * np.asarray(v["data_im"], dtype=np.float64))
            net.backend.save_tensor_data(k, data.reshape(dims, order="F"))
            net.nodes[k] = Node([str(x) for x in v["indices"]], dims, k)
        else:
            net.nodes[k] = Node([str(x) for x in v["indices"]], [int(x) for x in v["dims"]], str(v["data_label"]))
    net.input_qubits = [str(x) for x in d["input_qubits"]]
    net.output_qubits = [str(x) for x in d["output_qubits"]]
    net.qubit_ordering = [int(x) for x in d.get("qubit_ordering", range(1, net.number_qubits + 1))]
    net.node_layers = {str(k): int(v) for k, v in d.get("node_layers", {}).items()}
    net.counters = {"index": index, "node": node, "layer": max([0, *net.node_layers.values()])}
    return net


def decompose_gate(gate_data, threshold=1e-15):
    """src/layer3.jl:715-739: SVD split over positions (1,3) | (2,4)."""
    dims = gate_data.shape
    A = np.transpose(gate_data, (0, 2, 1, 3))
    A = np.reshape(A, (dims[0] * dims[2], dims[1] * dims[3]), order="F")
    U, S, Vh = np.linalg.svd(A)
    chi = int(np.sum(S > threshold))
    s = np.sqrt(S[:chi])
    B = np.reshape(U[:, :chi] * s[None, :], (dims[0], dims[2], chi), order="F")
    C = np.reshape(s[:, None] * Vh[:chi, :], (chi, dims[1], dims[3]), order="F")
    return B, C


def add_gate(net: TensorNetworkCircuit, gate_data, target_qubits, decompose=False):
    """src/layer3.jl:158-249. ``target_qubits`` are 1-based."""
    gate_data = np.asarray(gate_data, dtype=CDT)
    n = len(target_qubits)
    input_indices = [net.output_qubits[q - 1] for q in target_qubits]
    output_indices = [net.new_label("index") for _ in range(n)]
    for i, q in enumerate(target_qubits):
        net.output_qubits[q - 1] = output_indices[i]
    net.counters["layer"] += 1
    layer = net.counters["layer"]

    def rewire(node_label, input_index, output_index, qubit):
        net.edges[output_index] = Edge(node_label, net.edges[input_index].dst, qubit)
        dst = net.edges[input_index].dst
        if dst is not None:
            out_node = net.nodes[dst]
            out_node.indices = [output_index if x == input_index else x for x in out_node.indices]
        net.edges[input_index].dst = node_label

    if decompose and n == 2:
        parts = decompose_gate(gate_data)
        virtual = net.new_label("index")
        labels = [net.new_label("node") for _ in range(2)]
        net.edges[virtual] = Edge(labels[0], labels[1], None, True)
        for i in range(2):
            if i == 0:
                idx = [input_indices[0], output_indices[0], virtual]
            else:
                idx = [virtual, input_indices[1], output_indices[1]]
            net.nodes[labels[i]] = Node(idx, list(parts[i].shape), labels[i])
            net.node_layers[labels[i]] = layer
            net.backend.save_tensor_data(labels[i], parts[i])
            rewire(labels[i], input_indices[i], output_indices[i], target_qubits[i])
        return labels
    label = net.new_label("node")
    net.nodes[label] = Node(input_indices + output_indices, list(gate_data.shape), label)
    net.node_layers[label] = layer
    net.backend.save_tensor_data(label, gate_data)
    for q in range(n):
        rewire(label, input_indices[q], output_indices[q], target_qubits[q])
    return label


_INPUT_MAP = {
    "0": np.array([1.0, 0.0]),
    "1": np.array([0.0, 1.0]),
    "+": np.array([1.0, 1.0]) / math.sqrt(2),
    "-": np.array([1.0, -1.0]) / math.sqrt(2),
}


def add_input(net: TensorNetworkCircuit, config: str):
    """src/layer3.jl:257-284."""
    assert len(config) == net.number_qubits
    for idx, ch in zip(net.input_qubits, config):
        if net.edges[idx].src is None:
            label = net.new_label("node")
            data = _INPUT_MAP[ch]
            net.nodes[label] = Node([idx], [2], label)
            net.node_layers[label] = 0
            net.backend.save_tensor_data(label, data)
            net.edges[idx].src = label


def add_output(net: TensorNetworkCircuit, config: str):
    """src/layer3.jl:292-313 (only '0' and '1'; anything else acts like '1')."""
    assert len(config) == net.number_qubits
    for i in range(net.number_qubits):
        pos = net.qubit_ordering[i]
        idx, ch = net.output_qubits[pos - 1], config[i]
        if net.edges[idx].dst is None:
            label = net.new_label("node")
            data = np.array([1.0, 0.0]) if ch == "0" else np.array([0.0, 1.0])
            net.nodes[label] = Node([idx], [2], label)
            net.node_layers[label] = -1
            net.backend.save_tensor_data(label, data)
            net.edges[idx].dst = label


# --------------------------------------------------------------------------
# L2: contraction (src/layer2.jl)
# --------------------------------------------------------------------------


def sort_indices(A: Node, B: Node):
    """src/layer2.jl:209-216."""
    common = [x for x in A.indices if x in B.indices]
    common = list(dict.fromkeys(common))
    rem_a = [x for x in dict.fromkeys(A.indices) if x not in common]
    rem_b = [x for x in dict.fromkeys(B.indices) if x not in common]
    uncommon = list(dict.fromkeys(rem_a + rem_b))
    return common, uncommon


def create_ncon_indices(A: Node, B: Node, common, uncommon):
    """src/layer2.jl:226-240: common -> +1..k, uncommon -> -1..-m."""
    m = {x: i + 1 for i, x in enumerate(common)}
    m.update({x: -(i + 1) for i, x in enumerate(uncommon)})
    return [m[x] for x in A.indices], [m[x] for x in B.indices]


def contract_pair(net: TensorNetworkCircuit, A_label, B_label=None):
    """src/layer2.jl:346-405 (and the edge overload :329-337 when B is None)."""
    if B_label is None:
        edge = A_label
        if edge in net.edges:
            e = net.edges[edge]
            return contract_pair(net, e.src, e.dst)
        return None
    if A_label == B_label:
        return None
    A, B = net.nodes[A_label], net.nodes[B_label]
    common, rem = sort_indices(A, B)
    ia, ib = create_ncon_indices(A, B, common, rem)
    dmap = dict(zip(A.indices + B.indices, A.dims + B.dims))
    cdims = [dmap[x] for x in common]
    odims = [dmap[x] for x in rem]
    record_compute_costs(net.backend.metrics, odims, cdims)
    C_label = net.new_label("node")
    net.nodes[C_label] = Node(list(rem), list(odims), C_label)
    for x in common:
        del net.edges[x]
    for x in rem:
        e = net.edges[x]
        if e.src in (A_label, B_label):
            e.src = C_label
        elif e.dst in (A_label, B_label):
            e.dst = C_label
    del net.nodes[A_label]
    del net.nodes[B_label]
    net.backend.contract_tensors(A_label, ia, B_label, ib, C_label)
    return C_label


def _layer_groups(net):
    groups: dict[int, list] = {}
    for k, v in net.node_layers.items():
        groups.setdefault(v, []).append(k)
    order = [k for k in sorted(groups) if k > 0]
    if -1 in groups:
        order.append(-1)
    return groups, order


def _final_permute_reshape(net, node_label, output_qubits, output_shape, set_indices):
    node = net.nodes[node_label]
    if len(node.indices) != 0:
        order = [node.indices.index(x) + 1 for x in output_qubits]
        if set_indices:
            node.indices[:] = list(output_qubits)
        net.backend.permute_tensor(node_label, order)
        if output_shape == "vector":
            net.backend.reshape_tensor(node_label, [list(range(1, len(node.indices) + 1))])
        elif output_shape != "":
            net.backend.reshape_tensor(node_label, output_shape)


def full_wavefunction_contraction(net: TensorNetworkCircuit, output_shape=""):
    """src/layer2.jl:132-195."""
    input_nodes = [net.edges[e].src for e in net.input_qubits]
    if any(x is None for x in input_nodes):
        raise ValueError("Please create nodes for each input before using wavefunction contraction")
    wf = input_nodes[0]
    for w in input_nodes[1:]:
        wf = contract_pair(net, wf, w)
    groups, order = _layer_groups(net)
    for layer in order:
        nodes = groups[layer]
        n = nodes[0]
        for n2 in nodes[1:]:
            n = contract_pair(net, n, n2)
        wf = contract_pair(net, wf, n)
    outq = [net.output_qubits[q - 1] for q in net.qubit_ordering]
    _final_permute_reshape(net, wf, outq, output_shape, set_indices=False)
    net.backend.save_output(wf)
    return wf


def contract_network(net: TensorNetworkCircuit, plan, output_shape=""):
    """src/layer2.jl:250-321: pair plan (list of pairs) or edge plan (list of edge labels)."""
    if len(plan) and isinstance(plan[0], (list, tuple)):
        for a, b in plan:
            contract_pair(net, a, b)
    else:
        for e in plan:
            contract_pair(net, e)
        while len(net.nodes) > 1:
            it = iter(net.nodes)
            n1 = next(it)
            n2 = next(it)
            contract_pair(net, n1, n2)
    out = f"node_{net.counters['node']}"
    _final_permute_reshape(net, out, list(net.output_qubits), output_shape, set_indices=True)
    net.backend.save_output(out)
    return out


def random_contraction_plan(net: TensorNetworkCircuit, rng=None):
    """src/layer2.jl:119-122: closed edges in random order."""
    rng = rng or np.random.default_rng()
    closed = [k for k, v in net.edges.items() if v.src is not None and v.dst is not None]
    perm = rng.permutation(len(closed))
    return [closed[i] for i in perm]


# --------------------------------------------------------------------------
# Boltzmann-greedy planner (src/layer2/bgreedy_contraction.jl:17-131)
# --------------------------------------------------------------------------


def _bgreedy_cost(A: Node, B: Node, alpha):
    """bgreedy_contraction.jl:76-94 (Gray & Kourtis heuristic)."""
    common, C_idx = sort_indices(A, B)
    a_open = [A.dims[i] for i in range(len(A.dims)) if A.indices[i] in C_idx]
    b_open = [B.dims[i] for i in range(len(B.dims)) if B.indices[i] in C_idx]
    C_dims = a_open + b_open
    sC = float(np.prod(C_dims)) if C_dims else 1.0
    sA = float(np.prod(A.dims)) if A.dims else 1.0
    sB = float(np.prod(B.dims)) if B.dims else 1.0
    costs = (math.sqrt(sA * sB * sC), sC)
    return sC - alpha * (sA + sB), C_idx, C_dims, costs


def bgreedy(net: TensorNetworkCircuit, alpha=1.0, tau=1.0, N=None, rng=None):
    """bgreedy_contraction.jl:17-66. Returns (plan, time_cost[, space_cost]).

    Sampling uses exp(-energy/tau) normalised with the maximum subtracted
    (same distribution as the reference, without overflow).
    """
    rng = rng or np.random.default_rng()
    if N is not None:
        best, best_cost = [], math.inf
        for _ in range(N):
            plan, tc, _sc = bgreedy(net, alpha, tau, None, rng)
            if tc < best_cost:
                best, best_cost = plan, tc
        return best, best_cost
    tensors = OrderedDict((k, Node(list(v.indices), list(v.dims), v.data_label)) for k, v in net.nodes.items())
    plan = []
    uniq = net.counters["node"]
    time_cost, space_cost = 0.0, 0.0
    while len(tensors) > 1:
        items = list(tensors.items())
        pairs, energy, cinfo = [], [], []
        for i in range(len(items)):
            for j in range(i + 1, len(items)):
                e, ci, cd, costs = _bgreedy_cost(items[i][1], items[j][1], alpha)
                pairs.append((items[i][0], items[j][0]))
                energy.append(e)
                cinfo.append((ci, cd, costs))
        en = -np.asarray(energy) / tau
        w = np.exp(en - en.max())
        k = int(rng.choice(len(pairs), p=w / w.sum()))
        a, b = pairs[k]
        ci, cd, costs = cinfo[k]
        uniq += 1
        del tensors[a]
        del tensors[b]
        tensors[f"node_{uniq}"] = Node(list(ci), list(cd), "intermediate_tensor")
        plan.append([a, b])
        time_cost += costs[0]
        space_cost = max(space_cost, costs[1])
    return plan, time_cost, space_cost


# --------------------------------------------------------------------------
# Slicing (src/layer2/slicing.jl)
# --------------------------------------------------------------------------


def multi_index_partition(dims, number_partitions, partition):
    """slicing.jl:12-26: CartesianIndices(dims[1:k])[partition] (column-major, 1-based)."""
    total, k = 1, 1
    while k < len(dims):
        total *= dims[k - 1]
        if total == number_partitions:
            break
        elif total > number_partitions:
            raise ValueError("Partitions and product of dimensions must match")
        k += 1
    sub = dims[:k]
    lin = partition - 1
    out = []
    for d in sub:
        out.append(lin % d + 1)
        lin //= d
    return tuple(out)


def partition_network_on_virtual_bonds(net, number_partitions, partition):
    """slicing.jl:37-57."""
    vb = [(k, e) for k, e in net.edges.items() if e.virtual]
    assert len(vb) > 0, "There must be some virtual bonds, try turning on decompose"
    dims = []
    for k, e in vb:
        data = net.backend.load_tensor_data(e.src)
        pos = [i for i, x in enumerate(net.nodes[e.src].indices) if x == k]
        dims.append(int(np.prod([data.shape[p] for p in pos])))
    order = np.argsort(np.asarray(dims), kind="stable")
    labels = [vb[i][0] for i in order]
    dims = [dims[i] for i in order]
    ci = multi_index_partition(tuple(dims), number_partitions, partition)
    return labels[: len(ci)], ci


def replace_with_view(net, node_label, bond_label, lo, hi):
    """slicing.jl:67-93 (node dims are left unchanged, as in the reference)."""
    node = net.nodes[node_label]
    bond_idx = node.indices.index(bond_label) + 1
    view = net.new_label("node")
    net.nodes[view] = Node(node.indices, node.dims, view)
    net.node_layers[view] = net.node_layers[node_label]
    for ei in node.indices:
        e = net.edges[ei]
        if e.src == node_label:
            e.src = view
        else:
            e.dst = view
    net.backend.view_tensor(view, node_label, bond_idx, lo, hi)
    net.backend.delete_tensor(node_label)
    del net.nodes[node_label]
    del net.node_layers[node_label]


def slice_tensor_network(net, bond_labels, bond_values):
    """slicing.jl:100-110."""
    for lab, v in zip(bond_labels, bond_values):
        n1, n2 = net.edges[lab].src, net.edges[lab].dst
        replace_with_view(net, n1, lab, v, v)
        replace_with_view(net, n2, lab, v, v)


# --------------------------------------------------------------------------
# Gates and circuits (src/layer3.jl:745-760, src/algorithms.jl:14-89)
# --------------------------------------------------------------------------

GATES = {
    "I": np.array([[1, 0], [0, 1]], dtype=CDT),
    "X": np.array([[0, 1], [1, 0]], dtype=CDT),
    "Y": np.array([[0, -1j], [1j, 0]], dtype=CDT),
    "Z": np.array([[1, 0], [0, -1]], dtype=CDT),
    "H": np.array([[1, 1], [1, -1]], dtype=CDT) / math.sqrt(2),
    "S": np.array([[1, 0], [0, 1j]], dtype=CDT),
    "T": np.array([[1, 0], [0, (1 + 1j) / math.sqrt(2)]], dtype=CDT),
}


def operator_to_tensor(U):
    """Qiskit operator (little-endian matrix) -> gate tensor, src/layer3.jl:566-568.

    ``data = reshape(permutedims(U, (2,1)), 2, ..., 2)`` (column-major), i.e.
    data[i1..in, o1..on] = U[o1 + 2 o2 + ..., i1 + 2 i2 + ...].
    """
    U = np.asarray(U, dtype=CDT)
    k = int(round(math.log2(U.shape[0])))
    return np.reshape(U.T, (2,) * (2 * k), order="F")


def u3(theta, phi, lam):
    """Qiskit U3 matrix."""
    c, s = math.cos(theta / 2), math.sin(theta / 2)
    return np.array(
        [[c, -np.exp(1j * lam) * s], [np.exp(1j * phi) * s, np.exp(1j * (phi + lam)) * c]], dtype=CDT
    )


def cphase(theta):
    return np.diag([1, 1, 1, np.exp(1j * theta)]).astype(CDT)


CX = np.array([[1, 0, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0], [0, 1, 0, 0]], dtype=CDT)  # control = first listed qubit
CZ = np.diag([1, 1, 1, -1]).astype(CDT)
SWAP = np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], dtype=CDT)


def qft_gates(n):
    """src/algorithms.jl:14-32 as a list of (matrix, 1-based qubits).

    h(i-1); cu1(pi/2^(j-i+1), j, i-1) for j=i..n-1; then swap(i-1, n-i).
    """
    gates = []
    for i in range(1, n + 1):
        gates.append((GATES["H"], [i]))
        for j in range(i, n):
            gates.append((cphase(math.pi / 2 ** (j - i + 1)), [j + 1, i]))
    for i in range(1, n // 2 + 1):
        gates.append((SWAP, [i, n - i + 1]))
    return gates


def ghz_gates(n):
    """src/algorithms.jl:79-89."""
    g = [(GATES["H"], [1])]
    for q in range(1, n):
        g.append((CX, [q, q + 1]))
    return g


def simple_preparation_gates(n, depth, rng):
    """src/algorithms.jl:41-72 with numpy randomness (the gate pattern is the same)."""
    g = [(GATES["H"], [q]) for q in range(1, n + 1)]
    for d in range(1, depth + 1):
        params = rng.random((n, 3))
        for q in range(1, n + 1):
            g.append((u3(*params[q - 1]), [q]))
        start = ((d + 1) % 2) + 1
        for q in range(start, n, 2):
            g.append((CX, [q, q + 1]))
    return g


def haar_su2(rng):
    """Haar-random SU(2): QR of a complex Gaussian, phase-fixed, divided by sqrt(det)."""
    z = (rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))) / math.sqrt(2)
    q, r = np.linalg.qr(z)
    d = np.diag(r)
    q = q * (d / np.abs(d))[None, :]
    q = q / np.sqrt(np.linalg.det(q))
    return q.astype(CDT)


def grid_patterns(rows, cols):
    """Four alternating nearest-neighbour CZ edge sets on a rows x cols grid.

    0: horizontal (c, c+1) with c even; 1: horizontal, c odd;
    2: vertical (r, r+1) with r even;   3: vertical, r odd.
    Qubits are numbered 1-based row-major: q = r*cols + c + 1.
    """
    pats = [[], [], [], []]
    for r in range(rows):
        for c in range(cols - 1):
            pats[c % 2].append((r * cols + c + 1, r * cols + c + 2))
    for r in range(rows - 1):
        for c in range(cols):
            pats[2 + r % 2].append((r * cols + c + 1, (r + 1) * cols + c + 1))
    return pats


def random_grid_gates(rows, cols, depth, seed):
    """Synthetic random grid circuit: each layer applies a Haar SU(2) to every
    qubit, then CZ on pattern ``layer mod 4``."""
    rng = np.random.default_rng(seed)
    pats = grid_patterns(rows, cols)
    n = rows * cols
    g = []
    for layer in range(depth):
        for q in range(1, n + 1):
            g.append((haar_su2(rng), [q]))
        for a, b in pats[layer % 4]:
            g.append((CZ, [a, b]))
    return g


def parse_qasm(text):
    """Minimal OPENQASM 2.0 reader for the reference's example circuits
    (qelib1 gates h, x, z, s, t, u1, u2, u3, cx, cz, swap; barriers and
    measurements ignored).  Returns a gate list with 1-based qubits."""
    import re

    one = {"h": lambda: GATES["H"], "x": lambda: GATES["X"], "z": lambda: GATES["Z"],
           "s": lambda: GATES["S"], "t": lambda: GATES["T"]}
    gates = []
    for raw in text.splitlines():
        line = raw.split("//")[0].strip().rstrip(";")
        if not line or line.startswith(("OPENQASM", "include", "qreg", "creg", "barrier", "measure")):
            continue
        m = re.match(r"([a-z0-9]+)\s*(\(([^)]*)\))?\s+(.*)", line)
        name, params, args = m.group(1), m.group(3), m.group(4)
        p = [float(eval(x, {"pi": math.pi})) for x in params.split(",")] if params else []
        qs = [int(x) + 1 for x in re.findall(r"\[(\d+)\]", args)]
        if name in one:
            gates.append((one[name](), qs))
        elif name == "u1":
            gates.append((u3(0.0, 0.0, p[0]), qs))
        elif name == "u2":
            gates.append((u3(math.pi / 2, p[0], p[1]), qs))
        elif name == "u3":
            gates.append((u3(*p), qs))
        elif name == "cx":
            gates.append((CX, qs))
        elif name == "cz":
            gates.append((CZ, qs))
        elif name == "swap":
            gates.append((SWAP, qs))
        else:
            raise ValueError(f"unsupported gate {name}")
    return gates


def build_network(n, gates, decompose=False, backend=None):
    """Equivalent of ``convert_qiskit_circ_to_network`` for a gate list."""
    net = TensorNetworkCircuit(n, backend)
    for U, qs in gates:
        add_gate(net, operator_to_tensor(U), qs, decompose=decompose)
    return net


# --------------------------------------------------------------------------
# Independent state-vector simulator (cross-check for the TN oracle)
# --------------------------------------------------------------------------


def statevector(n, gates, init=None):
    """Little-endian (qubit 1 = least significant bit) state after ``gates``.

    The TN ``full_wavefunction_contraction!(tn, "vector")`` output uses the
    same ordering (first tensor index fastest, column-major).
    """
    if init is None:
        psi = np.zeros(2**n, dtype=CDT)
        psi[0] = 1
    else:
        psi = np.array(init, dtype=CDT)
    # numpy C-order reshape: axis 0 is the most significant bit (qubit n)
    for U, qs in gates:
        k = len(qs)
        t = psi.reshape((2,) * n)
        axes = [n - q for q in qs]  # qubit q -> axis n-q
        # U index = o1 + 2 o2 + ... with qubit qs[0] least significant
        Ut = U.reshape((2,) * (2 * k))  # C-order: (o_k..o_1, i_k..i_1)
        # reorder to (o_1..o_k, i_1..i_k)
        Ut = np.transpose(Ut, list(range(k - 1, -1, -1)) + list(range(2 * k - 1, k - 1, -1)))
        t = np.tensordot(Ut, t, axes=(list(range(k, 2 * k)), axes))
        t = np.moveaxis(t, list(range(k)), axes)
        psi = t.reshape(-1)
    return psi


def execute_ssa_plan(leaves, leaf_labels, steps, out_labels=()):
    """Execute SSA pair steps over numpy leaves with integer labels (the CPU
    equivalent of a compiled plan).  A label is summed once no other live
    tensor and no output carries it (so a label shared by more than two
    tensors is a batch mode until its last use); the result's modes follow
    ``out_labels``.  Each pair is one ``tensordot`` (BLAS zgemm), like
    TensorOperations->BLAS, or one ``einsum`` when it keeps a shared label."""
    vals = [np.asarray(x) for x in leaves]
    labs = [list(l) for l in leaf_labels]
    cnt: dict[int, int] = {}
    for l in labs:
        for x in l:
            cnt[x] = cnt.get(x, 0) + 1
    for x in out_labels:
        cnt[x] = cnt.get(x, 0) + 1
    for i in range(len(steps) // 2):
        a, b = steps[2 * i], steps[2 * i + 1]
        la, lb = labs[a], labs[b]
        for x in la:
            cnt[x] -= 1
        for x in lb:
            cnt[x] -= 1
        common = [x for x in la if x in lb]
        if any(cnt[x] > 0 for x in common):
            # a hyper index (carried by a third live tensor or the output) stays
            # as a batch mode of this pair: one einsum with per-pair letters
            keep = [x for x in dict.fromkeys(la + lb) if cnt[x] > 0]
            letter = {x: chr(ord("a") + k) if k < 26 else chr(ord("A") + k - 26)
                      for k, x in enumerate(dict.fromkeys(la + lb))}
            spec = "".join(letter[x] for x in la) + "," + "".join(letter[x] for x in lb) + "->" + \
                "".join(letter[x] for x in keep)
            C = np.einsum(spec, vals[a], vals[b])
            lc = keep
        else:
            C = np.tensordot(vals[a], vals[b], axes=([la.index(x) for x in common], [lb.index(x) for x in common]))
            lc = [x for x in la if x not in common] + [x for x in lb if x not in common]
        for x in lc:
            cnt[x] += 1
        vals.append(C)
        labs.append(lc)
        vals[a] = vals[b] = None
    res, lr = vals[-1], labs[-1]
    if len(out_labels):
        res = np.transpose(res, [lr.index(x) for x in out_labels])
    return res


def network_leaves(net: TensorNetworkCircuit):
    """The network's current nodes as SSA leaves: (node names in node order,
    arrays, integer labels, label extents, label of each index name).
    Integer labels are numbered by first appearance over the nodes in order,
    so an SSA pair plan over the same network's node order (a compiled
    plan's ``steps``) applies to these leaves unchanged."""
    names = list(net.nodes.keys())
    label_of: dict[str, int] = {}
    dims: list[int] = []
    arrays, labels = [], []
    for nl in names:
        node = net.nodes[nl]
        a = np.asarray(net.backend.load_tensor_data(node.data_label), dtype=CDT)
        if a.ndim != len(node.indices):
            raise ValueError(f"node {nl}: array rank {a.ndim} != {len(node.indices)} indices")
        lab = []
        for idx, d in zip(node.indices, a.shape):
            if idx not in label_of:
                label_of[idx] = len(dims)
                dims.append(int(d))
            elif dims[label_of[idx]] != int(d):
                raise ValueError(f"index {idx} has extents {dims[label_of[idx]]} and {d}")
            lab.append(label_of[idx])
        arrays.append(a)
        labels.append(lab)
    return names, arrays, labels, dims, label_of


def contract_along_steps(net: TensorNetworkCircuit, steps, out_edges=()):
    """Contract the whole network along SSA ``steps`` over its node order
    (the pair-plan execution of src/layer2.jl:294-321, each pair a
    ``tensordot`` as src/layer1.jl:85-92); the result's modes follow
    ``out_edges`` (index names).  Returns the complex128 result array."""
    names, arrays, labels, dims, label_of = network_leaves(net)
    if len(steps) != 2 * (len(names) - 1):
        raise ValueError(f"{len(steps) // 2} steps for {len(names)} leaves")
    return execute_ssa_plan(arrays, labels, list(steps), [label_of[e] for e in out_edges])


def slice_leaves(leaves, leaf_labels, sliced, dims, s):
    """Leaves with the sliced labels fixed to the mixed-radix digits of slice
    ``s`` (first sliced label fastest); the fixed modes are removed."""
    vals = {}
    for x in sliced:
        vals[x] = s % dims[x]
        s //= dims[x]
    out, labs = [], []
    for t, l in zip(leaves, leaf_labels):
        idx = tuple(vals[x] if x in vals else slice(None) for x in l)
        out.append(np.asarray(t)[idx])
        labs.append([x for x in l if x not in vals])
    return out, labs


def random_bitstrings(n_qubits, count, seed):
    """Seeded uniform random output bitstrings (character i = qubit i+1)."""
    rng = np.random.default_rng(seed)
    bits = rng.integers(0, 2, size=(count, n_qubits))
    return ["".join("1" if b else "0" for b in row) for row in bits]


def amplitude_index(bitstring):
    """Index into a little-endian state vector of the output configuration
    ``bitstring`` (character i = qubit i+1)."""
    return sum((1 << i) for i, ch in enumerate(bitstring) if ch == "1")
