"""Layer 3: the tensor network of a circuit (PicoQuant's TensorNetworkCircuit).

Same graph semantics as the reference (src/layer3.jl:22-455): gates are nodes,
qubit wires are edges named ``index_<k>``, nodes are named ``node_<k>``, a
gate node's indices are ``[in_1..in_n, out_1..out_n]``, inputs are rank-1
nodes at layer 0 and outputs rank-1 nodes at layer -1.  Tensor data goes to
the backend (GB300Backend by default) through ``save_tensor_data``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Node:
    """src/layer3.jl:23-30."""

    indices: list
    dims: list
    data_label: str


@dataclass
class Edge:
    """src/layer3.jl:43-53."""

    src: str | None = None
    dst: str | None = None
    qubit: int | None = None
    virtual: bool = False


class TensorNetworkCircuit:
    """src/layer3.jl:56-118."""

    def __init__(self, qubits: int, backend=None):
        if backend is None:
            from .backend import GB300Backend

            backend = GB300Backend()
        self.backend = backend
        self.number_qubits = qubits
        labels = [f"index_{i}" for i in range(1, qubits + 1)]
        self.edges: dict[str, Edge] = {lab: Edge(None, None, i + 1, False) for i, lab in enumerate(labels)}
        self.input_qubits = list(labels)
        self.output_qubits = list(labels)
        self.nodes: dict[str, Node] = {}
        self.qubit_ordering = list(range(1, qubits + 1))
        self.counters = {"index": qubits, "node": 0, "layer": 0}
        self.node_layers: dict[str, int] = {}


def new_label(network: TensorNetworkCircuit, label_str: str) -> str:
    """src/layer3.jl:145-148."""
    network.counters[label_str] += 1
    return f"{label_str}_{network.counters[label_str]}"


# ---- forwarding to the backend (src/layer3.jl:124-134) ---------------------

def save_tensor_data(network, label, data):
    return network.backend.save_tensor_data(label, data)


def load_tensor_data(network, label):
    return network.backend.load_tensor_data(label)


def contract_tensors(network, A, ia, B, ib, C):
    return network.backend.contract_tensors(A, ia, B, ib, C)


def save_output(network, node, name="result"):
    return network.backend.save_output(node, name)


def reshape_tensor(network, tensor, groups):
    return network.backend.reshape_tensor(tensor, groups)


def permute_tensor(network, tensor, axes):
    return network.backend.permute_tensor(tensor, axes)


def delete_tensor(network, tensor):
    return network.backend.delete_tensor(tensor)


def view_tensor(network, view_node, node, bond_idx, bond_range):
    return network.backend.view_tensor(view_node, node, bond_idx, bond_range)


# ---- mutation ----------------------------------------------------------------

def decompose_gate(gate_data, threshold=1e-15):
    """src/layer3.jl:715-739: split a 2-qubit gate across (1,3)|(2,4) by SVD,
    keeping singular values above the absolute threshold."""
    d = gate_data.shape
    A = np.reshape(np.transpose(gate_data, (0, 2, 1, 3)), (d[0] * d[2], d[1] * d[3]), order="F")
    U, S, Vh = np.linalg.svd(A)
    chi = int(np.sum(S > threshold))
    s = np.sqrt(S[:chi])
    B = np.reshape(U[:, :chi] * s[None, :], (d[0], d[2], chi), order="F")
    Cm = np.reshape(s[:, None] * Vh[:chi, :], (chi, d[1], d[3]), order="F")
    return B, Cm


def _plumb(network, node_label, input_index, output_index, qubit):
    network.edges[output_index] = Edge(node_label, network.edges[input_index].dst, qubit)
    dst = network.edges[input_index].dst
    if dst is not None:
        out_node = network.nodes[dst]
        out_node.indices[:] = [output_index if x == input_index else x for x in out_node.indices]
    network.edges[input_index].dst = node_label


def add_gate(network: TensorNetworkCircuit, gate_data, target_qubits, decompose: bool = False):
    """src/layer3.jl:158-249 (``target_qubits`` 1-based)."""
    gate_data = np.asarray(gate_data, dtype=np.complex128)
    n = len(target_qubits)
    input_indices = [network.output_qubits[q - 1] for q in target_qubits]
    output_indices = [new_label(network, "index") for _ in range(n)]
    for i, q in enumerate(target_qubits):
        network.output_qubits[q - 1] = output_indices[i]
    network.counters["layer"] += 1
    layer = network.counters["layer"]
    if decompose and n == 2:
        parts = decompose_gate(gate_data)
        virtual_index = new_label(network, "index")
        labels = [new_label(network, "node") for _ in range(2)]
        network.edges[virtual_index] = Edge(labels[0], labels[1], None, True)
        for i in range(2):
            if i == 0:
                idx = [input_indices[0], output_indices[0], virtual_index]
            else:
                idx = [virtual_index, input_indices[1], output_indices[1]]
            network.nodes[labels[i]] = Node(idx, list(parts[i].shape), labels[i])
            network.node_layers[labels[i]] = layer
            save_tensor_data(network, labels[i], parts[i])
            _plumb(network, labels[i], input_indices[i], output_indices[i], target_qubits[i])
        return labels
    label = new_label(network, "node")
    network.nodes[label] = Node(input_indices + output_indices, list(gate_data.shape), label)
    network.node_layers[label] = layer
    save_tensor_data(network, label, gate_data)
    for q in range(n):
        _plumb(network, label, input_indices[q], output_indices[q], target_qubits[q])
    return label


_INPUTS = {
    "0": (1.0, 0.0),
    "1": (0.0, 1.0),
    "+": (1 / math.sqrt(2), 1 / math.sqrt(2)),
    "-": (1 / math.sqrt(2), -1 / math.sqrt(2)),
}


def add_input(network: TensorNetworkCircuit, config: str):
    """src/layer3.jl:257-284."""
    if len(config) != network.number_qubits:
        raise AssertionError("input configuration length must equal the number of qubits")
    for index, ch in zip(network.input_qubits, config):
        if network.edges[index].src is None:
            label = new_label(network, "node")
            network.nodes[label] = Node([index], [2], label)
            network.node_layers[label] = 0
            save_tensor_data(network, label, np.array(_INPUTS[ch], dtype=np.complex128))
            network.edges[index].src = label


def add_output(network: TensorNetworkCircuit, config: str):
    """src/layer3.jl:292-313 ('0' -> [1,0], anything else -> [0,1])."""
    if len(config) != network.number_qubits:
        raise AssertionError("output configuration length must equal the number of qubits")
    for i in range(network.number_qubits):
        pos = network.qubit_ordering[i]
        index, ch = network.output_qubits[pos - 1], config[i]
        if network.edges[index].dst is None:
            label = new_label(network, "node")
            data = np.array([1.0, 0.0] if ch == "0" else [0.0, 1.0], dtype=np.complex128)
            network.nodes[label] = Node([index], [2], label)
            network.node_layers[label] = -1
            save_tensor_data(network, label, data)
            network.edges[index].dst = label


# ---- accessors (src/layer3.jl:324-455) ----------------------------------------

def edges(network):
    return network.edges


def getnode(network, label):
    return network.nodes[label]


def getedge(network, label):
    return network.edges[label]


def inneighbours(network, node_label):
    out = []
    for index in network.nodes[node_label].indices:
        e = network.edges[index]
        if e.src is not None and e.src != node_label and not e.virtual:
            out.append(e.src)
    return out


def outneighbours(network, node_label):
    out = []
    for index in network.nodes[node_label].indices:
        e = network.edges[index]
        if e.dst is not None and e.dst != node_label and not e.virtual:
            out.append(e.dst)
    return out


def virtualneighbours(network, node_label):
    out = []
    for index in network.nodes[node_label].indices:
        e = network.edges[index]
        if e.dst is not None and e.dst != node_label and e.virtual:
            out.append(e.dst)
        elif e.src is not None and e.src != node_label and e.virtual:
            out.append(e.src)
    return out


def neighbours(network, node_label):
    return inneighbours(network, node_label) + outneighbours(network, node_label) + virtualneighbours(
        network, node_label)


def inedges(network, node_label):
    return [x for x in network.nodes[node_label].indices
            if not network.edges[x].virtual and network.edges[x].dst == node_label]


def outedges(network, node_label):
    return [x for x in network.nodes[node_label].indices
            if not network.edges[x].virtual and network.edges[x].src == node_label]


def virtualedges(network, node_label):
    return [x for x in network.nodes[node_label].indices if network.edges[x].virtual]


# ---- serialisation (src/layer3.jl:579-707) ----------------------------------
# Same keys and value formats as the reference, so a network description moves
# between the two implementations: edges {src, dst, virtual, qubit}; nodes
# {indices, dims (as strings), data_label}; the tensor data stay in the backend.

def edge_to_dict(edge: Edge) -> dict:
    """src/layer3.jl:584-587."""
    return {"src": edge.src, "dst": edge.dst, "virtual": edge.virtual, "qubit": edge.qubit}


def edge_from_dict(d) -> Edge:
    """src/layer3.jl:594-599 (``qubit`` / ``virtual`` optional, as in the
    older example files that carry only src/dst)."""
    return Edge(d["src"], d["dst"], d.get("qubit"), bool(d.get("virtual", False)))


def node_to_dict(node: Node) -> dict:
    """src/layer3.jl:606-611."""
    return {"indices": [str(x) for x in node.indices], "dims": [str(int(x)) for x in node.dims],
            "data_label": str(node.data_label)}


def node_from_dict(d) -> Node:
    """src/layer3.jl:618-623."""
    return Node([str(x) for x in d["indices"]], [int(x) for x in d["dims"]], str(d["data_label"]))


def to_dict(network: TensorNetworkCircuit, with_data: bool = False) -> dict:
    """src/layer3.jl:630-647 (key order kept).  ``with_data`` also embeds each
    node's tensor as the reference's example networks do (``data_re``,
    ``data_im`` flattened column-major, ``data_dims``), read back from the
    backend, so the file carries everything needed to contract it
    elsewhere."""
    nodes = {}
    for k, v in network.nodes.items():
        nd = node_to_dict(v)
        if with_data:
            a = np.asarray(network.backend.load_tensor_data(v.data_label), dtype=np.complex128)
            flat = a.reshape(-1, order="F")
            nd.update({"data_re": flat.real.tolist(), "data_im": flat.imag.tolist(),
                       "data_dims": [int(x) for x in a.shape]})
        nodes[str(k)] = nd
    return {
        "number_qubits": network.number_qubits,
        "edges": {str(k): edge_to_dict(v) for k, v in network.edges.items()},
        "nodes": nodes,
        "input_qubits": [str(x) for x in network.input_qubits],
        "output_qubits": [str(x) for x in network.output_qubits],
        "qubit_ordering": [int(x) for x in network.qubit_ordering],
        "node_layers": {str(k): int(v) for k, v in network.node_layers.items()},
    }


def network_from_dict(d, backend=None) -> TensorNetworkCircuit:
    """src/layer3.jl:654-681: the graph of ``d`` on ``backend``; the label
    counters continue after the largest node and index numbers present.
    Nodes that embed their tensor (``data_re``, ``data_im``, ``data_dims``,
    as written by ``to_dict(..., with_data=True)`` and as in the reference's
    example networks, examples/ghz_3.json) are uploaded to the backend under
    the node's name; the others refer by ``data_label`` to tensors the
    backend already holds.  Files without ``qubit_ordering`` /
    ``node_layers`` get the identity ordering and no layers."""
    net = TensorNetworkCircuit(int(d["number_qubits"]), backend)
    net.edges = {}
    index = 0
    for k, v in d["edges"].items():
        index = max(index, int(k.split("_")[-1]))
        net.edges[k] = edge_from_dict(v)
    net.nodes = {}
    node = 0
    for k, v in d["nodes"].items():
        node = max(node, int(k.split("_")[-1]))
        if "data_re" in v:
            dims = [int(x) for x in v["data_dims"]]
            data = np.asarray(v["data_re"], dtype=np.float64) + 1j * np.asarray(v["data_im"], dtype=np.float64)
            net.nodes[k] = Node([str(x) for x in v["indices"]], dims, k)
            save_tensor_data(net, k, data.reshape(dims, order="F"))
        else:
            net.nodes[k] = node_from_dict(v)
    net.input_qubits = [str(x) for x in d["input_qubits"]]
    net.output_qubits = [str(x) for x in d["output_qubits"]]
    net.qubit_ordering = [int(x) for x in d.get("qubit_ordering", range(1, net.number_qubits + 1))]
    net.node_layers = {str(k): int(v) for k, v in d.get("node_layers", {}).items()}
    net.counters = {"index": index, "node": node, "layer": max([0, *net.node_layers.values()])}
    return net


def to_json(network: TensorNetworkCircuit, indent: int = 0, with_data: bool = False) -> str:
    """src/layer3.jl:688-695 (``with_data`` as in ``to_dict``)."""
    import json

    return json.dumps(to_dict(network, with_data), indent=indent if indent else None)


def network_from_json(json_str: str, backend=None) -> TensorNetworkCircuit:
    """src/layer3.jl:702-705."""
    import json

    return network_from_dict(json.loads(json_str), backend)
