"""The compressed (MPS) contraction path: bond compression by SVD and the
MPS amplitudes (src/layer2.jl:452-700, src/mps.jl:1-110).

Same order of operations as the reference: gate nodes are absorbed into the
per-qubit MPS tensors layer by layer (``contract_pair``, one device kernel per
pair), then the bonds between neighbouring updated tensors are compressed by
a contraction followed by an SVD split with a relative threshold and a
maximum rank.  The SVD itself runs in the backend's ``decompose_tensor``:
for the GB300 backend LAPACK on the host (the default) or the library's
one-sided Jacobi SVD on the device (``GB300Backend(svd="device")``).
"""
from __future__ import annotations

import numpy as np

from .contraction import contract_pair, create_ncon_indices, sort_indices
from .network import Edge, Node, inneighbours, new_label, permute_tensor, reshape_tensor, save_output


def decompose_tensor(network, node_label, left_indices, right_indices, threshold=1e-13, max_rank=0,
                     left_label=None, right_label=None):
    """src/layer2.jl:487-560: split a node into two joined by a new virtual
    edge (the backend's SVD); returns (left_label, right_label)."""
    node = network.nodes[node_label]
    pos = {v: k + 1 for k, v in enumerate(node.indices)}
    left_positions = [pos[x] for x in left_indices]
    right_positions = [pos[x] for x in right_indices]
    B_label = left_label if left_label is not None else new_label(network, "node")
    C_label = right_label if right_label is not None else new_label(network, "node")
    chi = network.backend.decompose_tensor(node_label, left_positions, right_positions, threshold=threshold,
                                           max_rank=max_rank, left_label=B_label, right_label=C_label)
    B_dims = [node.dims[i - 1] for i in left_positions]
    C_dims = [node.dims[i - 1] for i in right_positions]
    if chi > 0:
        vdim = chi
    else:  # a backend that learns the extent only later (the DSL backend)
        vdim = min(int(np.prod(B_dims)), int(np.prod(C_dims)))
        if max_rank > 0:
            vdim = min(vdim, max_rank)
    index_label = new_label(network, "index")
    network.nodes[B_label] = Node(list(left_indices) + [index_label], B_dims + [vdim], B_label)
    network.nodes[C_label] = Node([index_label] + list(right_indices), [vdim] + C_dims, C_label)
    for index, new in [(x, B_label) for x in left_indices] + [(x, C_label) for x in right_indices]:
        e = network.edges[index]
        if e.src == node_label:
            e.src = new
        elif e.dst == node_label:
            e.dst = new
    network.edges[index_label] = Edge(B_label, C_label, None, True)
    if node_label not in (B_label, C_label):
        del network.nodes[node_label]
    return B_label, C_label


def compress_bond(network, node_1, node_2, threshold=1e-13, max_rank=0):
    """src/layer2.jl:452-474: contract two neighbours and split them again."""
    left = network.nodes[node_1]
    right = network.nodes[node_2]
    left_indices = [x for x in left.indices if x not in right.indices]
    right_indices = [x for x in right.indices if x not in left.indices]
    combined = contract_pair(network, node_1, node_2)
    return decompose_tensor(network, combined, left_indices, right_indices, threshold=threshold,
                            max_rank=max_rank, left_label=node_1, right_label=node_2)


def compress_tensor_chain(network, nodes, threshold=1e-13, max_rank=0):
    """src/layer2.jl:423-450: compress the bonds of a chain of tensors with a
    forward then a backward sweep of ``compress_bond`` over consecutive
    pairs (singular values below ``threshold`` and beyond ``max_rank``,
    0 = unbounded, are dropped).  The chain's tensors must be joined only
    to their neighbours by virtual bonds."""
    for i in range(len(nodes) - 1):
        compress_bond(network, nodes[i], nodes[i + 1], threshold=threshold, max_rank=max_rank)
    for i in range(len(nodes) - 2, -1, -1):
        compress_bond(network, nodes[i], nodes[i + 1], threshold=threshold, max_rank=max_rank)


def _gate_layers(network):
    layers: dict[int, list] = {}
    for k, v in network.node_layers.items():
        if k in network.nodes:
            layers.setdefault(v, []).append(k)
    order = [k for k in sorted(layers) if k > 0]
    if -1 in layers:
        order.append(-1)
    return layers, order


def contract_mps_tensor_network_circuit(network, max_bond=2, threshold=1e-13, max_rank=0, pbc=False):
    """src/layer2.jl:572-628: absorb every gate layer into the MPS tensors
    (one per input qubit), compressing the bonds between neighbouring updated
    tensors; saves each final MPS tensor under its own name and returns the
    MPS node labels in qubit order."""
    mps_nodes = [network.edges[x].src for x in network.input_qubits]
    if any(x is None for x in mps_nodes):
        raise AssertionError("Input qubit values must be set")
    layers, order = _gate_layers(network)
    for layer in order:
        updated = []
        for node in layers[layer]:
            inp = inneighbours(network, node)[0]
            if inp not in mps_nodes:
                raise AssertionError(f"{inp} not in mps nodes")
            idx = mps_nodes.index(inp)
            mps_nodes[idx] = contract_pair(network, inp, node)
            updated.append(idx)
        updated.sort()
        for a, b in zip(updated, updated[1:]):
            dist = b - a
            if pbc:
                dist = min(dist, a + len(mps_nodes) - b)
            if dist != 1:
                raise AssertionError("Gates between non-neighboring qubits")
            compress_bond(network, mps_nodes[a], mps_nodes[b], threshold=threshold, max_rank=max_rank)
    for node in mps_nodes:
        save_output(network, node, str(node))
    return mps_nodes


def contract_tensor_network_circuit_with_compression(network, max_bond=2, threshold=1e-13, max_rank=0):
    """src/layer2.jl:656-700: as the MPS contraction, compressing every pair of
    consecutively updated tensors whether or not they are neighbours."""
    nodes = [network.edges[x].src for x in network.input_qubits]
    if any(x is None for x in nodes):
        raise AssertionError("Input qubit values must be set")
    layers, order = _gate_layers(network)
    for layer in order:
        updated = []
        for node in layers[layer]:
            inp = inneighbours(network, node)[0]
            idx = nodes.index(inp)
            nodes[idx] = contract_pair(network, inp, node)
            updated.append(idx)
        for a, b in zip(updated, updated[1:]):
            compress_bond(network, nodes[a], nodes[b], threshold=threshold, max_rank=max_rank)
    for node in nodes:
        save_output(network, node, str(node))
    return nodes


def calculate_mps_amplitudes(network, mps_nodes, result="result"):
    """src/layer2.jl:636-645: contract the MPS tensors into the full state
    vector in qubit order."""
    out = mps_nodes[0]
    for node in mps_nodes[1:]:
        out = contract_pair(network, out, node)
    permute_tensor(network, out, network.qubit_ordering)
    reshape_tensor(network, out, [list(range(1, len(mps_nodes) + 1))])
    save_output(network, out, result)
    return out


class MPSState:
    """src/mps.jl:9-110: amplitudes read from an MPS without forming the
    state.  Each qubit's tensor is copied once, in the backend, with its
    output index moved first (the reference keeps the same per-qubit data on
    the host); an amplitude takes each copy's slab for the requested bit
    (``view_tensor``) and contracts the slabs along the chain with the
    backend's ``contract_tensors`` (on the device for the GB300 backend), in
    the reference's order and with its ncon labels."""

    _next_uid = 0

    def __init__(self, network, mps_nodes):
        n = len(mps_nodes)
        self.n = n
        self.backend = network.backend
        MPSState._next_uid += 1
        self._tag = f"__mpsstate{MPSState._next_uid}"
        self.nodes, self.site = [], []
        outs = set(network.output_qubits)
        positions = []
        be = self.backend
        for i, nl in enumerate(mps_nodes):
            node = network.nodes[nl]
            p = next(k for k, x in enumerate(node.indices) if x in outs)
            positions.append(p)
            other = [k for k in range(len(node.indices)) if k != p]
            lab = f"{self._tag}_site{i + 1}"
            # copy (a view over the whole first mode), then the output index first
            be.view_tensor(lab, node.data_label, 1, range(1, node.dims[0] + 1))
            be.permute_tensor(lab, [p + 1] + [k + 1 for k in other])
            self.site.append(lab)
            self.nodes.append(Node([node.indices[k] for k in other], [node.dims[k] for k in other], f"n_{i + 1}"))
        self.ordering = [0] * n
        for i, e in zip(range(n), network.qubit_ordering):
            self.ordering[e - 1] = i

    def size(self):
        return tuple([2] * self.n)

    def __len__(self):
        return 2 ** self.n

    def _slab(self, i, bit):
        """Site i's slab for output value ``bit`` as a tensor over its other
        indices: a width-1 view of the output mode, that unit mode then
        merged into its neighbour (a reshape, no data move)."""
        lab = f"{self._tag}_slab{i + 1}"
        self.backend.view_tensor(lab, self.site[i], 1, range(bit + 1, bit + 2))
        r = len(self.nodes[i].indices)
        groups = [[1, 2]] + [[k] for k in range(3, r + 2)] if r else [[1]]
        self.backend.reshape_tensor(lab, groups)
        return lab

    def __getitem__(self, conf):
        """``state["0110"]`` (character i is the output of qubit
        ``qubit_ordering[i]``) or ``state[(1, 2, 2, 1)]`` (1-based values as
        in the reference's array interface)."""
        if isinstance(conf, str):
            bits = [1 if ch == "1" else 0 for ch in conf]
        else:
            bits = [(int(x) - 1) for x in conf]
        be = self.backend
        n1 = self.nodes[0]
        cur = self._slab(0, bits[self.ordering[0]])
        for idx in range(1, self.n):
            n2 = self.nodes[idx]
            common, remaining = sort_indices(n1, n2)
            ia, ib = create_ncon_indices(n1, n2, common, remaining)
            nxt = self._slab(idx, bits[self.ordering[idx]])
            out = f"{self._tag}_chain{idx}"
            be.contract_tensors(cur, ia, nxt, ib, out)  # consumes both slabs
            cur = out
            n1 = Node(list(remaining), [1] * len(remaining), "n1")
        v = be.load_tensor_data(cur)
        be.delete_tensor(cur)
        return complex(np.asarray(v).reshape(-1)[0])

    def close(self):
        """Release the per-qubit copies held in the backend."""
        for lab in self.site:
            self.backend.delete_tensor(lab)
        self.site = []
