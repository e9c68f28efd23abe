"""Layer 2: contraction orchestration (PicoQuant's contract_pair! & co.).

Same order of operations, index classification, ncon labels and metrics as
src/layer2.jl:119-405; every pairwise contraction goes to the backend's
``contract_tensors`` (one GB300 kernel launch per pair).  For repeated or
large contractions use ``planning.NetworkPlan``, which compiles the whole pair
plan once and runs it from an arena / CUDA graph.
"""
from __future__ import annotations

import numpy as np

from .backend import record_compute_costs
from .network import Node, new_label, permute_tensor, reshape_tensor, save_output


def sort_indices(A: Node, B: Node):
    """src/layer2.jl:209-216: (common, uncommon) index lists."""
    common = list(dict.fromkeys(x for x in A.indices if x in B.indices))
    rem_a = [x for x in dict.fromkeys(A.indices) if x not in common]
    rem_b = [x for x in dict.fromkeys(B.indices) if x not in common]
    return common, list(dict.fromkeys(rem_a + rem_b))


def create_ncon_indices(A: Node, B: Node, common, uncommon):
    """src/layer2.jl:226-240: common -> +1..k, uncommon -> -1..-m."""
    m = {x: i + 1 for i, x in enumerate(common)}
    m.update({x: -(i + 1) for i, x in enumerate(uncommon)})
    return [m[x] for x in A.indices], [m[x] for x in B.indices]


def contract_pair(network, A_label, B_label=None):
    """src/layer2.jl:346-405; with one argument, the edge overload (:329-337)."""
    if B_label is None:
        e = network.edges.get(A_label)
        if e is None:
            return None
        return contract_pair(network, e.src, e.dst)
    if A_label == B_label:
        return None
    A, B = network.nodes[A_label], network.nodes[B_label]
    common, remaining = sort_indices(A, B)
    ia, ib = create_ncon_indices(A, B, common, remaining)
    dims = dict(zip(A.indices + B.indices, A.dims + B.dims))
    cdims = [dims[x] for x in common]
    odims = [dims[x] for x in remaining]
    record_compute_costs(network.backend, odims, cdims)
    C_label = new_label(network, "node")
    network.nodes[C_label] = Node(list(remaining), odims, C_label)
    for x in common:
        del network.edges[x]
    for x in remaining:
        e = network.edges[x]
        if e.src in (A_label, B_label):
            e.src = C_label
        elif e.dst in (A_label, B_label):
            e.dst = C_label
    del network.nodes[A_label]
    del network.nodes[B_label]
    network.backend.contract_tensors(A_label, ia, B_label, ib, C_label)
    return C_label


def layer_order(network):
    """Nodes grouped by layer, gate layers ascending then the output layer
    (src/layer2.jl:149-161)."""
    groups: dict[int, list] = {}
    for k, v in network.node_layers.items():
        groups.setdefault(v, []).append(k)
    order = [k for k in sorted(groups) if k > 0]
    if -1 in groups:
        order.append(-1)
    return groups, order


def _finish(network, node_label, output_indices, output_shape, relabel):
    node = network.nodes[node_label]
    if len(node.indices) != 0:
        order = [node.indices.index(x) + 1 for x in output_indices]
        if relabel:
            node.indices[:] = list(output_indices)
        permute_tensor(network, node_label, order)
        if output_shape == "vector":
            reshape_tensor(network, node_label, [list(range(1, len(node.indices) + 1))])
        elif output_shape != "":
            reshape_tensor(network, node_label, output_shape)


def full_wavefunction_contraction(network, output_shape=""):
    """src/layer2.jl:132-195."""
    input_nodes = [network.edges[e].src for e in network.input_qubits]
    if any(x is None for x in input_nodes):
        raise ValueError("Please create nodes for each input before using wavefunction contraction")
    wf = input_nodes[0]
    for w in input_nodes[1:]:
        wf = contract_pair(network, wf, w)
    groups, order = layer_order(network)
    for layer in order:
        nodes = groups[layer]
        n = nodes[0]
        for n2 in nodes[1:]:
            n = contract_pair(network, n, n2)
        wf = contract_pair(network, wf, n)
    outq = [network.output_qubits[q - 1] for q in network.qubit_ordering]
    _finish(network, wf, outq, output_shape, relabel=False)
    save_output(network, wf)
    return wf


def contract_network(network, plan, output_shape=""):
    """src/layer2.jl:250-321: a pair plan ([[A, B], ...]) or an edge plan ([edge, ...])."""
    if len(plan) and isinstance(plan[0], (list, tuple)):
        for A, B in plan:
            contract_pair(network, A, B)
    else:
        for e in plan:
            contract_pair(network, e)
        while len(network.nodes) > 1:
            it = iter(network.nodes)
            n1, n2 = next(it), next(it)
            contract_pair(network, n1, n2)
    out = f"node_{network.counters['node']}"
    _finish(network, out, list(network.output_qubits), output_shape, relabel=True)
    save_output(network, out)
    return out


def random_contraction_plan(network, rng=None):
    """src/layer2.jl:119-122: the closed edges in random order."""
    rng = rng if rng is not None else np.random.default_rng()
    closed = [k for k, v in network.edges.items() if v.src is not None and v.dst is not None]
    return [closed[i] for i in rng.permutation(len(closed))]


# ---- slicing (src/layer2/slicing.jl) -------------------------------------------

def multi_index_partition(dims, number_partitions, partition):
    """src/layer2/slicing.jl:12-26: the 1-based CartesianIndex of ``partition``
    over the leading dims whose product equals ``number_partitions``."""
    total, k = 1, 1
    while k < len(dims):
        total *= dims[k - 1]
        if total == number_partitions:
            break
        if total > number_partitions:
            raise ValueError("Partitions and product of dimensions must match")
        k += 1
    lin = partition - 1
    out = []
    for d in dims[:k]:
        out.append(lin % d + 1)
        lin //= d
    return tuple(out)


def partition_network_on_virtual_bonds(network, number_partitions, partition):
    """src/layer2/slicing.jl:37-57."""
    vb = [(k, e) for k, e in network.edges.items() if e.virtual]
    if not vb:
        raise AssertionError("There must be some virtual bonds, try turning on decompose")
    dims = []
    for k, e in vb:
        shp = network.backend.shape(e.src) if hasattr(network.backend, "shape") else \
            network.backend.load_tensor_data(e.src).shape
        pos = [i for i, x in enumerate(network.nodes[e.src].indices) if x == k]
        dims.append(int(np.prod([shp[p] for p in pos])))
    order = np.argsort(np.asarray(dims), kind="stable")
    labels = [vb[i][0] for i in order]
    dims = [dims[i] for i in order]
    ci = multi_index_partition(tuple(dims), number_partitions, partition)
    return labels[: len(ci)], ci


def replace_with_view(network, node_label, bond_label, bond_range):
    """src/layer2/slicing.jl:67-93 (the node keeps its dims, as in the reference)."""
    node = network.nodes[node_label]
    bond_idx = node.indices.index(bond_label) + 1
    view = new_label(network, "node")
    network.nodes[view] = Node(node.indices, node.dims, view)
    network.node_layers[view] = network.node_layers[node_label]
    for ei in node.indices:
        e = network.edges[ei]
        if e.src == node_label:
            e.src = view
        else:
            e.dst = view
    network.backend.view_tensor(view, node_label, bond_idx, bond_range)
    network.backend.delete_tensor(node_label)
    del network.nodes[node_label]
    del network.node_layers[node_label]


def slice_tensor_network(network, bond_labels, bond_values):
    """src/layer2/slicing.jl:100-110."""
    for lab, v in zip(bond_labels, bond_values):
        n1, n2 = network.edges[lab].src, network.edges[lab].dst
        replace_with_view(network, n1, lab, (v, v))
        replace_with_view(network, n2, lab, (v, v))
