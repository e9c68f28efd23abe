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


def merge_common_bonds(network, a_label, b_label):
    """src/layer2.jl:25-71: when two nodes share more than one index, move
    the shared indices last in both tensors (``permute_tensor``) and merge
    them into one new virtual index (``reshape_tensor``, column-major, no
    data move beyond the permutation), replacing the shared edges by one.
    Both tensors order their shared indices as ``a`` holds them (the
    reference orders each by its own index order, which pairs the wrong
    elements when the two orders differ; where they agree the result is the
    same)."""
    from .network import Edge

    a, b = network.nodes[a_label], network.nodes[b_label]
    common = [x for x in a.indices if x in b.indices]
    if len(common) <= 1:
        return
    a_common = [k for k, x in enumerate(a.indices) if x in b.indices]
    a_rest = [k for k, x in enumerate(a.indices) if x not in b.indices]
    b_common = [b.indices.index(x) for x in common]
    b_rest = [k for k, x in enumerate(b.indices) if x not in a.indices]
    permute_tensor(network, a_label, [k + 1 for k in a_rest + a_common])
    permute_tensor(network, b_label, [k + 1 for k in b_rest + b_common])
    new_edge = new_label(network, "index")
    dim = int(np.prod([a.dims[k] for k in a_common]))
    dims_a = dict(zip(a.indices, a.dims))
    dims_b = dict(zip(b.indices, b.dims))
    idx_a = [a.indices[k] for k in a_rest] + [new_edge]
    idx_b = [b.indices[k] for k in b_rest] + [new_edge]
    network.nodes[a_label] = Node(idx_a, [dims_a[x] for x in idx_a[:-1]] + [dim], a_label)
    network.nodes[b_label] = Node(idx_b, [dims_b[x] for x in idx_b[:-1]] + [dim], b_label)
    for lab, rest, com in ((a_label, a_rest, a_common), (b_label, b_rest, b_common)):
        l, m = len(rest), len(com)
        reshape_tensor(network, lab, [[k] for k in range(1, l + 1)] + [list(range(l + 1, l + m + 1))])
    network.edges[new_edge] = Edge(a_label, b_label, None, True)
    for e in common:
        del network.edges[e]


def inorder_contraction(network):
    """src/layer2.jl:78-112: contract the network layer by layer from the
    inputs: every node of a gate layer (then of the output layer) absorbs its
    distinct in-neighbours, then each pair of the layer's new nodes (``y >
    x`` by name, x varying fastest) has its shared bonds merged."""
    from .network import inneighbours

    groups: dict[int, list] = {}
    for k, v in network.node_layers.items():
        groups.setdefault(v, []).append(k)
    layers = [k for k in sorted(groups) if k > 0]
    if -1 in groups:
        layers.append(-1)
    for layer in layers:
        new_nodes = []
        for node in groups[layer]:
            for in_node in list(dict.fromkeys(inneighbours(network, node))):
                node = contract_pair(network, in_node, node)
            new_nodes.append(node)
        for y in new_nodes:
            for x in new_nodes:
                if y > x:
                    merge_common_bonds(network, x, y)


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
