"""Gate tensors and the synthetic circuit workloads.

Gate tensor layout follows the reference's qiskit import
(src/layer3.jl:566-568): for a k-qubit operator U in qiskit's little-endian
convention, data[i1..ik, o1..ok] = U[o1 + 2 o2 + ..., i1 + 2 i2 + ...].
"""
from __future__ import annotations

import math

import numpy as np

from .network import TensorNetworkCircuit, add_gate

H = np.array([[1, 1], [1, -1]], dtype=np.complex128) / math.sqrt(2)
X = np.array([[0, 1], [1, 0]], dtype=np.complex128)
Z = np.array([[1, 0], [0, -1]], dtype=np.complex128)
CZ = np.diag([1, 1, 1, -1]).astype(np.complex128)
CX = np.array([[1, 0, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0], [0, 1, 0, 0]], dtype=np.complex128)
SWAP = np.array([[1, 0, 0, 0], [0, 0, 1, 0], [0, 1, 0, 0], [0, 0, 0, 1]], dtype=np.complex128)


def cphase(theta):
    return np.diag([1, 1, 1, np.exp(1j * theta)]).astype(np.complex128)


def operator_to_tensor(U):
    """Little-endian operator matrix -> gate tensor (column-major reshape of U^T)."""
    U = np.asarray(U, dtype=np.complex128)
    k = int(round(math.log2(U.shape[0])))
    return np.reshape(U.T, (2,) * (2 * k), order="F")


def qft_gates(n):
    """src/algorithms.jl:14-32: H on qubit i, controlled phases pi/2^(j-i+1)
    between qubits j and i-1 (0-based), then swaps reversing qubit order."""
    g = []
    for i in range(1, n + 1):
        g.append((H, [i]))
        for j in range(i, n):
            g.append((cphase(math.pi / 2 ** (j - i + 1)), [j + 1, i]))
    for i in range(1, n // 2 + 1):
        g.append((SWAP, [i, n - i + 1]))
    return g


def ghz_gates(n):
    """src/algorithms.jl:79-89."""
    return [(H, [1])] + [(CX, [q, q + 1]) for q in range(1, n)]


def haar_su2(rng):
    """Haar-random SU(2): QR of a complex Gaussian with the phase of R's
    diagonal removed, scaled by 1/sqrt(det)."""
    z = (rng.standard_normal((2, 2)) + 1j * rng.standard_normal((2, 2))) / math.sqrt(2)
    q, r = np.linalg.qr(z)
    d = np.diag(r)
    q = q * (d / np.abs(d))[None, :]
    return (q / np.sqrt(np.linalg.det(q))).astype(np.complex128)


def grid_patterns(rows, cols):
    """Four alternating nearest-neighbour edge sets: horizontal from even
    columns, horizontal from odd columns, vertical from even rows, vertical
    from odd rows (qubits 1-based, row-major)."""
    pats = [[], [], [], []]
    for r in range(rows):
        for c in range(cols - 1):
            pats[c % 2].append((r * cols + c + 1, r * cols + c + 2))
    for r in range(rows - 1):
        for c in range(cols):
            pats[2 + r % 2].append((r * cols + c + 1, (r + 1) * cols + c + 1))
    return pats


def random_grid_gates(rows, cols, depth, seed):
    """Random grid circuit: per layer a seeded Haar SU(2) on every qubit, then
    CZ on edge pattern ``layer mod 4``."""
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


def fuse_single_qubit_gates(gates):
    """The same circuit with every run of single-qubit gates folded into the
    next two-qubit gate on that qubit (operator convention of
    ``operator_to_tensor``: the first listed qubit is the low bit, so
    U_a (x) U_b is kron(U_b, U_a)); single-qubit gates with no later two-qubit
    gate are emitted at the end.  Exact; a state-vector order then sweeps the
    state once per remaining gate."""
    pending: dict[int, np.ndarray] = {}
    out = []
    for U, qs in gates:
        U = np.asarray(U, dtype=np.complex128)
        if len(qs) == 1:
            q = qs[0]
            pending[q] = U @ pending[q] if q in pending else U
        elif len(qs) == 2:
            a, b = qs
            pa = pending.pop(a, np.eye(2, dtype=np.complex128))
            pb = pending.pop(b, np.eye(2, dtype=np.complex128))
            out.append((U @ np.kron(pb, pa), [a, b]))
        else:
            for q in qs:
                if q in pending:
                    out.append((pending.pop(q), [q]))
            out.append((U, list(qs)))
    for q in sorted(pending):
        out.append((pending[q], [q]))
    return out


def _apply_on(B, U, qs, block):
    """U (on ``qs``, the first listed qubit the low bit) times the operator B
    on ``block`` (first qubit the low bit): B's row bits are the tensor axes
    of a C-order reshape, axis a holding bit m - 1 - a."""
    m, k = len(block), len(qs)
    T = B.reshape((2,) * m + (B.shape[1],))
    Ut = np.asarray(U, dtype=np.complex128).reshape((2,) * (2 * k))
    tgt = [m - 1 - block.index(qs[j]) for j in reversed(range(k))]
    R = np.tensordot(Ut, T, axes=(list(range(k, 2 * k)), tgt))
    return np.moveaxis(R, list(range(k)), tgt).reshape(B.shape)


def fuse_gates(gates, max_qubits=4):
    """The same circuit as blocks of at most ``max_qubits`` qubits (operator
    convention of ``operator_to_tensor``), so that a state-vector order sweeps
    the state once per block.  Greedy in circuit order: a gate joins the block
    that is the latest on each of its qubits when that block has room; when
    its qubits' latest blocks differ, those blocks are merged with it if each
    is still the latest on all of its own qubits (so it can move past every
    block in between, which acts on other qubits) and the union fits; else
    the gate starts a block (a gate wider than ``max_qubits`` is a block of
    its own).  Exact: only commuting blocks are reordered."""
    blocks = []   # [qubits (first = low bit), matrix, alive]
    last = {}     # qubit -> index of its latest block
    for U, qs in gates:
        qs = list(qs)
        U = np.asarray(U, dtype=np.complex128)
        owners = sorted({last[q] for q in qs if q in last})
        target = None
        if len(owners) == 1:
            b = owners[0]
            if len(set(blocks[b][0]) | set(qs)) <= max_qubits:
                target = b
        elif len(owners) > 1:
            union = set(qs)
            for b in owners:
                union |= set(blocks[b][0])
            if len(union) <= max_qubits and all(last[q] == b for b in owners for q in blocks[b][0]):
                qubits, M = [], np.ones((1, 1), dtype=np.complex128)
                for b in owners:  # disjoint blocks: the later one's bits above
                    qubits += blocks[b][0]
                    M = np.kron(blocks[b][1], M)
                    blocks[b][2] = False
                blocks.append([qubits, M, True])
                target = len(blocks) - 1
                for q in qubits:
                    last[q] = target
        if target is None:
            blocks.append([list(qs), U.copy(), True])
            target = len(blocks) - 1
        else:
            blk = blocks[target]
            for q in qs:
                if q not in blk[0]:
                    blk[0].append(q)  # a new highest bit
                    blk[1] = np.kron(np.eye(2, dtype=np.complex128), blk[1])
            blk[1] = _apply_on(blk[1], U, qs, blk[0])
        for q in qs:
            last[q] = target
    return [(M, qubits) for qubits, M, alive in blocks if alive]


def grid_shape(n_qubits):
    """Most square rows x cols factorisation of a qubit count (rows <= cols)."""
    best = (1, n_qubits)
    for r in range(1, int(math.isqrt(n_qubits)) + 1):
        if n_qubits % r == 0:
            best = (r, n_qubits // r)
    return best


def random_bitstrings(n_qubits, count, seed):
    rng = np.random.default_rng(seed)
    bits = rng.integers(0, 2, size=(count, n_qubits))
    return ["".join("1" if b else "0" for b in row) for row in bits]


def build_network(n_qubits, gates, decompose=False, backend=None):
    """Tensor network of a gate list (the role of
    ``convert_qiskit_circ_to_network``, src/layer3.jl:544-573)."""
    net = TensorNetworkCircuit(n_qubits, backend)
    for U, qs in gates:
        add_gate(net, operator_to_tensor(U), qs, decompose=decompose)
    return net
