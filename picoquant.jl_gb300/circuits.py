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
