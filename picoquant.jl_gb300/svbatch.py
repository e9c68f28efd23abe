"""Many circuits' amplitudes from grouped state-vector passes.

For workloads of many small-to-medium circuits each asked for a few dozen
amplitudes, the circuits are given as blocks of at most four qubits
(``circuits.fuse_gates``) and run by ``pq_svbatch_*``: every circuit's state
(complex64) is one arena slice, launch s applies the s-th block of every
circuit of a chunk (circuits packed into chunks by size under a byte budget),
and the whole batch -- initialisation, every block launch and the gather of
the requested amplitudes -- is one CUDA graph replayed on each execution.
The reference contracts each circuit separately (src/layer2.jl:294-321, one
``contract_pair!`` per gate); the amplitudes are those of the full state in
the reference's little-endian order (qubit 1 = least significant bit,
src/layer2.jl:180-189).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


def bitstring_index(bits: str) -> int:
    """Amplitude index of an output bitstring (character i = qubit i+1)."""
    return sum(1 << i for i, ch in enumerate(bits) if ch == "1")


class StateVectorBatch:
    """``circuits``: a list of (n_qubits, blocks, bitstrings) with blocks
    [(U, qubits)] -- U the 2^k x 2^k operator (out, in) of qubits (1-based,
    the first listed the least significant bit of U's index), k <= 4 -- and
    the output bitstrings whose amplitudes are wanted.  ``state_budget_bytes``
    bounds the states resident at once (chunks run one after another)."""

    def __init__(self, backend, circuits, state_budget_bytes=64 << 30):
        self.be = backend
        self.lib = L.lib()
        nq, nb, nk, qbits, mats, na, idx = [], [], [], [], [], [], []
        for n, blocks, bitstrings in circuits:
            nq.append(int(n))
            nb.append(len(blocks))
            for U, qs in blocks:
                U = np.asarray(U, dtype=np.complex128)
                k = len(qs)
                if U.shape != (1 << k, 1 << k):
                    raise ValueError(f"block on {k} qubits has a {U.shape} matrix")
                nk.append(k)
                qbits += [int(q) - 1 for q in qs]
                m = U.reshape(-1, order="F")
                mats.append(np.stack([m.real, m.imag], axis=1).reshape(-1))
            na.append(len(bitstrings))
            idx += [bitstring_index(b) for b in bitstrings]
        self.n_amps = na
        # bytes one execution moves at least: every block pass reads and
        # writes its circuit's whole complex64 state once
        self.algorithmic_bytes = sum(16 * (1 << int(n)) * len(blocks) for n, blocks, _ in circuits)
        mats = np.concatenate(mats) if mats else np.zeros(2)
        a32 = lambda v: np.ascontiguousarray(v if len(v) else [0], dtype=np.int32)
        arrs = [a32(nq), a32(nb), a32(nk), a32(qbits)]
        mats = np.ascontiguousarray(mats, dtype=np.float64)
        na_a = a32(na)
        idx_a = np.ascontiguousarray(idx if idx else [0], dtype=np.int64)
        h = C.c_void_p()
        rc = self.lib.pq_svbatch_create(backend.ctx, len(circuits), *(x.ctypes.data_as(L.i32p) for x in arrs),
                                        mats.ctypes.data_as(L.f64p), na_a.ctypes.data_as(L.i32p),
                                        idx_a.ctypes.data_as(L.i64p), int(state_budget_bytes), C.byref(h))
        L.check(rc, backend.ctx, "pq_svbatch_create")
        self.h = h

    def info(self):
        la, ch, ar = C.c_int64(), C.c_int64(), C.c_int64()
        L.check(self.lib.pq_svbatch_info(self.h, C.byref(la), C.byref(ch), C.byref(ar)), self.be.ctx, "svbatch_info")
        return {"kernel_launches": la.value, "chunks": ch.value, "arena_bytes": ar.value}

    def execute(self):
        """Run the batch; returns one complex128 array of amplitudes per
        circuit, in the order given."""
        tot = sum(self.n_amps)
        out = np.empty(2 * max(1, tot), dtype=np.float64)
        L.check(self.lib.pq_svbatch_execute(self.h, out.ctypes.data_as(L.f64p)), self.be.ctx, "svbatch_execute")
        amps = out[0:2 * tot:2] + 1j * out[1:2 * tot:2]
        res, p = [], 0
        for n in self.n_amps:
            res.append(amps[p:p + n])
            p += n
        return res

    def close(self):
        if getattr(self, "h", None):
            self.lib.pq_svbatch_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass
