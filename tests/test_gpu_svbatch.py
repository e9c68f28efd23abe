"""Grouped state vectors of many circuits (pq_svbatch_*) against the FP64
oracle's state-vector simulator of the original, unfused gates.

Tolerance: complex64 states with FP32 block products, 2e-6 of the largest
amplitude magnitude of each circuit's state.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _circuits(pq, specs, n_bits=16):
    from pqgb300 import circuits as CI

    out, raw = [], []
    for i, (n, d) in enumerate(specs):
        r, c = CI.grid_shape(n)
        gates = pq.random_grid_gates(r, c, d, seed=500 + i)
        bits = pq.random_bitstrings(n, n_bits, seed=900 + i)
        out.append((n, CI.fuse_gates(gates, 4), bits))
        raw.append((n, r, c, d, 500 + i, bits))
    return out, raw


SPECS = [(6, 5), (9, 7), (12, 9), (14, 6), (10, 12), (7, 3), (13, 8)]


def _reference(O, raw):
    refs = []
    for n, r, c, d, seed, bits in raw:
        sv = O.statevector(n, O.random_grid_gates(r, c, d, seed=seed))
        refs.append((sv[[O.amplitude_index(b) for b in bits]], np.max(np.abs(sv))))
    return refs


def test_svbatch_matches_oracle(pq, O):
    from pqgb300.svbatch import StateVectorBatch

    circs, raw = _circuits(pq, SPECS)
    refs = _reference(O, raw)
    be = pq.GB300Backend(pq.PREC_C64)
    sb = StateVectorBatch(be, circs)
    info = sb.info()
    assert info["chunks"] == 1
    # one launch per block index of the deepest circuit, plus init and gather
    assert info["kernel_launches"] == 2 + max(len(b) for _, b, _ in circs)
    for _ in range(2):  # the first execution records the graph, the second replays it
        got = sb.execute()
        for g, (ref, scale) in zip(got, refs):
            assert np.max(np.abs(g - ref)) <= 2e-6 * scale
    sb.close()
    be.close()


def test_svbatch_chunks_give_the_same_amplitudes(pq, O):
    """A budget of one 2^14-amplitude state splits the batch: the 14-qubit
    circuit alone, then every smaller one (2^13 + 2^12 + ... fits); the
    amplitudes are bit-identical to one chunk's."""
    from pqgb300.svbatch import StateVectorBatch

    circs, raw = _circuits(pq, SPECS)
    be = pq.GB300Backend(pq.PREC_C64)
    one = StateVectorBatch(be, circs).execute()
    sb = StateVectorBatch(be, circs, state_budget_bytes=8 << 14)
    assert sb.info()["chunks"] == 2
    many = sb.execute()
    for a, b in zip(one, many):
        assert np.array_equal(a, b)
    sb.close()
    be.close()


def test_svbatch_rejects_bad_input(pq):
    from pqgb300 import _lib as L
    from pqgb300.svbatch import StateVectorBatch

    be = pq.GB300Backend(pq.PREC_C64)
    H = np.array([[1, 1], [1, -1]]) / np.sqrt(2)
    with pytest.raises(L.PQError):
        StateVectorBatch(be, [(3, [(H, [4])], ["000"])])  # qubit 4 of a 3-qubit circuit
    with pytest.raises(L.PQError):
        StateVectorBatch(be, [(3, [(np.eye(32), [1, 2, 3, 4, 5])], ["000"])])  # five-qubit block
    with pytest.raises(ValueError):
        StateVectorBatch(be, [(3, [(np.eye(4), [1])], ["000"])])  # matrix of the wrong size
    sb = StateVectorBatch(be, [(3, [(H, [2])], ["000", "010"])])
    got = sb.execute()[0]
    assert np.allclose(got, [1 / np.sqrt(2), 1 / np.sqrt(2)], atol=1e-7)
    sb.close()
    be.close()
