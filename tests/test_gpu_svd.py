"""The device SVD split (pq_decompose_tensor) against LAPACK's, after the
reference's decompose tests (test/layer1_tests.jl, the `decompose_tensor!`
cases; truncation rule src/layer1.jl:166-176).

Singular vectors are unique only up to a phase (and a rotation inside a
degenerate subspace), so the factors are compared through what is unique:
the bond extent chi, the singular values (the squared column norms of the
left factor B = U sqrt(S)) and the truncated product B C.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rand(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def _low_rank(rng, shape, left, rank):
    """A tensor whose (left | rest) matricisation has the given rank."""
    ld = [shape[i - 1] for i in left]
    rest = [i for i in range(1, len(shape) + 1) if i not in left]
    rd = [shape[i - 1] for i in rest]
    m, n = int(np.prod(ld)), int(np.prod(rd))
    A = _rand(rng, (m, rank)) @ _rand(rng, (rank, n))
    T = A.reshape(tuple(ld) + tuple(rd), order="F")
    order = list(left) + rest
    return np.transpose(T, np.argsort([o - 1 for o in order]))


def _split(pq, be, T, left, right, threshold=1e-13, max_rank=0):
    be.save_tensor_data("t", T)
    chi = be.decompose_tensor("t", left, right, threshold=threshold, max_rank=max_rank,
                              left_label="b", right_label="c")
    assert not be.has_tensor("t")
    return chi, np.asarray(be.load_tensor_data("b")), np.asarray(be.load_tensor_data("c"))


def _check(pq, T, left, right, B, Cm, chi, tol, threshold=1e-13, max_rank=0, eps_dtype=np.float64):
    rB, rC, rchi = pq.decompose_array(T, left, right, threshold, max_rank, eps_dtype=eps_dtype)
    assert chi == rchi
    ld = [T.shape[i - 1] for i in left]
    rd = [T.shape[i - 1] for i in right]
    assert B.shape == tuple(ld) + (chi,) and Cm.shape == (chi,) + tuple(rd)
    m, n = int(np.prod(ld)), int(np.prod(rd))
    Bm, Cmm = B.reshape(m, chi, order="F"), Cm.reshape(chi, n, order="F")
    rBm, rCm = rB.reshape(m, chi, order="F"), rC.reshape(chi, n, order="F")
    scale = np.linalg.norm(T)
    # singular values: ||B_j||^2 = sigma_j, in decreasing order
    sig, rsig = np.sum(np.abs(Bm) ** 2, axis=0), np.sum(np.abs(rBm) ** 2, axis=0)
    assert np.max(np.abs(sig - rsig), initial=0.0) <= tol * scale
    assert np.all(np.diff(sig) <= tol * scale)
    # the truncated product
    assert np.max(np.abs(Bm @ Cmm - rBm @ rCm), initial=0.0) <= tol * scale
    # B's columns are orthogonal, C's rows too
    G = Bm.conj().T @ Bm
    assert np.max(np.abs(G - np.diag(np.diag(G))), initial=0.0) <= tol * scale
    H = Cmm @ Cmm.conj().T
    assert np.max(np.abs(H - np.diag(np.diag(H))), initial=0.0) <= tol * scale


CASES = [
    # (shape, left positions, right positions)
    ((4, 4, 4, 4), [1, 2], [3, 4]),     # square 16 x 16
    ((2, 8, 8), [2, 3], [1]),            # 64 x 2: tall, chi <= 2
    ((2, 8, 8), [1], [3, 2]),            # 2 x 64: wide (the conjugate-transpose side)
    ((3, 5, 7), [3, 1], [2]),            # 21 x 5, odd column count
    ((5, 3, 7, 2), [2], [4, 1, 3]),      # 3 x 70
    ((16, 16, 4, 2), [1, 3], [2, 4]),    # 64 x 32
    ((2, 128, 2, 2), [2, 4], [1, 3]),    # 256 x 4
    ((7,), [1], []),                     # a vector: 7 x 1
]


# complex128 contexts decompose in FP64; the others in FP32, as LAPACK does
# for the reference's ComplexF32 backend.  FP32 Jacobi keeps the singular
# values to a few 1e-6 of the largest (rounding of the rotations over ~10
# sweeps), hence the wider bound there.
PRECS = [("c128", 1e-12, np.float64), ("c64", 2e-5, np.float32)]


@pytest.mark.parametrize("prec,tol,eps_dtype", PRECS)
@pytest.mark.parametrize("shape,left,right", CASES)
def test_device_svd_random_matches_lapack(pq, shape, left, right, prec, tol, eps_dtype):
    rng = np.random.default_rng(len(shape) * 100 + sum(shape))
    T = _rand(rng, shape)
    be = pq.GB300Backend(pq.PREC_C128 if prec == "c128" else pq.PREC_C64, svd="device")
    chi, B, Cm = _split(pq, be, T, left, right)
    _check(pq, T, left, right, B, Cm, chi, tol, eps_dtype=eps_dtype)
    be.close()


def test_device_svd_truncates_like_the_reference(pq):
    """Rank-deficient splits keep exactly the numerical rank; max_rank caps
    it; a relative threshold drops the small singular values."""
    rng = np.random.default_rng(11)
    be = pq.GB300Backend(pq.PREC_C128, svd="device")
    for shape, left, right, rank in (((4, 4, 4, 4), [1, 3], [2, 4], 3),
                                     ((2, 64, 4), [2], [1, 3], 5),
                                     ((2, 64, 4), [1, 3], [2], 1)):
        T = _low_rank(rng, shape, left, rank)
        chi, B, Cm = _split(pq, be, T, left, right)
        assert chi == rank
        _check(pq, T, left, right, B, Cm, chi, 1e-12)
    T = _rand(rng, (8, 8, 8))
    chi, B, Cm = _split(pq, be, T, [1], [2, 3], max_rank=3)
    assert chi == 3
    _check(pq, T, [1], [2, 3], B, Cm, chi, 1e-12, max_rank=3)
    # graded singular values 1, 1e-1, ..., 1e-7: threshold 1e-4 keeps four
    U, _ = np.linalg.qr(_rand(rng, (16, 8)))
    V, _ = np.linalg.qr(_rand(rng, (8, 8)))
    A = (U * 10.0 ** -np.arange(8)) @ V.conj().T
    T = A.reshape(4, 4, 8, order="F")
    chi, B, Cm = _split(pq, be, T, [1, 2], [3], threshold=1e-4)
    assert chi == 4
    _check(pq, T, [1, 2], [3], B, Cm, chi, 1e-12, threshold=1e-4)
    # an all-zero tensor has no singular value above the threshold: chi = 0
    chi, B, Cm = _split(pq, be, np.zeros((4, 2, 8), dtype=np.complex128), [1, 2], [3])
    assert chi == 0 and B.shape == (4, 2, 0) and Cm.shape == (0, 8)
    be.close()


def test_device_svd_complex64_context(pq):
    """In a complex64 context the threshold floor is sqrt(eps(Float32)), as
    for the reference's ComplexF32 backend; the input and factors above the
    small-tensor size are stored as complex64."""
    rng = np.random.default_rng(5)
    be = pq.GB300Backend(pq.PREC_C64, svd="device", small_elems=64)
    T = _rand(rng, (16, 16, 16))
    chi, B, Cm = _split(pq, be, T, [1, 3], [2])
    _check(pq, T, [1, 3], [2], B, Cm, chi, 2e-5, eps_dtype=np.float32)
    be.close()


def test_device_svd_rejects_bad_splits(pq):
    from pqgb300 import _lib as L

    rng = np.random.default_rng(1)
    be = pq.GB300Backend(pq.PREC_C128, svd="device")
    be.save_tensor_data("t", _rand(rng, (4, 4, 4)))
    with pytest.raises(pq.PQError) as e:
        be.decompose_tensor("t", [1, 1], [3], left_label="b", right_label="c")
    assert e.value.code == L.PQ_ERR_INVALID
    with pytest.raises(pq.PQError) as e:
        be.decompose_tensor("t", [1], [2], left_label="b", right_label="c")
    assert e.value.code == L.PQ_ERR_INVALID
    assert be.has_tensor("t")  # a refused split leaves the input alone
    be.save_tensor_data("w", _rand(rng, (512, 512)))
    with pytest.raises(pq.PQError) as e:
        be.decompose_tensor("w", [1], [2], left_label="b", right_label="c")
    assert e.value.code == L.PQ_ERR_UNSUPPORTED
    be.close()


def test_mps_with_device_svd(pq, O):
    """The compressed path with every bond split on the device gives the
    circuit's state (oracle state vector)."""
    n = 5
    rng = np.random.default_rng(21)
    gates = [(pq.haar_su2(rng), [q]) for q in range(1, n + 1)]
    gates += [(pq.CX, [q, q + 1]) for q in range(1, n)]
    gates += [(pq.haar_su2(rng), [q]) for q in range(1, n + 1)]
    gates += [(pq.CZ, [q, q + 1]) for q in range(2, n, 2)]
    for prec, tol in ((pq.PREC_C128, 1e-12), (pq.PREC_C64, 2e-5)):
        be = pq.GB300Backend(prec, svd="device")
        tn = pq.build_network(n, gates, backend=be, decompose=True)
        pq.add_input(tn, "0" * n)
        mps = pq.contract_mps_tensor_network_circuit(tn)
        pq.calculate_mps_amplitudes(tn, mps)
        wf = np.asarray(pq.load_tensor_data(tn, "result")).reshape(-1)
        assert np.max(np.abs(wf - O.statevector(n, gates))) < tol
        be.close()
