"""The FP64 fidelity check on the device (pq_tensor_norm2) against numpy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", [(1,), (3, 5), (2,) * 10, (1 << 20,), (700, 1300)])
@pytest.mark.parametrize("prec", ["c128", "c64"])
def test_norm2_matches_numpy(pq, shape, prec):
    """Squared norms of random tensors: one element, ragged sizes, more
    blocks than the first pass launches (grid-stride), complex128 and
    complex64 storage (compared with the stored values)."""
    rng = np.random.default_rng(sum(shape))
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    be = pq.GB300Backend(pq.PREC_C128 if prec == "c128" else pq.PREC_C64, small_elems=0 if prec == "c64" else None)
    be.save_tensor_data("t", a)
    stored = np.asarray(be.load_tensor_data("t")).astype(np.complex128)
    ref = float(np.sum(stored.real ** 2 + stored.imag ** 2, dtype=np.float64))
    got = be.norm2("t")
    assert abs(got - ref) <= 1e-14 * ref
    assert got == be.norm2("t")  # deterministic
    be.close()


def test_norm2_of_qft10_state_is_one(pq):
    """QFT-10 on |0...0> (config 1) is a unit vector: the device FP64 norm
    is 1 to rounding."""
    be = pq.GB300Backend(pq.PREC_C128)
    tn = pq.build_network(10, pq.qft_gates(10), backend=be)
    pq.add_input(tn, "0" * 10)
    pq.full_wavefunction_contraction(tn, "vector")
    assert abs(be.norm2("result") - 1.0) < 1e-13
    be.close()


def test_norm2_missing_tensor(pq):
    from pqgb300 import _lib as L

    be = pq.GB300Backend(pq.PREC_C64)
    with pytest.raises(pq.PQError) as e:
        be.norm2("nothing")
    assert e.value.code == L.PQ_ERR_NOT_FOUND
    be.close()
