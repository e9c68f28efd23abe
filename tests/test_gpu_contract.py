"""Pairwise contraction kernels vs the FP64 oracle (through the C ABI).

Tolerances: complex128 contexts must agree to 1e-12 relative (max-abs error
over max |ref|); complex64 contexts to 2e-6 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {0: 1e-12, 1: 2e-6, "c64all": 2e-6}


def rel_err(a, b):
    a = np.asarray(a).reshape(-1)
    b = np.asarray(b).reshape(-1)
    return float(np.max(np.abs(a - b)) / max(1e-300, float(np.max(np.abs(b)))))


def rand_tensor(rng, dims):
    return rng.standard_normal(dims) + 1j * rng.standard_normal(dims)


def make_case(rng, n_common, n_a, n_b, dim_choices=(1, 2, 3, 4), big=False):
    """Random ncon-style labels: positive shared, negative free, shuffled."""
    dims = {}
    labels = list(range(1, n_common + 1)) + [-(i + 1) for i in range(n_a + n_b)]
    for l in labels:
        dims[l] = int(rng.choice(dim_choices))
    ia = list(range(1, n_common + 1)) + [-(i + 1) for i in range(n_a)]
    ib = list(range(1, n_common + 1)) + [-(n_a + i + 1) for i in range(n_b)]
    rng.shuffle(ia)
    rng.shuffle(ib)
    A = rand_tensor(rng, [dims[l] for l in ia])
    B = rand_tensor(rng, [dims[l] for l in ib])
    return A, ia, B, ib


@pytest.fixture(params=[0, 1, "c64all"], ids=["c128", "c64", "c64all"])
def backend(request, pq):
    if request.param == "c64all":  # every tensor stored as complex64
        be = pq.GB300Backend(precision=1, small_elems=0)
    else:
        be = pq.GB300Backend(precision=request.param)
    yield be
    be.close()


def run_pair(be, A, ia, B, ib):
    be.save_tensor_data("A", A)
    be.save_tensor_data("B", B)
    be.contract_tensors("A", ia, "B", ib, "C")
    return be.load_tensor_data("C")


@pytest.mark.parametrize("seed", range(12))
def test_random_small_pairs(backend, O, seed):
    rng = np.random.default_rng(seed)
    nc, na, nb = rng.integers(0, 4), rng.integers(0, 5), rng.integers(0, 5)
    A, ia, B, ib = make_case(rng, nc, na, nb)
    got = run_pair(backend, A, ia, B, ib)
    ref = O.contract_tensors_arrays(A, ia, B, ib)
    assert np.shape(got) == np.shape(ref) or (np.ndim(ref) == 0)
    assert rel_err(got, ref) < TOL[backend.precision]
    # inputs are consumed
    assert not backend.has_tensor("A") and not backend.has_tensor("B")


def test_gate_application_bond2(backend, O):
    # rank-12 state x 2-qubit gate, contracted modes in the middle of A
    rng = np.random.default_rng(1)
    A = rand_tensor(rng, (2,) * 12)
    G = rand_tensor(rng, (2, 2, 2, 2))
    ia = [-1, -2, -3, 1, -4, -5, 2, -6, -7, -8, -9, -10]
    ib = [1, 2, -11, -12]
    got = run_pair(backend, A, ia, G, ib)
    ref = O.contract_tensors_arrays(A, ia, G, ib)
    assert got.shape == ref.shape == (2,) * 12
    assert rel_err(got, ref) < TOL[backend.precision]


def test_gemm_class_permuted(backend, O):
    # large M, N, K with interleaved modes -> tiled GEMM kernel
    rng = np.random.default_rng(2)
    ia = [-1, 1, -2, 2, -3, 3, -4, 4, -5, -6, 5, -7, 6, -8]
    ib = [3, -9, 1, -10, 5, 2, -11, 6, 4, -12, -13, -14, -15, -16]
    A = rand_tensor(rng, [2] * len(ia))
    B = rand_tensor(rng, [2] * len(ib))
    got = run_pair(backend, A, ia, B, ib)
    ref = O.contract_tensors_arrays(A, ia, B, ib)
    assert rel_err(got, ref) < TOL[backend.precision] * 4


def test_large_k_generic_chunked(backend, O):
    # K = 4096 > table size with a small result
    rng = np.random.default_rng(3)
    ia = [-1] + list(range(1, 13))
    ib = list(range(12, 0, -1)) + [-2]
    A = rand_tensor(rng, [3] + [2] * 12)
    B = rand_tensor(rng, [2] * 12 + [3])
    got = run_pair(backend, A, ia, B, ib)
    ref = O.contract_tensors_arrays(A, ia, B, ib)
    assert rel_err(got, ref) < TOL[backend.precision] * 8


def test_non_power_of_two_dims(backend, O):
    rng = np.random.default_rng(4)
    A, ia, B, ib = make_case(rng, 2, 3, 3, dim_choices=(3, 5, 6, 7))
    got = run_pair(backend, A, ia, B, ib)
    assert rel_err(got, O.contract_tensors_arrays(A, ia, B, ib)) < TOL[backend.precision]


def test_full_contraction_to_scalar_and_outer_product(backend, O):
    rng = np.random.default_rng(5)
    A = rand_tensor(rng, (2, 3, 4))
    B = rand_tensor(rng, (4, 2, 3))
    got = run_pair(backend, A, [1, 2, 3], B, [3, 1, 2])
    ref = O.contract_tensors_arrays(A, [1, 2, 3], B, [3, 1, 2])
    assert rel_err(got, ref) < TOL[backend.precision]
    got = run_pair(backend, A, [-1, -2, -3], B, [-4, -5, -6])
    ref = O.contract_tensors_arrays(A, [-1, -2, -3], B, [-4, -5, -6])
    assert got.shape == (2, 3, 4, 4, 2, 3)
    assert rel_err(got, ref) < TOL[backend.precision]


def test_errors_are_reported(backend, pq):
    from pqgb300 import _lib as L

    with pytest.raises(L.PQError) as e:
        backend.contract_tensors("nope", [1], "nada", [1], "C")
    assert e.value.code == L.PQ_ERR_NOT_FOUND
    backend.save_tensor_data("x", np.ones((2, 3)))
    backend.save_tensor_data("y", np.ones((4, 3)))
    with pytest.raises(L.PQError) as e:
        backend.contract_tensors("x", [1, -1], "y", [1, -2], "z")  # extent 2 vs 4
    assert e.value.code == L.PQ_ERR_INVALID
    with pytest.raises(L.PQError) as e:
        backend.contract_tensors("x", [1], "y", [1, -2], "z")  # wrong label count
    assert e.value.code == L.PQ_ERR_INVALID
    assert backend.load_tensor_data("missing") is None
    # memory cap: fault injection on the host
    backend.set_mem_cap(backend.mem_in_use() + 1024)
    with pytest.raises(L.PQError) as e:
        backend.save_tensor_data("big", np.ones((64, 64)))
    assert e.value.code == L.PQ_ERR_OOM
    backend.set_mem_cap(0)
    backend.save_tensor_data("big", np.ones((64, 64)))
    backend.sync()


def test_backend_ops(backend, O):
    rng = np.random.default_rng(6)
    T = rand_tensor(rng, (2, 3, 4, 5))
    backend.save_tensor_data("t", T)
    backend.permute_tensor("t", [3, 1, 4, 2])
    assert rel_err(backend.load_tensor_data("t"), O.permute_array(T, [3, 1, 4, 2])) < TOL[backend.precision]
    backend.reshape_tensor("t", [[1, 2], [3, 4]])
    ref = O.reshape_array(O.permute_array(T, [3, 1, 4, 2]), [8, 15])
    got = backend.load_tensor_data("t")
    assert got.shape == (8, 15) and rel_err(got, ref) < TOL[backend.precision]
    backend.save_tensor_data("u", T)
    backend.view_tensor("v", "u", 3, (2, 3))
    assert rel_err(backend.load_tensor_data("v"), O.tensor_view_array(T, 3, 2, 3)) < TOL[backend.precision]
    backend.view_tensor("w", "u", 1, range(2, 3))
    assert backend.load_tensor_data("w").shape == (1, 3, 4, 5)
    backend.save_output("u", "result")
    assert rel_err(backend.load_tensor_data("result"), T) < TOL[backend.precision]
    idx = np.array([0, 7, 119], dtype=np.int64)
    assert rel_err(backend.gather("u", idx), T.reshape(-1, order="F")[idx]) < TOL[backend.precision]
    backend.delete_tensor("u")
    assert backend.load_tensor_data("u") is None
