"""Split-precision tensor-core class (tcgen05, 3xTF32) vs the FP64 oracle.

GEMM-shaped pairs in PREC_3XTF32 contexts (M, N >= 64, K >= 16) run on the
tcgen05 kernels; tolerance 1e-5 relative to the largest result magnitude
(3xTF32 products with FP32 accumulation over K <= 1024).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


def rel_err(a, b):
    a = np.asarray(a).reshape(-1)
    b = np.asarray(b).reshape(-1)
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def rand(rng, dims):
    return rng.standard_normal(dims) + 1j * rng.standard_normal(dims)


@pytest.fixture(params=[(2, None), (2, 0), (4, None)], ids=["3xtf32-mixed", "3xtf32-c64all", "6xtf32-mixed"])
def be(request, pq):
    prec, small = request.param
    b = pq.GB300Backend(prec, small_elems=small)
    yield b
    b.close()


def run(be, A, ia, B, ib):
    be.save_tensor_data("A", A)
    be.save_tensor_data("B", B)
    n0 = be.launch_count()
    be.contract_tensors("A", ia, "B", ib, "C")
    launched = be.launch_count() - n0
    return be.load_tensor_data("C"), launched


def test_plain_matrix_product(be, O):
    rng = np.random.default_rng(0)
    A = rand(rng, (256, 64))
    B = rand(rng, (64, 128))
    got, nl = run(be, A, [-1, 1], B, [1, -2])
    assert nl == 3  # pack A, pack B, tcgen05 GEMM
    assert rel_err(got, A @ B) < TOL


@pytest.mark.parametrize("m,n,k", [(400, 72, 40), (128, 128, 64), (130, 260, 48), (1000, 96, 272)])
def test_ragged_tiles(be, O, m, n, k):
    rng = np.random.default_rng(m + n + k)
    A = rand(rng, (k, m))
    B = rand(rng, (n, k))
    got, nl = run(be, A, [1, -1], B, [-2, 1])
    assert nl == 3
    assert rel_err(got, A.T @ B.T) < TOL


def test_permuted_bond2_modes(be, O):
    # interleaved free / contracted bond-2 modes in both operands
    rng = np.random.default_rng(3)
    ia = [-1, 1, -2, 2, -3, 3, -4, 4, -5, -6, 5, -7, 6, -8]
    ib = [3, -9, 1, -10, 5, 2, -11, 6, 4, -12, -13, -14, -15, -16]
    A = rand(rng, [2] * len(ia))
    B = rand(rng, [2] * len(ib))
    got, nl = run(be, A, ia, B, ib)
    assert nl == 3
    assert rel_err(got, O.contract_tensors_arrays(A, ia, B, ib)) < TOL


def test_batched_hyper_mode_via_plan(pq, O, be):
    # a label shared by both operands and the result (batch) inside a plan
    rng = np.random.default_rng(4)
    A = rand(rng, (96, 32, 5))   # m, k, z
    B = rand(rng, (32, 80, 5))   # k, n, z
    be.save_tensor_data("a", A)
    be.save_tensor_data("b", B)
    import ctypes as C
    from pqgb300 import _lib as L

    h = C.c_void_p()
    rc = be.lib.pq_plan_create(be.ctx, 2, L.arr(C.c_int32, [3, 3]), L.arr(C.c_int32, [0, 1, 3, 1, 2, 3]), 4,
                               L.arr(C.c_int64, [96, 32, 80, 5]), 1, L.arr(C.c_int32, [0, 1]), 3,
                               L.arr(C.c_int32, [0, 2, 3]), C.byref(h))
    L.check(rc, be.ctx, "plan_create")
    ids = L.arr(C.c_int64, [be.id_of("a"), be.id_of("b")])
    L.check(be.lib.pq_plan_execute(h, ids, be.id_of("r")), be.ctx, "execute")
    got = be.load_tensor_data("r")
    ref = np.einsum("mkz,knz->mnz", A, B)
    assert rel_err(got, ref) < TOL
    be.lib.pq_plan_destroy(h)


@pytest.mark.parametrize("prec", [2, 4], ids=["3xtf32", "6xtf32"])
def test_tc_plan_amplitude(pq, O, prec):
    """A sliced single amplitude on the tensor-core path vs the state vector."""
    be = pq.GB300Backend(prec)
    r, c, d = 4, 4, 10
    bits = "0110100111001010"
    g = pq.random_grid_gates(r, c, d, seed=3)
    net = pq.build_network(16, g, backend=be, decompose=True)
    pq.add_input(net, "0" * 16)
    pq.add_output(net, bits)
    steps, cm, mx, _ = pq.planning.best_flop_plan(net, out_edges=[], candidates=("sweep",))
    plan = pq.NetworkPlan(net, steps=steps, out_edges=[])
    sliced = plan.choose_slices(max_sliced=4, log2_target=28)
    amp = plan.run_sliced(sliced, batch=16)
    ref = O.statevector(16, g)[O.amplitude_index(bits)]
    assert abs(amp - ref) / 2.0 ** -8 < 1e-6
    plan.close()
    be.close()
