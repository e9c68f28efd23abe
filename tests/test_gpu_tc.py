"""Split-precision tensor-core class (tcgen05, 3xTF32) vs the FP64 oracle.

GEMM-shaped pairs in PREC_3XTF32 contexts (M, N >= 64, K >= 16) run on the
tcgen05 kernels; tolerance 1e-5 relative to the largest result magnitude
(3xTF32 products with FP32 accumulation over K <= 1024).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5
TC_LAUNCHES = 4  # result index table, pack A, pack B, persistent tcgen05 GEMM
OZ_LAUNCHES = 5  # exponents of A and B, slices of B, result index table, GEMM


def launches_for(be, k):
    return OZ_LAUNCHES if be.precision in (3, 5) and k <= 512 else TC_LAUNCHES


def rel_err(a, b):
    a = np.asarray(a).reshape(-1)
    b = np.asarray(b).reshape(-1)
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def rand(rng, dims):
    return rng.standard_normal(dims) + 1j * rng.standard_normal(dims)


@pytest.fixture(params=[(2, None), (2, 0), (4, None), (5, None), (5, 0), (3, None)],
                ids=["3xtf32-mixed", "3xtf32-c64all", "6xtf32-mixed", "ozaki-mixed", "ozaki-c64all", "3xbf16-mixed"])
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
    assert nl == launches_for(be, 64)
    assert rel_err(got, A @ B) < TOL


@pytest.mark.parametrize("m,n,k", [(400, 72, 40), (128, 128, 64), (130, 260, 48), (1000, 96, 272), (200, 80, 600)])
def test_ragged_tiles(be, O, m, n, k):
    rng = np.random.default_rng(m + n + k)
    A = rand(rng, (k, m))
    B = rand(rng, (n, k))
    got, nl = run(be, A, [1, -1], B, [-2, 1])
    assert nl == launches_for(be, k)
    assert rel_err(got, A.T @ B.T) < TOL


def test_persistent_tiles_across_batch(pq, O, be):
    # more output tiles than SMs: each persistent CTA walks several tiles,
    # crossing batch (z) boundaries; ragged M, N and K
    rng = np.random.default_rng(5)
    m, n, k, z = 1000, 100, 40, 7
    A = rand(rng, (m, k, z))
    B = rand(rng, (k, n, z))
    be.save_tensor_data("a", A)
    be.save_tensor_data("b", B)
    import ctypes as C
    from pqgb300 import _lib as L

    h = C.c_void_p()
    rc = be.lib.pq_plan_create(be.ctx, 2, L.arr(C.c_int32, [3, 3]), L.arr(C.c_int32, [0, 1, 3, 1, 2, 3]), 4,
                               L.arr(C.c_int64, [m, k, n, z]), 1, L.arr(C.c_int32, [0, 1]), 3,
                               L.arr(C.c_int32, [3, 2, 0]), C.byref(h))
    L.check(rc, be.ctx, "plan_create")
    ids = L.arr(C.c_int64, [be.id_of("a"), be.id_of("b")])
    L.check(be.lib.pq_plan_execute(h, ids, be.id_of("r")), be.ctx, "execute")
    got = be.load_tensor_data("r")
    ref = np.einsum("mkz,knz->znm", A, B)
    assert rel_err(got, ref) < TOL
    be.lib.pq_plan_destroy(h)


def test_truncation_bias_is_corrected(pq):
    """The tensor core truncates accumulations; the kernel adds the expected
    shrinkage back.  The mean relative change of |C| over a large random
    product stays within 1e-8 (uncorrected it is about -9e-8), so it does not
    build up along a chain of contractions."""
    rng = np.random.default_rng(6)
    A = rand(rng, (512, 256)).astype(np.complex64)
    B = rand(rng, (256, 256)).astype(np.complex64)
    ref = A.astype(np.complex128) @ B.astype(np.complex128)
    for prec in (2, 4):
        be = pq.GB300Backend(prec, small_elems=0)
        got, nl = run(be, A, [-1, 1], B, [1, -2])
        be.close()
        assert nl == TC_LAUNCHES
        bias = float(np.mean(np.abs(got) / np.abs(ref)) - 1)
        assert abs(bias) < 1e-8, (prec, bias)


def test_permuted_bond2_modes(be, O):
    # interleaved free / contracted bond-2 modes in both operands
    rng = np.random.default_rng(3)
    ia = [-1, 1, -2, 2, -3, 3, -4, 4, -5, -6, 5, -7, 6, -8]
    ib = [3, -9, 1, -10, 5, 2, -11, 6, 4, -12, -13, -14, -15, -16]
    A = rand(rng, [2] * len(ia))
    B = rand(rng, [2] * len(ib))
    got, nl = run(be, A, ia, B, ib)
    assert nl == launches_for(be, 2 ** 6)
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


@pytest.mark.parametrize("prec", [2, 4, 5, 3], ids=["3xtf32", "6xtf32", "ozaki", "3xbf16"])
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
    # three bf16 slices keep about 21 bits: a looser bound for that mode
    assert abs(amp - ref) / 2.0 ** -8 < (2e-5 if prec == 3 else 1e-6)
    plan.close()
    be.close()


# ---- exact-accumulation (Ozaki scheme) kernels ------------------------------

def ozaki_backend(pq, small=0):
    return pq.GB300Backend(5, small_elems=small)


def ozaki_bound(A, B, ref):
    from oracle import ozaki_oracle as Z

    return Z.error_bound(np.asarray(A, dtype=np.complex128), np.asarray(B, dtype=np.complex128), ref)


def test_ozaki_matches_cpu_restatement(pq):
    """The device result equals the CPU restatement of the scheme (exact level
    0 and 1 sums, one final rounding): bit for bit on most elements (the
    device's FP32 level-2..4 sum, about 2^-30 of the scale, moves a few % of
    the final roundings), otherwise within one complex64 ulp plus 2^-28 of
    |row of A| |column of B|; and it is the FP64 product up to the scheme's
    error bound."""
    from oracle import ozaki_oracle as Z

    rng = np.random.default_rng(7)
    A = rand(rng, (512, 256)).astype(np.complex64)
    B = rand(rng, (256, 192))  # complex128 (a small tensor)
    be = ozaki_backend(pq, small=1 << 16)
    got, nl = run(be, A, [-1, 1], B, [1, -2])
    be.close()
    assert nl == OZ_LAUNCHES
    got = got.astype(np.complex64)
    orc, _ = Z.ozaki_matmul(A.astype(np.complex128), B)
    na = np.sqrt(np.sum(np.abs(A.astype(np.complex128)) ** 2, axis=1))
    nb = np.sqrt(np.sum(np.abs(B) ** 2, axis=0))
    for part in (np.real, np.imag):
        g, o = part(got).astype(np.float64), part(orc).astype(np.float64)
        ulp = np.spacing(np.abs(o).astype(np.float32)).astype(np.float64)
        assert np.all(np.abs(g - o) <= ulp + 2.0 ** -28 * np.outer(na, nb))
        assert np.mean(g == o) > 0.95
    ref = A.astype(np.complex128) @ B
    assert np.all(np.abs(got - ref) <= ozaki_bound(A, B, ref))


def test_ozaki_row_scales_and_zero_rows(pq):
    """Rows and columns of wildly different magnitude (per-row scaling), an
    all-zero row of A and an all-zero column of B."""
    rng = np.random.default_rng(8)
    A = rand(rng, (300, 128)) * np.exp2(rng.integers(-60, 60, size=(300, 1)))
    B = rand(rng, (128, 100)) * np.exp2(rng.integers(-40, 40, size=(1, 100)))
    A[17] = 0
    B[:, 5] = 0
    A = A.astype(np.complex64)
    be = ozaki_backend(pq)
    got, nl = run(be, A, [-1, 1], B.astype(np.complex64), [1, -2])
    be.close()
    assert nl == OZ_LAUNCHES
    B = B.astype(np.complex64).astype(np.complex128)
    ref = A.astype(np.complex128) @ B
    assert np.all(got[17] == 0) and np.all(got[:, 5] == 0)
    assert np.all(np.abs(got - ref) <= ozaki_bound(A, B, ref))


@pytest.mark.parametrize("m,n,k", [(4096, 16, 64), (3000, 24, 48), (2000, 8, 256), (16, 5000, 32), (40, 900, 96)])
def test_ozaki_narrow_pairs(pq, m, n, k):
    """Narrow pairs: 16- and 32-wide tiles for small N, and A/B swapped when
    M is the narrow side (boundary tensors absorbing one qubit's tensor)."""
    rng = np.random.default_rng(m + n + k)
    A = rand(rng, (m, k)).astype(np.complex64)
    B = rand(rng, (k, n)).astype(np.complex64)
    be = ozaki_backend(pq)
    got, nl = run(be, A, [-1, 1], B, [1, -2])
    be.close()
    assert nl == OZ_LAUNCHES
    A, B = A.astype(np.complex128), B.astype(np.complex128)
    ref = A @ B
    assert np.all(np.abs(got - ref) <= ozaki_bound(A, B, ref))


def test_3xbf16_matches_cpu_restatement(pq):
    """Three bf16 slices: the device result is the CPU restatement with
    n_slices = 3 up to one final rounding, within the scheme's bound."""
    from oracle import ozaki_oracle as Z

    rng = np.random.default_rng(10)
    A = rand(rng, (384, 128)).astype(np.complex64)
    B = rand(rng, (128, 200)).astype(np.complex64)
    be = pq.GB300Backend(3, small_elems=0)
    got, nl = run(be, A, [-1, 1], B, [1, -2])
    be.close()
    assert nl == OZ_LAUNCHES
    A, B = A.astype(np.complex128), B.astype(np.complex128)
    orc, _ = Z.ozaki_matmul(A, B, n_slices=3)
    ref = A @ B
    assert np.all(np.abs(got - ref) <= Z.error_bound(A, B, ref, n_slices=3))
    assert np.max(np.abs(got - orc)) <= 2.0 ** -22 * np.max(np.abs(orc))


def test_ozaki_k512_exact_limit(pq):
    """K = 512 is the largest K whose level sums stay exact; K = 513 runs on
    the 6xTF32 kernels."""
    rng = np.random.default_rng(9)
    for k, launches in ((512, OZ_LAUNCHES), (513, TC_LAUNCHES)):
        A = rand(rng, (256, k)).astype(np.complex64)
        B = rand(rng, (k, 128)).astype(np.complex64)
        be = ozaki_backend(pq)
        got, nl = run(be, A, [-1, 1], B, [1, -2])
        be.close()
        assert nl == launches
        ref = A.astype(np.complex128) @ B.astype(np.complex128)
        if launches == OZ_LAUNCHES:
            assert np.all(np.abs(got - ref) <= ozaki_bound(A, B, ref))
        else:
            assert rel_err(got, ref) < TOL
