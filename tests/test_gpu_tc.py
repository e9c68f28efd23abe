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


@pytest.mark.parametrize("order", ["mk", "km"])
def test_ozaki_row_scales_and_zero_rows(pq, order):
    """Rows and columns of wildly different magnitude (per-row scaling), an
    all-zero row of A and an all-zero column of B; A contiguous along M (row
    per thread exponent pass) or along K (row per warp)."""
    rng = np.random.default_rng(8)
    A = rand(rng, (300, 128)) * np.exp2(rng.integers(-60, 60, size=(300, 1)))
    B = rand(rng, (128, 100)) * np.exp2(rng.integers(-40, 40, size=(1, 100)))
    A[17] = 0
    B[:, 5] = 0
    A = A.astype(np.complex64)
    be = ozaki_backend(pq)
    if order == "km":
        got, nl = run(be, A.T, [1, -1], B.astype(np.complex64), [1, -2])
    else:
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


def _restatement_match(got, A, B):
    """complex64 result vs the CPU restatement: within one ulp plus 2^-28 of
    |row of A| |column of B|, bit-identical on most elements."""
    from oracle import ozaki_oracle as Z

    orc, _ = Z.ozaki_matmul(A, B)
    na = np.sqrt(np.sum(np.abs(A) ** 2, axis=1))
    nb = np.sqrt(np.sum(np.abs(B) ** 2, axis=0))
    for part in (np.real, np.imag):
        g, o = part(got).astype(np.float64), part(orc).astype(np.float64)
        ulp = np.spacing(np.abs(o).astype(np.float32)).astype(np.float64)
        assert np.all(np.abs(g - o) <= ulp + 2.0 ** -28 * np.outer(na, nb))
        assert np.mean(g == o) > 0.95


@pytest.mark.parametrize("order", ["mk", "km"])
@pytest.mark.parametrize("n,k,small", [(16, 40, 0), (16, 256, 0), (32, 24, 0), (32, 72, 0), (48, 40, 0),
                                       (64, 256, 0), (16, 48, 1 << 30)],
                         ids=["n16-k40", "n16-k256", "n32-k24", "n32-k72", "n48-k40", "n64-k256", "n16-c128"])
def test_ozaki_narrow_many_tiles_per_cta(pq, order, n, k, small):
    """Narrow tiles (N <= 64: two accumulator sets in TMEM, alternate tiles)
    over many row tiles: 64 * 152 * 3 + 37 rows give every persistent CTA
    three or four tiles (the last one ragged), and with an odd number of K
    tiles the two converter groups (alternate K tiles) swap roles from one
    tile to the next; A contiguous along M or along K (the K-major exponent
    pass), complex64 or complex128, with an all-zero row; a ragged last K
    tile."""
    rng = np.random.default_rng(n + k)
    m = 64 * 152 * 3 + 37
    A = rand(rng, (m, k))
    A[1000] = 0
    B = rand(rng, (k, n))
    if not small:
        A, B = A.astype(np.complex64), B.astype(np.complex64)
    be = ozaki_backend(pq, small=small)
    if order == "km":
        got, nl = run(be, A.T, [1, -1], B, [1, -2])  # stored column-major: K contiguous
    else:
        got, nl = run(be, A, [-1, 1], B, [1, -2])
    be.close()
    assert nl == OZ_LAUNCHES
    A, B = A.astype(np.complex128), B.astype(np.complex128)
    ref = A @ B
    assert np.all(got[1000] == 0)
    assert np.all(np.abs(got - ref) <= ozaki_bound(A, B, ref))
    if not small:
        _restatement_match(got, A, B)


def test_ozaki_narrow_tiles_across_batch(pq, O):
    """A narrow batched pair (hyper mode z kept in the result): persistent
    CTAs cross z boundaries as well as row tiles, three K tiles per tile."""
    import ctypes as C
    from pqgb300 import _lib as L

    rng = np.random.default_rng(12)
    m, k, n, z = 3000, 40, 16, 9
    A = rand(rng, (m, k, z)).astype(np.complex64)
    B = rand(rng, (k, n, z)).astype(np.complex64)
    be = ozaki_backend(pq)
    be.save_tensor_data("a", A)
    be.save_tensor_data("b", B)
    h = C.c_void_p()
    rc = be.lib.pq_plan_create(be.ctx, 2, L.arr(C.c_int32, [3, 3]), L.arr(C.c_int32, [0, 1, 3, 1, 2, 3]), 4,
                               L.arr(C.c_int64, [m, k, n, z]), 1, L.arr(C.c_int32, [0, 1]), 3,
                               L.arr(C.c_int32, [3, 2, 0]), C.byref(h))
    L.check(rc, be.ctx, "plan_create")
    ids = L.arr(C.c_int64, [be.id_of("a"), be.id_of("b")])
    n0 = be.launch_count()
    L.check(be.lib.pq_plan_execute(h, ids, be.id_of("r")), be.ctx, "execute")
    assert be.launch_count() - n0 == OZ_LAUNCHES
    got = be.load_tensor_data("r")
    be.lib.pq_plan_destroy(h)
    be.close()
    A, B = A.astype(np.complex128), B.astype(np.complex128)
    for iz in range(z):
        ref = A[:, :, iz] @ B[:, :, iz]
        assert np.all(np.abs(got[iz].T - ref) <= ozaki_bound(A[:, :, iz], B[:, :, iz], ref))


def test_3xbf16_narrow_many_tiles_per_cta(pq):
    """Three bf16 slices on 16-wide tiles, two or three tiles per CTA."""
    from oracle import ozaki_oracle as Z

    rng = np.random.default_rng(13)
    A = rand(rng, (64 * 152 * 2 + 5, 64)).astype(np.complex64)
    B = rand(rng, (64, 16)).astype(np.complex64)
    be = pq.GB300Backend(3, small_elems=0)
    got, nl = run(be, A, [-1, 1], B, [1, -2])
    be.close()
    assert nl == OZ_LAUNCHES
    A, B = A.astype(np.complex128), B.astype(np.complex128)
    ref = A @ B
    assert np.all(np.abs(got - ref) <= Z.error_bound(A, B, ref, n_slices=3))


def test_ozaki_tall_narrow_pair(pq):
    """More than 65535 * 128 rows (a 2^23-row boundary tensor absorbing a
    16-column gate tensor over K = 32, stored contiguous along K): the exact
    path takes it, the exponent pass on grid x with no 65535 limit."""
    rng = np.random.default_rng(14)
    m, k, n = (1 << 23) + 4097, 32, 16
    A = rng.standard_normal((m, 2 * k), dtype=np.float32).view(np.complex64)
    B = rand(rng, (k, n)).astype(np.complex64)
    be = ozaki_backend(pq)
    got, nl = run(be, A.T, [1, -1], B, [1, -2])  # A.T is (K, M) column-major: no host copy
    be.close()
    assert nl == OZ_LAUNCHES
    rows = np.concatenate([np.arange(64), rng.choice(m, 4096, replace=False), np.arange(m - 64, m)])
    A, B = A[rows].astype(np.complex128), B.astype(np.complex128)
    ref = A @ B
    assert np.all(np.abs(got[rows] - ref) <= ozaki_bound(A, B, ref))


@pytest.mark.parametrize("ia", [[1, -1, -2, 2, -3, 3, -4, 4, -5, 5, -6, 6, -7, -8, -9, -10],
                                [1, 2, -1, -2, 3, -3, 4, -4, 5, -5, 6, -6, -7, -8, -9, -10],
                                [1, 2, 3, -1, -2, 4, -3, 5, -4, 6, -5, -6, -7, -8, -9, -10]],
                         ids=["k-run-2", "k-run-4", "k-run-8"])
def test_ozaki_stride1_mode_contracted(pq, O, ia):
    """A's unit-stride mode is contracted, in a run of 2, 4 or 8 elements
    before its first open mode (a boundary tensor whose fastest qubits meet
    the gate tensor): the exponent pass reads A K-major with 2, 4 or 8 lanes
    per row; all bond-2 modes, K = 64, M = 1024, N = 16."""
    rng = np.random.default_rng(15 + len(ia))
    ib = [1, 2, 3, 4, 5, 6, -11, -12, -13, -14]
    A = (rand(rng, [2] * len(ia)) * np.exp2(rng.integers(-30, 30, size=[2] * len(ia)) // 8)).astype(np.complex64)
    B = rand(rng, [2] * len(ib)).astype(np.complex64)
    be = ozaki_backend(pq)
    got, nl = run(be, A, ia, B, ib)
    be.close()
    assert nl == OZ_LAUNCHES
    ref = O.contract_tensors_arrays(A.astype(np.complex128), ia, B.astype(np.complex128), ib)
    assert rel_err(got, ref) < 3e-7


@pytest.mark.parametrize("small", [1 << 16, 1 << 62], ids=["c64-storage", "c128-storage"])
def test_ozaki4_matches_cpu_restatement(pq, small):
    """Four bf16 slices (PQ_PREC_OZAKI4, ten slice-pair products): the device
    result is the CPU restatement with n_slices = 4 up to the FP32 sum of the
    small levels and the output rounding, and the FP64 product within the
    scheme's bound; with every tensor stored as complex128 the result is not
    rounded to complex64 at all."""
    from oracle import ozaki_oracle as Z

    rng = np.random.default_rng(12)
    A = rand(rng, (384, 256))
    B = rand(rng, (256, 200))
    if small < (1 << 62):
        A = A.astype(np.complex64).astype(np.complex128)
    be = pq.GB300Backend(pq.PREC_OZAKI4, small_elems=small)
    got, nl = run(be, A, [-1, 1], B, [1, -2])
    be.close()
    assert nl == OZ_LAUNCHES
    c128 = small >= (1 << 62)
    orc, _ = Z.ozaki_matmul(A, B, out_dtype=np.complex128 if c128 else np.complex64, n_slices=4)
    ref = A @ B
    bound = Z.error_bound(A, B, ref, n_slices=4)
    assert np.all(np.abs(got - ref) <= bound)
    na = np.sqrt(np.sum(np.abs(A) ** 2, axis=1))
    nb = np.sqrt(np.sum(np.abs(B) ** 2, axis=0))
    tol = (2.0 ** -23 * np.abs(orc) if small < (1 << 62) else 0) + 2.0 ** -28 * np.outer(na, nb)
    assert np.all(np.abs(got - orc) <= tol)


def test_ozaki4_c128_plan_amplitude(pq, O):
    """A sliced amplitude with four slices and complex128 storage against
    the state vector: the error is far below the complex64-storage modes'."""
    be = pq.GB300Backend(pq.PREC_OZAKI4, small_elems=1 << 62)
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
    assert abs(amp - ref) / 2.0 ** -8 < 1e-7
    plan.close()
    be.close()
