"""CPU checks of the exact-accumulation scheme's restatement (oracle/ozaki_oracle.py):
the slicing is exact, the level sums stay on their grids, and the result is
the FP64 product up to the final rounding."""
import numpy as np

from oracle import ozaki_oracle as Z


def rand(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def test_pairs_are_levels_up_to_four():
    assert len(Z.PAIRS) == 15
    assert all(i + j <= 4 for i, j in Z.PAIRS)
    assert len(set(Z.PAIRS)) == 15


def test_slices_exact_in_bf16_and_reconstruct():
    rng = np.random.default_rng(0)
    x = rng.uniform(-1, 1, 100000)
    x[:5] = [0.0, -0.999999940395, 0.999999940395, 2.0 ** -40, -(2.0 ** -8)]
    s = Z.slices(x)
    for i, si in enumerate(s):
        assert Z.bf16_exact(si)
        g = 2.0 ** (7 * (i + 1))
        assert np.all(np.rint(si * g) == si * g)  # on the slice grid
        assert np.all(np.abs(si) <= (1.0 if i == 0 else 2.0 ** (-7 * i - 1)))
    assert np.max(np.abs(x - sum(s))) <= 2.0 ** -36


def test_row_exponents_bound_rows():
    rng = np.random.default_rng(1)
    X = rand(rng, (50, 40)) * np.exp2(rng.integers(-50, 50, size=(50, 1)))
    X[3] = 0
    e = Z.row_exponents(X)
    assert e[3] == Z.ZERO_EXP
    live = e != Z.ZERO_EXP
    m = np.maximum(np.abs(X.real), np.abs(X.imag)).max(axis=1)
    assert np.all(m[live] < np.exp2(e[live].astype(float)))
    assert np.all(m[live] >= np.exp2(e[live].astype(float) - 1))


def test_level_sums_on_exact_grids_for_k512():
    rng = np.random.default_rng(2)
    A = rand(rng, (16, 512))
    B = rand(rng, (512, 8))
    _, lv = Z.ozaki_matmul(A, B)
    for part in (lv[0].real, lv[0].imag):
        assert np.all(np.rint(part * 2.0 ** 14) == part * 2.0 ** 14)
        assert np.max(np.abs(part)) * 2.0 ** 14 < 2.0 ** 24  # fits the FP32 significand
    for part in (lv[1].real, lv[1].imag):
        assert np.all(np.rint(part * 2.0 ** 21) == part * 2.0 ** 21)
        assert np.max(np.abs(part)) * 2.0 ** 21 < 2.0 ** 24


def test_result_is_rounded_fp64_product():
    rng = np.random.default_rng(3)
    A = rand(rng, (64, 256)).astype(np.complex64).astype(np.complex128)
    B = rand(rng, (256, 48))
    C, _ = Z.ozaki_matmul(A, B)
    ref = A @ B
    assert np.all(np.abs(C - ref) <= Z.error_bound(A, B, ref))
