"""FP64 CPU restatement of the exact-accumulation tensor-core contraction
(PQ_PREC_OZAKI) -- test infrastructure only.

The Ozaki scheme (Ozaki, Ogita, Oishi, Rump, "Error-free transformations of
matrix multiplication by using fast routines of matrix multiplication and its
applicability", Numer. Algorithms 59, 2012) as the library runs it:

* every row of A (over K) and every column of B is scaled by 2^-e, e the
  frexp exponent of the largest |Re| or |Im| of that row / column;
* a scaled value x in (-1, 1) is cut into five slices
  s0 = rint(x 2^7) 2^-7, s_i = rint((x - s0 - ... - s_{i-1}) 2^{7(i+1)}) 2^{-7(i+1)};
* the complex product is formed from the 15 slice pairs (i, j) with
  i + j <= 4, summed per level 0, 1 and 2-4; level 0 and 1 sums are exact
  (FP32 on the device, FP64 here), and the result is
  (L0 + L1 + L2) 2^(ea + eb) rounded once to the output type.

Level-0 and level-1 sums are exact in both places, so the device result
equals ``ozaki_matmul`` up to the FP32 rounding of the small level-2-4 sum
(about 2^-30 relative) before the final rounding.
"""
from __future__ import annotations

import numpy as np

N_SLICES = 5
BITS = 7


def pairs(n_slices=N_SLICES):
    """Slice pairs (i, j) with i + j < n_slices (15 for five slices, 6 for
    the three of PQ_PREC_3XBF16)."""
    return [(i, lvl - i) for lvl in range(n_slices) for i in range(lvl + 1)]


PAIRS = pairs()
ZERO_EXP = -4096


def row_exponents(X):
    """frexp exponent of max(|Re|, |Im|) over each row of X (rows x K);
    ZERO_EXP for an all-zero row."""
    m = np.maximum(np.abs(X.real), np.abs(X.imag)).max(axis=1)
    e = np.frexp(m)[1].astype(np.int64)
    e[m == 0] = ZERO_EXP
    return e


def slices(x, n_slices=N_SLICES):
    """The fixed-grid slices of x (|x| < 1), each exact in bf16."""
    out = []
    r = np.array(x, dtype=np.float64)
    for i in range(n_slices):
        g = 2.0 ** (BITS * (i + 1))
        s = np.rint(r * g) / g
        out.append(s)
        r = r - s
    return out


def bf16_exact(v):
    """True where v is exactly representable in bf16 (8 significant bits)."""
    v = np.asarray(v, dtype=np.float64)
    m, _ = np.frexp(v)
    return np.all(np.rint(m * 256) == m * 256)


def ozaki_matmul(A, B, out_dtype=np.complex64, n_slices=N_SLICES):
    """C = A @ B (A: M x K, B: K x N complex) the way the device computes it;
    returns (C rounded to out_dtype, levels (L0, L1, L2) complex, unscaled)."""
    ea = row_exponents(A)
    eb = row_exponents(B.T)
    sa = np.where(ea == ZERO_EXP, 0, -ea).astype(np.float64)
    sb = np.where(eb == ZERO_EXP, 0, -eb).astype(np.float64)
    As = A * np.exp2(sa)[:, None]
    Bs = B * np.exp2(sb)[None, :]
    ar, ai = slices(As.real, n_slices), slices(As.imag, n_slices)
    br, bi = slices(Bs.real, n_slices), slices(Bs.imag, n_slices)
    lv = [np.zeros((A.shape[0], B.shape[1]), dtype=np.complex128) for _ in range(3)]
    for i, j in pairs(n_slices):
        lvl = min(i + j, 2)
        lv[lvl] += (ar[i] @ br[j] - ai[i] @ bi[j]) + 1j * (ar[i] @ bi[j] + ai[i] @ br[j])
    scale = np.exp2((ea[:, None] + eb[None, :]).astype(np.float64))
    zero = (ea[:, None] == ZERO_EXP) | (eb[None, :] == ZERO_EXP)
    C = np.where(zero, 0, (lv[0] + lv[1] + lv[2]) * scale)
    return C.astype(out_dtype), lv


def error_bound(A, B, ref, n_slices=N_SLICES):
    """Per-element bound on |device result - A @ B| (A: M x K, B: K x N):
    the output rounding (2^-24 relative per component, |.| <= 2^-23 |ref|)
    plus, per real product, the dropped slice pairs of level >= n_slices and
    the slice residuals (below 2^-(7 n_slices - 1) of the row / column scales
    2^ea, 2^eb, with a factor 2 of margin), two
    real products per component and K terms, and the truncations of the small
    level-2-4 accumulator (below 2^-30 of the scales after K terms)."""
    ea = row_exponents(A).astype(np.float64)
    eb = row_exponents(B.T).astype(np.float64)
    K = A.shape[1]
    scale = np.exp2(np.minimum(ea, 4096)[:, None] + np.minimum(eb, 4096)[None, :])
    return 2.0 ** -23 * np.abs(ref) + (2.0 ** -(7 * n_slices - 3) * K + 2.0 ** -29) * scale
