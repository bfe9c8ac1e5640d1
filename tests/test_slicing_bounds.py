"""The sliced-product arithmetic of the tensor-core kernels, restated in numpy.

The kernels split each operand of a complex 64 x 64 (or larger) product into
bf16 slices holding small integers and accumulate the slice products of one
level s + t in an FP32 accumulator of tensor memory (ozaki.cuh, tc_ozaki.cu).
That accumulation is exact only if every partial sum is an integer of at most
2^24 in magnitude; the kernels' error bound then follows from the dropped
levels and the last slice's rounding.  These checks run the same scaling
(powers of two from the exponent of each row / column maximum), the same
round-to-nearest peeling and the same level bookkeeping in float64 on random
operands, including rows and columns of very different magnitude, and assert:

  * every slice is an integer in [-2^b, 2^b] (b = 7 for the 8-bit slices of the
    d = 64 kernels, 5 for the 6-bit slices of the large-d GEMM);
  * every partial sum of every level, in the order the tensor core adds the
    K blocks, stays below 2^24, so FP32 holds it exactly;
  * the product matches the float64 product to a few units of 2^(-bits S)
    of the row and column scales.
"""
import numpy as np
import pytest


def scale_exp(m):
    """e with m < 2^e (m > 0): the exponent of the row / column maximum."""
    m = np.maximum(m, 2.0 ** -100)
    return np.floor(np.log2(m)).astype(np.int64) + 1


def peel(t, S, base):
    """Round-to-nearest slices: t = sum_s q_s base^(-s) + remainder."""
    qs = []
    for _ in range(S):
        q = np.rint(t)
        qs.append(q)
        t = (t - q) * base
    return qs


def sliced_product(A, B, S, bits, lmax):
    """C = A B (complex, d x d) the way the kernels form it; returns C and the
    largest partial level sum seen (in units of the integer slices)."""
    d = A.shape[0]
    base = 2.0 ** (bits + 1)
    lim = 2.0 ** bits
    # Real-stacked operands: [[A_r, -A_i], [A_i, A_r]] (rows 2d, K 2d) and [B_r; B_i].
    As = np.block([[A.real, -A.imag], [A.imag, A.real]])
    Bs = np.vstack([B.real, B.imag])
    ea = scale_exp(np.maximum(np.abs(A.real), np.abs(A.imag)).max(axis=1))
    eb = scale_exp(np.maximum(np.abs(B.real), np.abs(B.imag)).max(axis=0))
    ra = np.concatenate([ea, ea])                       # row scale of stacked row i
    qa = peel(As * 2.0 ** (bits - ra)[:, None], S, base)
    qb = peel(Bs * 2.0 ** (bits - eb)[None, :], S, base)
    for q in qa + qb:
        assert np.all(q == np.rint(q)) and np.abs(q).max() <= lim
    # Level sums, accumulated over K blocks of 128 real terms in order, with
    # the slice products of one level added one after the other.
    kb = 128
    worst = 0.0
    levels = []
    for L in range(lmax + 1):
        acc = np.zeros((2 * d, d))
        for k0 in range(0, 2 * d, kb):
            for s in range(S):
                t = L - s
                if t < 0 or t >= S:
                    continue
                acc = acc + qa[s][:, k0:k0 + kb] @ qb[t][k0:k0 + kb, :]
                worst = max(worst, np.abs(acc).max())
        levels.append(acc)
    D = sum(lv * base ** (-L) for L, lv in enumerate(levels))
    D = D * 2.0 ** (ra[:, None] - bits) * 2.0 ** (eb[None, :] - bits)
    return D[:d] + 1j * D[d:], worst


def operands(rng, d, spread):
    A = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    B = rng.standard_normal((d, d)) + 1j * rng.standard_normal((d, d))
    if spread:
        # rows / columns whose magnitudes differ by up to 2^spread
        A *= 2.0 ** rng.uniform(-spread, 0, size=(d, 1))
        B *= 2.0 ** rng.uniform(-spread, 0, size=(1, d))
    return A, B


@pytest.mark.parametrize("S", [2, 3, 4])
@pytest.mark.parametrize("spread", [0, 20])
def test_eight_bit_slices_accumulate_exactly(S, spread):
    """d = 64 kernels (split and plain forms): 8-bit slices, levels <= S - 1."""
    rng = np.random.default_rng(100 * S + spread)
    A, B = operands(rng, 64, spread)
    C, worst = sliced_product(A, B, S, bits=7, lmax=S - 1)
    assert worst < 2.0 ** 24
    ref = A @ B
    scale = np.abs(A).max(axis=1)[:, None] * np.abs(B).max(axis=0)[None, :] * 64
    err = np.abs(C - ref) / scale
    assert err.max() < 4 * 2.0 ** (-8 * S), err.max()


@pytest.mark.parametrize("d", [64, 512, 1536])
def test_six_bit_slices_of_the_large_gemm(d):
    """The large-d GEMM: five 6-bit slices, levels <= 4, K = d complex columns
    in blocks of 64; sums stay below 2^24 up to d = 1536, its largest size."""
    rng = np.random.default_rng(d)
    A, B = operands(rng, d, 10)
    C, worst = sliced_product(A, B, 5, bits=5, lmax=4)
    assert worst < 2.0 ** 24
    ref = A @ B
    scale = np.abs(A).max(axis=1)[:, None] * np.abs(B).max(axis=0)[None, :] * d
    err = np.abs(C - ref) / scale
    assert err.max() < 4 * 2.0 ** (-30), err.max()


def test_hermitian_b_from_a_slices():
    """For Hermitian X the slices of B = X (column scales) are the conjugated
    slices of A = X (row scales), so a product can read its B operand from A's
    slices (the split kernel's Hermitian steps) with the same numbers."""
    rng = np.random.default_rng(7)
    Z = rng.standard_normal((64, 64)) + 1j * rng.standard_normal((64, 64))
    X = (Z + Z.conj().T) / 2
    ea = scale_exp(np.maximum(np.abs(X.real), np.abs(X.imag)).max(axis=1))
    eb = scale_exp(np.maximum(np.abs(X.real), np.abs(X.imag)).max(axis=0))
    assert np.array_equal(ea, eb)
    qa_r = peel(X.real * 2.0 ** (7 - ea)[:, None], 3, 256.0)
    qa_i = peel(X.imag * 2.0 ** (7 - ea)[:, None], 3, 256.0)
    qb_r = peel(X.real * 2.0 ** (7 - eb)[None, :], 3, 256.0)
    qb_i = peel(X.imag * 2.0 ** (7 - eb)[None, :], 3, 256.0)
    for s in range(3):
        assert np.array_equal(qb_r[s], qa_r[s].T)
        assert np.array_equal(qb_i[s], -qa_i[s].T)
