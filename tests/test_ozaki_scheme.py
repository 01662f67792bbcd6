"""The digit scheme behind fg_dense_gemm_nt, restated with Python integers and checked on
the CPU (exact rational arithmetic for the references):

* the cut of a row into 7 signed 8-bit digits (row exponent from the largest biased exponent
  with one bit of headroom, |x| 2^-e < 1/4; 56 fraction bits, nearest digits by arithmetic
  shifts) gives digits in [-128, 128] and a leading digit in [-64, 64] -- exact bf16 values --
  and reconstructs every value to within 2^(e_i - 56);
* the FP32 accumulators stay exact: a weight class k = s + t sums at most 7 digit pairs, at
  most two of them with a leading digit (products <= 2^13) and at most six without (<= 2^14),
  so with K <= 170 every partial sum is an integer below 6 2^14 170 < 2^24;
* the epilogue's integer bookkeeping (hi in units of 2^-16 for classes 0-2, lo in units of
  2^-56 for classes 3-7, carries above 2^40 moved into hi) gives the same value;
* the product from the 34 kept digit pairs (s + t <= 7, s, t <= 6), K = 170 in one exact
  chunk, is within k 2^-52 max|a_i| max|b_j| of the exact product (the dropped pairs cost
  ~k 2^-57; the rest is the low bits of values far below their row's maximum), and within
  k 2^-57 when every value is within two binades of its row's maximum.
"""
from fractions import Fraction

import numpy as np

S = 7


def row_exponent(row):
    bits = [int(np.float64(v).view(np.int64)) & 0x7FFFFFFFFFFFFFFF for v in row]
    mx = max(bits) if bits else 0
    if mx == 0:
        return 0
    E = mx >> 52
    return (E if E else 1) - 1020


def cut(row, e):
    """digits[l][s] with row[l] ~= 2^e sum_s d_s 2^(-8(s+1))."""
    out = []
    for v in row:
        b = int(np.float64(v).view(np.int64)) & ((1 << 64) - 1)
        E = (b >> 52) & 0x7FF
        mant = (b & ((1 << 52) - 1)) | ((1 << 52) if E else 0)
        sh = (E if E else 1) - 1019 - e
        F = mant << sh if sh >= 0 else (mant >> -sh if sh > -64 else 0)
        if b >> 63:
            F = -F
        d = []
        for s in range(S - 1):
            q = 48 - 8 * s
            dg = (F + (1 << (q - 1))) >> q
            F -= dg << q
            d.append(dg)
        d.append(F)
        out.append(d)
    return out


def value(d, e):
    return sum(Fraction(x) * Fraction(2) ** (e - 8 * (s + 1)) for s, x in enumerate(d))


def test_digits_are_bf16_exact_and_reconstruct():
    rng = np.random.default_rng(0)
    for scale in (1.0, 1e-300, 1e300, 3.7e-5):
        row = rng.normal(size=64) * scale
        row[::7] *= 1e-9   # elements far below the row maximum lose their bits below 2^(e-56)
        row[::17] = 0.0
        e = row_exponent(row)
        for v, d in zip(row, cut(row, e)):
            assert all(-128 <= x <= 128 for x in d) and -64 <= d[0] <= 64
            assert abs(Fraction(float(v)) - value(d, e)) < Fraction(2) ** (e - 56)


def test_accumulators_stay_below_2_24():
    # worst cases at K = 170: class 6 = two pairs with a leading digit (|d_0| <= 64) and five
    # without; class 7 = six pairs without; classes 0-5 have fewer pairs
    K = 170
    assert (2 * 64 * 128 + 5 * 128 * 128) * K < 2 ** 24
    assert 6 * 128 * 128 * K < 2 ** 24
    assert 6 * 128 * 128 * (K + 1) >= 2 ** 24  # 170 is the largest such K


def test_kept_pairs_error_bound():
    rng = np.random.default_rng(1)
    m, n, k = 6, 5, 170
    A = rng.normal(size=(m, k))
    A[1:] = np.sign(A[1:]) * (1.0 + rng.random(size=(m - 1, k)))   # within two binades of the maximum
    A *= np.ldexp(1.0, rng.integers(-20, 21, size=m))[:, None]
    B = rng.normal(size=(n, k))
    B[1:] = np.sign(B[1:]) * (1.0 + rng.random(size=(n - 1, k)))   # within two binades of the maximum
    B[0, ::3] *= 1e-12
    ea = [row_exponent(A[i]) for i in range(m)]
    eb = [row_exponent(B[j]) for j in range(n)]
    da = [cut(A[i], ea[i]) for i in range(m)]
    db = [cut(B[j], eb[j]) for j in range(n)]
    for i in range(m):
        for j in range(n):
            cls = []
            for kk in range(8):
                c = sum(da[i][l][s] * db[j][l][kk - s] for l in range(k) for s in range(max(0, kk - 6), min(kk, 6) + 1))
                assert abs(c) < 2 ** 24
                cls.append(c)
            hi = cls[0] * 65536 + cls[1] * 256 + cls[2]
            lo = (cls[3] << 32) + (cls[4] << 24) + (cls[5] << 16) + (cls[6] << 8) + cls[7]
            carry = lo >> 40
            hi, lo = hi + carry, lo - (carry << 40)
            assert abs(lo) < 2 ** 40 and abs(hi) < 2 ** 53
            approx = (Fraction(hi) * Fraction(2) ** -16 + Fraction(lo) * Fraction(2) ** -56) * \
                Fraction(2) ** (ea[i] + eb[j] - 16)
            exact = sum(Fraction(float(x)) * Fraction(float(y)) for x, y in zip(A[i], B[j]))
            scale = Fraction(k) * Fraction(float(np.abs(A[i]).max())) * Fraction(float(np.abs(B[j]).max()))
            assert abs(approx - exact) <= scale * Fraction(2) ** -52
            if i > 0 and j > 0:
                assert abs(approx - exact) <= scale * Fraction(2) ** -57
