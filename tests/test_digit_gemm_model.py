"""CPU model of the arithmetic of the tensor-core FP64 product (csrc/tc_dgemm.cu), in Python integers.

The kernel splits every element of op(A) (op(B)) into eight signed 7-bit digits at a power-of-two
scale per row (column), sums the digit products with s + t = g per 64-wide K block (exact in FP32
because each block sum stays below 2^21), combines the block sums in pairs 2^7 G_g + G_{g+1} (int32)
and accumulates them into one int64 per output with weights 2^(7(6-g) - R). This model follows the
same steps element by element and checks the bounds the kernel relies on (digit range, block sums
< 2^21, pair sums in int32, int64 range) and the error bound stated in the kernel against exact
rational arithmetic."""
import struct
from fractions import Fraction

import numpy as np
import pytest

S, BK = 8, 64


def row_exp(maxabs):
    """E with max|x| < 2^E, from the IEEE exponent field as the kernel does."""
    ex = struct.unpack("<Q", struct.pack("<d", maxabs))[0] >> 52
    return max(ex, 1) - 1022


def digits(x, E):
    bits = struct.unpack("<q", struct.pack("<d", x))[0]
    ab = bits & 0x7FFFFFFFFFFFFFFF
    ex = ab >> 52
    mant = ab & ((1 << 52) - 1)
    if ex:
        mant |= 1 << 52
    else:
        ex = 1
    sh = ex - 1020 - E
    if mant == 0:
        Y = 0
    elif sh >= 0:
        assert sh <= 2
        Y = mant << sh
    elif sh > -64:
        Y = (mant + (1 << (-sh - 1))) >> (-sh)
    else:
        Y = 0
    assert Y < 2 ** 55
    d = [0] * S
    for s in range(S - 1, 0, -1):
        v = Y & 127
        if v >= 64:
            v -= 128
        d[s] = v
        Y = (Y - v) >> 7
    d[0] = Y
    assert 0 <= d[0] <= 64 and all(-64 <= v <= 63 for v in d[1:])
    if bits < 0:
        d = [-v for v in d]
    return d


def model_gemm(A, B):
    """C = A @ B through the kernel's integer steps (A m x K, B K x n, float64)."""
    m, K = A.shape
    n = B.shape[1]
    Kp = -(-K // BK) * BK
    R = 0
    while (1 << (R + 1)) < Kp:
        R += 1
    EA = [row_exp(float(np.max(np.abs(A[i])))) for i in range(m)]
    EB = [row_exp(float(np.max(np.abs(B[:, j])))) for j in range(n)]
    da = [[digits(float(A[i, k]), EA[i]) for k in range(K)] for i in range(m)]
    db = [[digits(float(B[k, j]), EB[j]) for k in range(K)] for j in range(n)]
    C = np.zeros((m, n))
    for i in range(m):
        for j in range(n):
            acc = 0
            for k0 in range(0, K, BK):
                G = [sum(da[i][k][s] * db[j][k][g - s] for k in range(k0, min(K, k0 + BK)) for s in range(g + 1))
                     for g in range(S)]
                assert max(abs(x) for x in G) <= 2 ** 21      # exact in the FP32 tensor-memory accumulator
                for g in range(0, S, 2):                       # read back in pairs (g, g + 1)
                    p = (G[g] << 7) + G[g + 1]
                    assert abs(p) < 2 ** 31                    # int32
                    sh = 7 * (S - 2 - g) - R
                    acc += p << sh if sh >= 0 else (p + (1 << (-sh - 1))) >> (-sh)
                    assert abs(acc) < 2 ** 63                  # int64 accumulator
            C[i, j] = float(Fraction(acc) * Fraction(2) ** (EA[i] + EB[j] - 61 + R))
    return C


def exact(A, B):
    m, n = A.shape[0], B.shape[1]
    out = np.zeros((m, n))
    for i in range(m):
        for j in range(n):
            out[i, j] = float(sum(Fraction(float(a)) * Fraction(float(b)) for a, b in zip(A[i], B[:, j])))
    return out


@pytest.mark.parametrize("m,n,K,seed", [(3, 4, 64, 0), (2, 3, 200, 1), (4, 2, 130, 2)])
def test_model_matches_exact_product(m, n, K, seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((m, K)) * np.exp(rng.uniform(-8, 8, (m, 1)))   # per-row scales differ
    B = rng.standard_normal((K, n))
    B[rng.random((K, n)) < 0.1] = 0.0
    C = model_gemm(A, B)
    ref = exact(A, B)
    bound = K * np.abs(A).max(1)[:, None] * np.abs(B).max(0)[None, :] * (2.0 ** -53 + K * 2.0 ** -65)
    assert np.all(np.abs(C - ref) <= bound)


def test_model_largest_block_sums():
    """Digits 63 in every position but the last: group sums near the 2^21 bound stay exact."""
    Y = 63 * sum(128 ** j for j in range(1, 8))
    x = Y * 2.0 ** -54
    assert digits(x, row_exp(x)) == [63] * 7 + [0]
    K = 128
    A = np.full((2, K), x)
    B = np.full((K, 2), -x)
    C = model_gemm(A, B)
    ref = exact(A, B)
    assert np.all(np.abs(C - ref) <= K * x * x * 2.0 ** -52)


def test_digits_reconstruct():
    rng = np.random.default_rng(5)
    for x in list(rng.standard_normal(200) * 10.0 ** rng.integers(-300, 300, 200)) + [0.0, -0.0, 5e-324, 1.0, -1.0]:
        E = row_exp(abs(x)) + int(rng.integers(0, 3))
        d = digits(x, E)
        val = Fraction(sum(v * 128 ** (S - 1 - s) for s, v in enumerate(d))) * Fraction(2) ** (E - 55)
        assert abs(val - Fraction(x)) <= Fraction(2) ** (E - 56)
