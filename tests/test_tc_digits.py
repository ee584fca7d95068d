"""CPU model of the tensor-core product's arithmetic (no GPU).

The kernel cuts each row of A and each column of B into S = 6 fixed-point digits of 8 bits,
a = 2^e * sum_i alpha_i 256^-i (|alpha_i| <= 128), multiplies digits exactly (bf16 x bf16 ->
fp32), sums at most 240 digit products exactly in fp32, keeps the digit pairs of weight
256^-t, t <= 7, and adds them in integers.  This restatement checks the format's claims in
NumPy integer arithmetic: digits reproduce the fixed-point value exactly and fit bf16, partial
sums stay below 2^22, and the product error stays below 2^-44 of K * max|A(i,:)| * max|B(:,j)|.
"""
import numpy as np

S, KITEM = 6, 240


def _exponent(v):
    """e with |v| < 2^(e - 1) for every entry (from the largest biased exponent)."""
    ef = (np.abs(v).view(np.int64) >> 52) & 0x7FF
    m = int(ef.max()) if v.size else 0
    return -1021 if m == 0 else m - 1021


def _digits(v, e):
    """Balanced base-256 digits of round(v * 2^(8S - e)); the top digit takes the rest."""
    V = np.rint(np.ldexp(v, 8 * S - e)).astype(np.int64)
    d = np.zeros(v.shape + (S,), np.int64)
    for j in range(S - 1, 0, -1):
        q = ((V + 128) & 255) - 128
        d[..., j] = q
        V = (V - q) >> 8
    d[..., 0] = V
    return d


def _product(A, B):
    M, K = A.shape
    out = np.zeros((M, B.shape[1]))
    er = np.array([_exponent(A[i]) for i in range(M)])
    Ad = np.stack([_digits(A[i], er[i]) for i in range(M)])                  # M x K x S
    for kb in range(0, K, KITEM):
        ke = min(K, kb + KITEM)
        for c in range(B.shape[1]):
            e = _exponent(B[kb:ke, c])
            Bd = _digits(B[kb:ke, c], e)                                   # k x S
            assert np.abs(Ad).max() <= 128 and np.abs(Bd).max() <= 128    # exact in bf16
            D = np.einsum("mki,kj->mij", Ad[:, kb:ke], Bd)                 # exact digit-pair sums
            assert np.abs(D).max() < 2 ** 22                              # exact in fp32
            for i in range(M):
                tot = 0
                for a in range(S):
                    for b in range(S - a):                               # weight 256^-(a+b+2) <= 256^-7
                        tot += int(D[i, a, b]) << (8 * (S - 1 - a - b))
                out[i, c] += np.ldexp(float(tot), int(er[i]) + e - 8 * (S + 1))
    return out


def test_digits_reproduce_the_fixed_point_value():
    r = np.random.default_rng(0)
    v = r.standard_normal(1000) * 10.0 ** r.uniform(-8, 8, 1000)
    v[:3] = [0.0, 2.0 ** 40, -(1.0 - 2.0 ** -53) * 2.0 ** 40]
    e = _exponent(v)
    d = _digits(v, e)
    back = np.zeros(v.shape, np.int64)
    for j in range(S):
        back = back * 256 + d[:, j]
    assert np.array_equal(back, np.rint(np.ldexp(v, 8 * S - e)).astype(np.int64))
    assert np.abs(d).max() <= 128


def test_product_error_bound():
    r = np.random.default_rng(1)
    for M, K in ((7, 50), (5, 500), (3, 241)):
        A = r.standard_normal((M, K)) * 10.0 ** r.uniform(-6, 6, (M, 1))
        B = r.standard_normal((K, 4)) * 10.0 ** r.uniform(-6, 6, (1, 4))
        A[0, 0] = 2.0 ** 20
        C = _product(A, B)
        scale = K * np.abs(A).max(1)[:, None] * np.abs(B).max(0)[None, :]
        assert np.all(np.abs(C - A @ B) <= 2.0 ** -44 * scale)
