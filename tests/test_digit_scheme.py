"""The digit scheme of the tensor-core Jacobian, restated in numpy: each
float-float value (hi, lo) of a row or column, scaled by a power of two to
|x| < 128, is cut into 7 balanced base-256 digits of hi and of lo, added; the
digit products are summed per level t + u.  These checks hold the bounds the
kernel relies on: every digit is an integer in [-256, 256] (exact in bf16),
every level sum over K <= 64 terms and at most four digit pairs stays below
2^24 (exact in FP32), and the levels rebuild the product sum to the FP64
rounding level."""
import numpy as np

S = 7


def split_ff(x):
    hi = x.astype(np.float32)
    lo = (x - hi.astype(np.float64)).astype(np.float32)
    return hi, lo


def digits(v32, sc):
    """balanced base-256 digits of v32 * sc (float32 arithmetic, as the kernel)"""
    r = (v32 * np.float32(sc)).astype(np.float32)
    out = []
    for _ in range(S):
        a = np.rint(r).astype(np.float32)
        out.append(a)
        r = ((r - a) * np.float32(256.0)).astype(np.float32)
    return out


def row_digits(x):
    """x: (rows, K) float64 -> per-digit integer arrays and the row exponents"""
    hi, lo = split_ff(x)
    mx = np.max(np.abs(hi), axis=1, keepdims=True)
    E = np.where(mx > 0, np.floor(np.log2(np.where(mx > 0, mx, 1))) + 1, 0)  # mx < 2^E
    sc = np.exp2(7 - E)
    dh, dl = digits(hi, sc), digits(lo, sc)
    return [a + b for a, b in zip(dh, dl)], E


def test_digit_bounds_level_sums_and_accuracy():
    rng = np.random.default_rng(0)
    K = 64
    # rows spanning a few decades (neighbourhood values of a field) with signs
    A = rng.standard_normal((40, K)) * np.exp(rng.uniform(-4, 4, (40, 1)))
    B = rng.standard_normal((K, 24)) * np.exp(rng.uniform(-4, 4, (1, 24)))
    da, Ea = row_digits(A)
    db, Eb = row_digits(B.T)
    for d in da + db:
        assert np.all(np.abs(d) <= 256) and np.all(d == np.round(d))
    total = np.zeros((A.shape[0], B.shape[1]))
    for L in range(S):
        acc = np.zeros_like(total)
        pairs = [(t, L - t) for t in range(L + 1) if t < S and L - t < S]
        for t, u in pairs:
            acc += da[t].astype(np.float64) @ db[u].astype(np.float64).T
        if L <= 3:  # the kernel keeps these levels apart: their sums must be exact in FP32
            assert len(pairs) <= 4 and np.max(np.abs(acc)) < 2.0 ** 24
        total += acc * 256.0 ** -L
    approx = total * np.exp2(Ea + Eb.T - 14)
    exact = A @ B
    scale = np.abs(A) @ np.abs(B)
    assert np.max(np.abs(approx - exact) / scale) < 2.0 ** -48
