"""The float-float arithmetic of the residual products (spmm_ff_kernel) and of
the Jacobian's recombination, restated in numpy with FP32 rounding at every
step: a compensated sum of exact products (TwoProd by FMA, cross terms,
TwoSum) carries about 2^-46 of sum |a||x|, the accuracy the mixed path's
reliable updates rely on for stopping tests of 1e-13 and coarser."""
import numpy as np

f32 = np.float32


def split(x):
    hi = f32(x)
    return hi, f32(x - np.float64(hi))


def fma32(a, b, c):
    # a*b + c rounded to FP32: a*b is exact in FP64 for FP32 a, b; the sum is
    # rounded twice (FP64, then FP32), which moves no bound this test checks
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def ff_mac(sh, sl, ah, al, bh, bl):
    """(sh, sl) += (ah, al) * (bh, bl), as ff2_mac does lane by lane"""
    p = f32(ah * bh)
    e = fma32(ah, bh, -p)
    e = fma32(ah, bl, e)
    e = fma32(al, bh, e)
    t = f32(sh + p)
    bp = f32(t - sh)
    err = f32(f32(sh - f32(t - bp)) + f32(p - bp))
    return t, f32(sl + f32(err + e))


def test_float_float_row_sums():
    rng = np.random.default_rng(1)
    worst = 0.0
    for _ in range(200):
        m = int(rng.integers(5, 30))
        a = rng.standard_normal(m) * np.exp(rng.uniform(-3, 3, m))
        x = rng.standard_normal(m) * np.exp(rng.uniform(-3, 3, m))
        sh = sl = f32(0.0)
        for ai, xi in zip(a, x):
            ah, al = split(ai)
            xh, xl = split(xi)
            sh, sl = ff_mac(sh, sl, ah, al, xh, xl)
        got = np.float64(sh) + np.float64(sl)
        exact = float(np.sum(np.array(a, dtype=np.longdouble) * np.array(x, dtype=np.longdouble)))
        worst = max(worst, abs(got - exact) / float(np.sum(np.abs(a * x))))
    assert worst < 2.0 ** -45
