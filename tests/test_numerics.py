"""CPU: the arithmetic the mixed form's kernels build on, restated in numpy.

* f2d_exact (csrc/lm_kernels.cuh): float -> double by integer bit operations
  is exact for every finite normal float.
* df_add_prod / df_add (csrc/lm_kernels.cuh): sums of w a b over FP32 values
  kept as FP32 (hi, lo) pairs — products split exactly with an FMA, Knuth's
  two-sum — carry about 48 bits, so the point sums V, v and the camera
  gradient sums stay FP64-grade even where their terms cancel.
* rcp_newton (csrc/lm_kernels.cuh): an FP32 reciprocal refined by one FP64
  Newton step is accurate to ~1e-14 relative over the range of depths.

The FMA of the device code is emulated by forming the product in FP64 (the
product of two FP32 values is exact there) and rounding once to FP32.
"""
import numpy as np

f32 = np.float32


def f2d_bits(u: np.ndarray) -> np.ndarray:
    """f2d_exact on normal floats: sign | (exponent + 896, mantissa >> 3) | mantissa << 29."""
    u = u.astype(np.uint32)
    hi = (u & np.uint32(0x80000000)) | (((u & np.uint32(0x7FFFFFFF)) >> np.uint32(3))
                                        + np.uint32(896 << 20))
    lo = (u << np.uint32(29)).astype(np.uint32)
    return ((hi.astype(np.uint64) << np.uint64(32)) | lo.astype(np.uint64)).view(np.float64)


def test_integer_float_to_double_is_exact():
    rng = np.random.default_rng(11)
    u = rng.integers(0, 2**32, 2_000_000, dtype=np.uint64).astype(np.uint32)
    ex = (u >> 23) & 0xFF
    u = u[(ex != 0) & (ex != 0xFF)]  # zero, subnormal, inf, NaN take the hardware path
    assert np.array_equal(f2d_bits(u), u.view(np.float32).astype(np.float64))


def fma32(a, b, c):
    """fmaf(a, b, c): exact a b + c rounded once (a b is exact in FP64)."""
    return f32(np.float64(a) * np.float64(b) + np.float64(c))


def df_add_prod(hi, lo, p, q, b):
    a = f32(p * b)
    c = f32(fma32(p, b, -a) + f32(q * b))
    s = f32(hi + a)
    bb = f32(s - hi)
    lo = f32(lo + f32(f32(f32(hi - f32(s - bb)) + f32(a - bb)) + c))
    return s, lo


def test_double_float_sums_of_products_reach_fp64_grade():
    rng = np.random.default_rng(5)
    worst = 0.0
    for _ in range(200):
        m = int(rng.integers(2, 40))
        w = rng.uniform(0.0, 1.0, m).astype(np.float32)
        a = rng.normal(0.0, 1e3, m).astype(np.float32)
        b = rng.normal(0.0, 1e3, m).astype(np.float32)
        # cancellation: the terms nearly sum to zero
        b[-1] = f32(-(np.sum(np.float64(w[:-1]) * a[:-1] * b[:-1])) / (np.float64(w[-1]) * a[-1]))
        hi, lo = f32(0.0), f32(0.0)
        for k in range(m):
            p = f32(w[k] * a[k])
            q = fma32(w[k], a[k], -p)
            hi, lo = df_add_prod(hi, lo, p, q, b[k])
        got = np.float64(hi) + np.float64(lo)
        exact = sum((np.float64(w[k]) * np.float64(a[k])) * np.float64(b[k]) for k in range(m))
        scale = float(np.sum(np.abs(np.float64(w) * a * np.float64(b))))
        worst = max(worst, abs(got - exact) / scale)
    # about 48 bits relative to the size of the terms (FP32 alone: ~1e-7)
    assert worst < 1e-13, worst


def test_newton_reciprocal_of_depths():
    z = np.concatenate([np.geomspace(1.1e-6, 1e4, 20000), np.random.default_rng(2).uniform(1, 500, 20000)])
    r0 = (np.float32(1.0) / z.astype(np.float32)).astype(np.float64)
    r = r0 + r0 * (1.0 - z * r0)  # fma(r, fma(-x, r, 1), r)
    rel = np.abs(r * z - 1.0)
    assert rel.max() < 1e-13, rel.max()
