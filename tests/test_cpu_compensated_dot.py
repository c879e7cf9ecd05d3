"""The differentiable chain's dot products as compensated float32 sums (csrc/soft.cu:
soft_dot_add, soft_two_sum, soft_warp_dot), restated in numpy float32 and checked against the
exactly rounded sum of the products.

Per thread a product a b is split into p = fl(a b) and e = fma(a, b, -p) (exact: here the
double product of two floats is exact and so is its difference with p), e is added to lo and
p enters hi by TwoSum; a warp's 32 (hi, lo) pairs combine by a shuffle tree the same way, and
only then is hi + lo taken in double.  Claimed: the relative error of a warp's sum is about
2^-48, against about 2^-24 times the condition of a plain float32 sum.
"""
import math

import numpy as np

f32 = np.float32


def two_sum(hi, lo, v):
    s = f32(hi + v)
    bb = f32(s - hi)
    lo = f32(lo + f32(f32(hi - f32(s - bb)) + f32(v - bb)))
    return s, lo


def dot_add(hi, lo, a, b):
    p = f32(a * b)
    e = f32(float(a) * float(b) - float(p))     # fma(a, b, -p), exact
    lo = f32(lo + e)
    return two_sum(hi, lo, p)


def warp_dot(a, b, per_thread):
    """32 lanes, each summing per_thread consecutive products, then the shuffle tree."""
    hi = [f32(0)] * 32
    lo = [f32(0)] * 32
    for lane in range(32):
        for k in range(per_thread):
            i = lane * per_thread + k
            hi[lane], lo[lane] = dot_add(hi[lane], lo[lane], a[i], b[i])
    o = 16
    while o > 0:
        for lane in range(o):                   # lane takes lane + o (shfl_down)
            lo[lane] = f32(lo[lane] + lo[lane + o])
            hi[lane], lo[lane] = two_sum(hi[lane], lo[lane], hi[lane + o])
        o //= 2
    return float(hi[0]) + float(lo[0])


def test_compensated_warp_dot_is_near_the_exactly_rounded_sum():
    rng = np.random.default_rng(5)
    worst = 0.0
    plain_worst = 0.0
    for trial in range(40):
        n = 32 * 8
        # magnitudes over several decades and both signs, as DoG gradients and blurred volumes
        a = (rng.standard_normal(n) * 10.0 ** rng.uniform(-6, 0, n)).astype(np.float32)
        b = (rng.standard_normal(n) * 10.0 ** rng.uniform(-2, 2, n)).astype(np.float32)
        exact = math.fsum(float(x) * float(y) for x, y in zip(a, b))
        scale = math.fsum(abs(float(x) * float(y)) for x, y in zip(a, b))
        got = warp_dot(a, b, 8)
        worst = max(worst, abs(got - exact) / scale)
        plain = f32(0)
        for x, y in zip(a, b):
            plain = f32(plain + f32(x * y))
        plain_worst = max(plain_worst, abs(float(plain) - exact) / scale)
    assert worst < 2.0 ** -44, worst                 # about 2^-48 of the sum of magnitudes
    assert plain_worst > 2.0 ** -30, plain_worst     # a plain float32 sum is far coarser
