"""Numerical model (CPU, numpy) of the operand splits of the harmonic moments
kernels: a moment M = sum_j w_j b_j over a unit of 1,024 points with each
product formed from FP16 (or TF32) value + remainder halves of both operands,
as the tensor-core kernels form it, against the FP64 sum.

FP16 split (hm_moments_jobs<FP16>, hm_moments_tc_jobs): the basis value times
2^11, its value half the FP32 value truncated to 11 significant bits, the
remainder rounded to FP16; the weight times 2^(14 - e) (2^e above the unit's
largest |w|), its value half rounded to FP16, the remainder rounded to FP16.
TF32 split (hm_moments_jobs<TF32>): the basis value truncated to 11
significant bits and its remainder truncated again by the MMA; the weight
rounded to TF32 and its remainder.  Both carry all four partial products; the
model sums them exactly (FP64), so it measures the operand splits alone.
"""
import numpy as np


def trunc_bits(x, keep):
    """FP32 values with their significand cut to `keep` bits (truncation)."""
    u = np.asarray(x, dtype=np.float32).view(np.uint32)
    mask = np.uint32((0xFFFFFFFF << (24 - keep)) & 0xFFFFFFFF)
    return (u & mask).view(np.float32)


def fp16_split_basis(b):
    v = (b * np.float32(2048.0)).astype(np.float32)
    hi = trunc_bits(v, 11)
    lo = (v - hi).astype(np.float32).astype(np.float16).astype(np.float64)
    return hi.astype(np.float64), lo, 2048.0


def fp16_split_weight(w):
    e = int(np.frexp(np.max(np.abs(w)))[1])
    sc = np.float32(2.0 ** (14 - e))
    v = (w * sc).astype(np.float32)
    hi = v.astype(np.float16).astype(np.float32)
    lo = (v - hi).astype(np.float32).astype(np.float16).astype(np.float64)
    return hi.astype(np.float64), lo, float(sc)


def tf32_split(x):
    v = np.asarray(x, dtype=np.float32)
    hi = trunc_bits(v, 11)
    lo = trunc_bits((v - hi).astype(np.float32), 11)
    return hi.astype(np.float64), lo.astype(np.float64)


def moment_errors(seed, n=1024):
    rng = np.random.default_rng(seed)
    # basis values: orthonormal Pbar_lm e^{-i m phi} components, |b| <= about 5, many small
    b = (rng.standard_normal(n) * np.exp(rng.uniform(-8, 1.5, n))).astype(np.float32)
    # weights w u^n: a unit's common weight times powers of u in [-1, 1]
    w = (0.0417 * rng.uniform(-1, 1, n) ** rng.integers(0, 6)).astype(np.float32)
    exact = np.sum(w.astype(np.float64) * b.astype(np.float64))
    scale = np.sum(np.abs(w.astype(np.float64) * b.astype(np.float64)))
    bh, bl, bs = fp16_split_basis(b)
    wh, wl, ws = fp16_split_weight(w)
    f16 = np.sum((bh + bl) * (wh + wl)) / (bs * ws)
    th, tl = tf32_split(b)
    uh, ul = tf32_split(w)
    tf32 = np.sum((th + tl) * (uh + ul))
    return abs(f16 - exact) / scale, abs(tf32 - exact) / scale


def test_fp16_split_is_as_accurate_as_tf32_split():
    worst16 = worst32 = 0.0
    for seed in range(40):
        e16, e32 = moment_errors(seed)
        worst16, worst32 = max(worst16, e16), max(worst32, e32)
    # relative to the sum of |products| (about 1.9e-8 and 7.7e-8 on these
    # seeds): the FP16 split, with both value halves rounded to nearest where
    # the TF32 path truncates its remainders, is the more accurate of the two
    assert worst16 < 5e-8
    assert worst32 < 2e-7
    assert worst16 <= worst32
