"""The float-pair arithmetic the calibration's node-radiosity sweeps use in place of FP64 (vt_calib.cu: df_split,
df_mac): x held as (hi, lo) = (float(x), float(x - hi)); each product F_j x_j formed exactly for hi by an FMA plus the
lo part's product, summed by two-sum and renormalised. Restated here step by step in float32 (an FMA of two float32
factors is exact in float64 before its single rounding) and checked against exact rational sums: a 4096-term row
is good to about 1e-13 relative, where float32 alone gives about 1e-7."""
from fractions import Fraction

import numpy as np

f32 = np.float32


def _split(x):
    h = f32(x)
    return h, f32(x - float(h))


def _fma(a, b, c):
    # float32 FMA: the float64 product of two float32 values is exact; one rounding of the sum to float32
    return f32(float(a) * float(b) + float(c))


def _dot(F, B):
    sh, sl = f32(0), f32(0)
    for f, b in zip(F, B):
        bh, bl = _split(b)
        p = f32(f * bh)
        e = _fma(f, bl, _fma(f, bh, -p))
        t = f32(sh + p)
        v = f32(t - sh)
        lo = f32(sl + f32(f32(f32(sh - f32(t - v)) + f32(p - v)) + e))
        sh = f32(t + lo)
        sl = f32(lo - f32(sh - t))
    return float(sh) + float(sl)


def test_float_pair_row_sum_accuracy():
    rng = np.random.default_rng(1)
    worst, worst32 = 0.0, 0.0
    for _ in range(6):
        n = 4096
        F = (rng.random(n) * 1e-3).astype(np.float32)
        B = rng.random(n) * 50.0 + 1.0
        exact = sum(Fraction(float(a)) * Fraction(float(b)) for a, b in zip(F, B))
        worst = max(worst, float(abs(Fraction(_dot(F, B)) - exact) / exact))
        s32 = f32(0)
        for a, b in zip(F, B):
            s32 = f32(s32 + f32(a * f32(b)))
        worst32 = max(worst32, float(abs(Fraction(float(s32)) - exact) / exact))
    print(f"\nfloat-pair 4096-term sums: worst relative error {worst:.2e} (float32 alone: {worst32:.2e})")
    assert worst < 5e-13 and worst32 > 1e-9
