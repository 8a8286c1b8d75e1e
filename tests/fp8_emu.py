"""Numpy emulation of the FP8-B form's quantization (test infrastructure):
per-column power-of-two scales as the library computes them, and FP32 ->
FP8 E4M3 rounding (nearest even, saturating at 448)."""
from __future__ import annotations

import numpy as np


def fp8_scales(B):
    """Per-column power-of-two scales as the library computes them: the
    smallest 2^e with absmax / 2^e <= 448, from the FP32 quotient absmax / 448."""
    a = np.abs(np.asarray(B, np.float32)).max(axis=0)
    r = (a / np.float32(448.0)).astype(np.float32)
    mant, e = np.frexp(r)
    e = np.where(mant == 0.5, e - 1, e)
    s = np.ldexp(np.float32(1.0), e).astype(np.float32)
    return np.where((a > 0) & np.isfinite(a), s, np.float32(1.0)).astype(np.float32)


def e4m3_round(y):
    """FP32 -> FP8 E4M3, round to nearest even, saturating at 448 (finite inputs)."""
    y = np.asarray(y, np.float64)
    a = np.abs(y)
    e = np.floor(np.log2(np.where(a > 0, a, 1.0)))
    step = np.ldexp(1.0, (np.maximum(e, -6) - 3).astype(np.int64))  # 3 mantissa bits; subnormal step 2^-9
    q = np.minimum(np.round(a / step) * step, 448.0)
    return (np.sign(y) * q).astype(np.float32)
