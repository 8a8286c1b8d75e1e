"""CPU: the numpy E4M3 emulation the FP8-B parity tests rest on, checked
against the format itself: every finite E4M3 value (built here from its
bit fields) rounds to itself, every midpoint of two neighbours rounds to the
one with the even code, values just off a midpoint round to the nearer
neighbour, and magnitudes past 448 saturate. The column scales are powers of
two with absmax / scale in (224, 448]."""
from __future__ import annotations

import numpy as np

from fp8_emu import e4m3_round, fp8_scales


def e4m3_table():
    """(value, code) of the positive finite E4M3 numbers: exponent bias 7,
    3 mantissa bits, subnormals at exponent field 0, S.1111.111 is NaN."""
    out = []
    for e in range(16):
        for m in range(8):
            if e == 15 and m == 7:
                continue
            v = (m / 8.0) * 2.0 ** -6 if e == 0 else (1.0 + m / 8.0) * 2.0 ** (e - 7)
            out.append((v, e * 8 + m))
    return out


def test_table_is_the_format():
    t = e4m3_table()
    vals = [v for v, _ in t]
    assert len(t) == 127 and vals == sorted(vals)
    assert vals[-1] == 448.0 and vals[1] == 2.0 ** -9 and 2.0 ** -6 in vals


def test_representable_values_are_fixed_points():
    v = np.array([x for x, _ in e4m3_table()], np.float32)
    assert np.array_equal(e4m3_round(v), v)
    assert np.array_equal(e4m3_round(-v), -v)


def test_midpoints_round_to_even_codes_and_neighbours_to_nearest():
    t = e4m3_table()
    for (lo, clo), (hi, chi) in zip(t[:-1], t[1:]):
        mid = np.float32((lo + hi) / 2)
        if float(mid) != (lo + hi) / 2:
            continue  # midpoint not exact in FP32 (does not happen in this range)
        want = lo if clo % 2 == 0 else hi
        assert float(e4m3_round(mid)) == want, (lo, hi)
        below = np.nextafter(mid, np.float32(-np.inf), dtype=np.float32)
        above = np.nextafter(mid, np.float32(np.inf), dtype=np.float32)
        assert float(e4m3_round(below)) == lo and float(e4m3_round(above)) == hi, (lo, hi)


def test_saturation_and_zero():
    x = np.array([448.0, 449.0, 463.9, 464.0, 1e6, 0.0, -0.0, -1e6], np.float32)
    assert e4m3_round(x).tolist() == [448.0, 448.0, 448.0, 448.0, 448.0, 0.0, 0.0, -448.0]


def test_column_scales_are_powers_of_two_with_absmax_in_range():
    rng = np.random.default_rng(3)
    B = rng.uniform(-1, 1, size=(64, 40)).astype(np.float32)
    B *= (10.0 ** rng.uniform(-6, 6, size=40)).astype(np.float32)
    B[:, 0] = 0.0
    B[0, 1] = 448.0
    s = fp8_scales(B)
    assert s[0] == 1.0 and s[1] == 1.0
    mant, _ = np.frexp(s)
    assert np.all(mant == 0.5)  # powers of two
    a = np.abs(B).max(axis=0)
    r = a[1:] / s[1:]
    assert np.all(r <= 448.0) and np.all(r > 224.0)
