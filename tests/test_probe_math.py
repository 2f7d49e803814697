"""The probe kernel's division-free snorm16 decode (div32767 in candela_gb300/csrc/rq_probe.cu):
Markstein's correction step q0 = f * y, r = f - q0 * 32767 (one FMA, exact), q = q0 + r * y with
y = RN(1/32767) = 0x1.0002p-15, evaluated here with exact rationals, equals the IEEE quotient
f / 32767 for every int16 numerator, so the kernel's unpackSnorm2x16 equals the restatement's."""
import struct
from fractions import Fraction

import numpy as np

Y_HEX = "0x1.0002p-15"


def _bits(x: np.float32) -> int:
    return struct.unpack("<I", struct.pack("<f", x))[0]


def _round_f32(x: Fraction) -> np.float32:
    """x correctly rounded to binary32, ties to even."""
    if x == 0:
        return np.float32(0.0)
    c = np.float32(float(x))
    best = None
    for cand in (np.nextafter(c, np.float32(-np.inf)), c, np.nextafter(c, np.float32(np.inf))):
        d = abs(Fraction(float(cand)) - x)
        if best is None or d < best[0] or (d == best[0] and _bits(cand) % 2 == 0):
            best = (d, cand)
    return best[1]


def test_reciprocal_constant_is_correctly_rounded():
    y = np.float32(float.fromhex(Y_HEX))
    assert Fraction(float(y)) == Fraction(float.fromhex(Y_HEX))
    assert y == _round_f32(Fraction(1, 32767))


def test_markstein_quotient_equals_ieee_division_for_every_int16():
    y = Fraction(float.fromhex(Y_HEX))
    mismatches = []
    for f in range(-32768, 32768):
        q0 = _round_f32(f * y)
        r = f - Fraction(float(q0)) * 32767
        assert Fraction(float(np.float32(float(r)))) == r      # the FMA residual is exact
        q = _round_f32(r * y + Fraction(float(q0)))
        if q != np.float32(f) / np.float32(32767.0):
            mismatches.append(f)
    assert not mismatches, mismatches[:10]


def _ufloat_values(mbits):
    """Every finite value of an unsigned float with a 5-bit exponent (bias 15) and mbits mantissa
    bits, in code order (GL_R11F_G11F_B10F channels: 6 bits for R and G, 5 for B)."""
    vals = []
    for e in range(31):
        for m in range(1 << mbits):
            vals.append(Fraction(m, 1 << mbits) * Fraction(2) ** -14 if e == 0
                        else (1 + Fraction(m, 1 << mbits)) * Fraction(2) ** (e - 15))
    return vals


def test_r11g11b10_rounding_matches_an_exact_model():
    """The restatement's r11f_g11f_b10f rounding (which the probe kernel's equals bit for bit, by
    the GPU probe tests) against an exact model of the format: the closest finite value, ties to
    the even code; negative values and -inf to 0; above the largest finite value to it; +inf and
    NaN kept.  Checked at every code, every midpoint between neighbouring codes and 20,000 random
    values per channel width."""
    from oracle import oracle as O
    rng = np.random.default_rng(5)
    for mbits in (6, 5):
        vals = _ufloat_values(mbits)
        top = vals[-1]

        def model(x):
            if x <= 0:
                return Fraction(0)
            if x >= top:
                return top
            lo, hi = 0, len(vals) - 1
            while hi - lo > 1:
                mid = (lo + hi) // 2
                if vals[mid] <= x:
                    lo = mid
                else:
                    hi = mid
            dl, dh = x - vals[lo], vals[hi] - x
            if dl < dh or (dl == dh and lo % 2 == 0):
                return vals[lo]
            return vals[hi]

        xs = [float(v) for v in vals]
        xs += [float((a + b) / 2) for a, b in zip(vals[:-1], vals[1:])]
        xs += list(np.float32(10.0) ** rng.uniform(-9, 5.2, 20_000))
        for x in xs:
            x32 = np.float32(x)
            got = O.small_ufloat(float(x32), mbits)
            assert Fraction(float(got)) == model(Fraction(float(x32))), (mbits, float(x32), got)
        assert O.small_ufloat(-1.0, mbits) == 0.0 and O.small_ufloat(float("-inf"), mbits) == 0.0
        assert O.small_ufloat(float("inf"), mbits) == float("inf")
        assert np.isnan(O.small_ufloat(float("nan"), mbits))
        assert O.small_ufloat(1e30, mbits) == float(top)
