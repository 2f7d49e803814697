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
