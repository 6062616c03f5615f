"""CPU checks of the 2-D lid kernel's quotients by constants.

k_lid2d.cu forms x/d for d = 6, 9, 12, 18, 36 as RN(x*h + RN(x*l)) (one
multiply, one fused multiply-add) instead of a division.  Here the constants
are read from the source, checked to be h = 1/d rounded down and l = 1/d - h
rounded to nearest, and the formula -- with the fused multiply-add evaluated
exactly in rational arithmetic and rounded once, as the hardware does -- is
compared with IEEE division on random normal inputs and on inputs built to
put x/d next to a rounding midpoint."""
import math
import os
import random
import re
import struct
from fractions import Fraction as Fr

SRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                   "mglc_gb300", "csrc", "k_lid2d.cu")


def _pairs():
    s = open(SRC).read()
    out = {}
    for d, h, l in re.findall(r"RH(\d+) = (0x[0-9a-fp.+-]+), RL\1 = (0x[0-9a-fp.+-]+);", s):
        out[int(d)] = (float.fromhex(h), float.fromhex(l))
    return out


def _bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def test_constants_are_the_rounded_down_two_term_reciprocals():
    pairs = _pairs()
    assert sorted(pairs) == [6, 9, 12, 18, 36]
    for d, (h, l) in pairs.items():
        z = Fr(1, d)
        assert Fr(h) < z and math.nextafter(h, 1.0) > z  # h = RD(1/d)
        assert l == float(z - Fr(h)) and l > 0          # l = RN(1/d - h)


def test_fused_quotient_equals_division():
    rng = random.Random(11)
    for d, (h, l) in _pairs().items():
        for k in range(4000):
            if k % 3 == 0:
                x = rng.uniform(-1.0, 1.0) * 2.0 ** rng.randint(-200, 60)
            elif k % 3 == 1:
                x = struct.unpack("<d", struct.pack("<Q", rng.getrandbits(64)))[0]
                e = (_bits(x) >> 52) & 0x7FF
                if e < 123 or e == 2047:
                    continue
            else:  # x/d next to a midpoint between two doubles
                q = rng.uniform(0.5, 1.0) * 2.0 ** rng.randint(-60, 10)
                x = float((Fr(q) + Fr(math.ulp(q)) / 2) * d)
                x = math.nextafter(x, rng.choice([-math.inf, math.inf])) if k % 2 else x
            fast = float(Fr(x) * Fr(h) + Fr(x * l))
            assert _bits(fast) == _bits(x / d), (d, x.hex())
