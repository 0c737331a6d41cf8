"""The bounding kernel's two decisions taken without a division, checked on
random IEEE doubles against the divisions they replace (CPU).

In the cell loop of the bounding (plain_bound.cu, advectionTemplates.C:
245-347) two tests are decided on proved bounds:

* ``maxExtra / V > aTol`` on the bits of maxExtra against aTol V (1 +- 2^-40);
* the loop test ``|alphaOvershoot(alpha1New)| < aTol`` of the next iteration
  from a1 = (num1 - nf2 g) rden with g = (1/V) rDeltaT, rden = 1/den, when
  a1 lies in (-aTol/2, 1 + aTol/2) and exp(max(|num1|, |t2|)) + exp(rden)
  <= 2045 (biased exponents).
"""
import random
import struct

K_ATOL = 100.0 * 1.0e-15


def _bits(x):
    return struct.unpack("<q", struct.pack("<d", x))[0]


def _exp(x):
    return (_bits(x) >> 52) & 0x7FF


def _overshoot(a):
    p = 1.0 if a - 1.0 >= 0 else 0.0
    n = 1.0 if a <= 0 else 0.0
    return p * (a - 1.0) + n * a


def test_certified_loop_test_never_disagrees_with_the_division():
    rng = random.Random(1)
    certified = 0
    for _ in range(100000):
        rD = 10 ** rng.uniform(-2, 8)
        V = 10 ** rng.uniform(-12, 2)
        Sp = 0.0 if rng.random() < 0.7 else -rng.uniform(0, 10) * rD
        den = rD - Sp
        target = rng.choice([1.0, 0.0, 1.0 + rng.uniform(-1e-13, 1e-13), rng.uniform(-1e-13, 1e-13),
                             rng.uniform(-0.5, 1.5)])
        nf2 = rng.uniform(-1, 1) * V * 10 ** rng.uniform(-6, 1)
        num1 = target * den + nf2 / V * rD * (1 + rng.uniform(-1e-15, 1e-15))
        g = (1.0 / V) * rD
        rden = 1.0 / den
        t2 = nf2 * g
        a1 = (num1 - t2) * rden
        in_window = (_bits(a1) >= 0 and a1 < 1.0 + 0.5 * K_ATOL) or (_bits(a1) < 0 and -a1 < 0.5 * K_ATOL)
        if in_window and max(_exp(num1), _exp(t2)) + _exp(rden) <= 2045:
            certified += 1
            num = num1 - nf2 / V * rD
            assert abs(_overshoot(num / den)) < K_ATOL
    assert certified > 50000


def test_tolerance_band_never_disagrees_with_the_division():
    rng = random.Random(2)
    for _ in range(100000):
        V = 10 ** rng.uniform(-300, 10)
        t = K_ATOL * V
        lo, hi = t * (1.0 - 2.0 ** -40), t * (1.0 + 2.0 ** -40)
        if rng.random() < 0.8:
            me = t * (1 + rng.choice([0, 1, -1]) * 2.0 ** rng.uniform(-60, -30))
        else:
            me = rng.uniform(0, 2) * t
        exact = me / V > K_ATOL
        if me > hi:
            assert exact
        if me < lo:
            assert not exact
