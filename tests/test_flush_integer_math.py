"""The integer arithmetic of the tensor-core basis flush (csrc/flush_tc.cu),
restated with Python integers and checked exactly on the CPU.

- biased62 and digit<S>: an FP64 value v with |v| < 2^scale becomes
  q = trunc(v 2^(62 - scale)) plus DIGIT_BIAS, and its nine 7-bit fields are
  balanced digits in [-64, 64] with sum_s d_s 2^(56 - 7 s) = q, exact in BF16.
- The products: a diagonal sum D_d of (d + 1) digit pairs over K = 64 slots
  stays below 2^22 in magnitude, so FP32 accumulation is exact and the
  1.5 2^23 bias trick recovers it from the FP32 bits.
- diag_sum: from the nine biased FP32 bit patterns, floor(T / 2^12) of
  T = sum_d D_d 2^(7 (8 - d)) in 64-bit modular arithmetic.
- join_t: T 2^k rounded to FP64 with at most 0.5 ulp error.
"""
import math
import random
import struct
from fractions import Fraction

M64 = (1 << 64) - 1
M32 = (1 << 32) - 1
NDIG = 9
TC_K = 64
DIGIT_BIAS = 0x4081020408102040
MAGIC_BITS = 0x4B400000
HI_BIAS = MAGIC_BITS * 2113665
MID_BIAS = MAGIC_BITS * 66052
T_BIAS = ((HI_BIAS << 23) + MID_BIAS) & M64


def _bits(v: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", v))[0]


def _double(b: int) -> float:
    return struct.unpack("<d", struct.pack("<Q", b & M64))[0]


def exp_of_bits(bits: int) -> int:
    eb = (bits >> 52) & 0x7FF
    frac = bits & ((1 << 52) - 1)
    return eb - 1022 if eb else frac.bit_length() - 1074


def biased62(bits: int, scale: int) -> int:
    eb = (bits >> 52) & 0x7FF
    frac = bits & ((1 << 52) - 1)
    m = (frac | (1 << 52)) if eb else frac
    r = 1023 + scale - (eb if eb else 1)
    q = (((m << 10) & M64) >> r) if r < 64 else 0
    sg = M64 if bits >> 63 else 0
    q = ((q ^ sg) - sg) & M64
    return (q + DIGIT_BIAS) & M64


def digit(u: int, s: int) -> int:
    e = (u >> 56) if s == 0 else (u >> (56 - 7 * s)) & 127
    return e - 64


def diag_sum(bits9) -> int:
    def madw(a, b, c):
        return (a * b + c) & M64

    b = bits9
    h = madw(b[0], 1 << 21, madw(b[1], 1 << 14, madw(b[2], 1 << 7, b[3])))
    mid = madw(b[4], 1 << 16, madw(b[5], 1 << 9, (b[6] << 2) & M64))
    lo = (b[7] * 128 + b[8] - MAGIC_BITS * 129) & M32
    lo = lo - (1 << 32) if lo >> 31 else lo  # (int)
    t = (((h << 23) & M64) + mid - T_BIAS + ((lo >> 12) & M64)) & M64
    return t - (1 << 64) if t >> 63 else t


def join_t(t: int, k: int) -> float:
    sg = t < 0
    a = -t if sg else t
    if a == 0:
        return 0.0
    z = 64 - a.bit_length()
    w = (a << z) & M64
    mant = (w >> 11) + ((w >> 10) & 1)
    ebm1 = 63 - z + k + 1022
    assert 0 <= ebm1 <= 2044
    return _double(((ebm1 << 52) + mant) | (int(sg) << 63))


def _random_double(rng: random.Random, lo_exp: int, hi_exp: int) -> float:
    return rng.choice((-1.0, 1.0)) * math.ldexp(rng.random() + 0.5, rng.randint(lo_exp, hi_exp))


def test_digit_split_is_exact_and_balanced():
    rng = random.Random(1)
    cases = [(math.ldexp(1.0, 9) - math.ldexp(1.0, -43), 9), (-math.ldexp(1.0, 9) + math.ldexp(1.0, -43), 9),
             (math.ldexp(1.0, -1074), 0), (-5e-324, -1000), (0.0, 3)]
    for _ in range(20000):
        v = _random_double(rng, -60, 60)
        scale = exp_of_bits(_bits(v)) + rng.choice((0, 0, 1, 3, 20, 61, 70))
        cases.append((v, scale))
    for v, scale in cases:
        assert abs(v) < 2.0 ** scale
        u = biased62(_bits(v), scale)
        q = int(Fraction(v) * Fraction(2) ** (62 - scale))  # truncation toward zero
        ds = [digit(u, s) for s in range(NDIG)]
        assert sum(d << (56 - 7 * s) if d >= 0 else -((-d) << (56 - 7 * s)) for s, d in enumerate(ds)) == q
        assert all(-64 <= d <= 64 for d in ds), (v, scale, ds)


def test_diagonal_sums_are_exact_in_fp32():
    # |digit| <= 64: a product is at most 2^12, diagonal d holds d + 1 digit
    # pairs over K slots; below 2^22, the range of the FP32 bias trick
    worst = max((d + 1) for d in range(NDIG)) * TC_K * 64 * 64
    assert worst < 2 ** 22
    magic = struct.unpack("<f", struct.pack("<I", MAGIC_BITS))[0]
    for d in (-worst, -1, 0, 1, worst):
        f = struct.unpack("<f", struct.pack("<f", float(d) + magic))[0]
        assert struct.unpack("<I", struct.pack("<f", f))[0] == MAGIC_BITS + d


def test_diag_sum_is_floor_of_exact_total():
    rng = random.Random(2)
    bound = [(d + 1) * TC_K * 64 * 64 for d in range(NDIG)]
    cases = [[b for b in bound], [-b for b in bound], [0] * NDIG, [rng.choice((-1, 1)) for _ in range(NDIG)]]
    for _ in range(50000):
        cases.append([rng.randint(-b, b) for b in bound])
    for ds in cases:
        total = sum(d << (7 * (8 - i)) if d >= 0 else -((-d) << (7 * (8 - i))) for i, d in enumerate(ds))
        got = diag_sum([MAGIC_BITS + d for d in ds])
        assert got == total >> 12  # floor division by 2^12


def test_join_rounds_to_half_an_ulp():
    rng = random.Random(3)
    cases = [1, -1, (1 << 63) - 1, -((1 << 63) - 1), (1 << 53) + 1, (1 << 54) + 2, (1 << 55) + 7]
    for _ in range(50000):
        cases.append(rng.choice((-1, 1)) * rng.getrandbits(rng.randint(1, 63)))
    for t in cases:
        for k in (-1000, -56, 0, 40):
            got = join_t(t, k)
            exact = Fraction(t) * Fraction(2) ** k
            ulp = Fraction(math.ulp(got))
            assert abs(Fraction(got) - exact) <= ulp / 2, (t, k)
