"""The 2^(j/256) table of the varifold's FP64 exponential (csrc/sa_varifold.cu
c_exp2_256) against 60-digit decimal arithmetic: every entry is the double
nearest to 2^(j/256); the argument-reduction constants; and the exponential
and square-root algorithms emulated operation by operation in exact
arithmetic."""
import os
import re
from decimal import Decimal, getcontext

SRC = os.path.join(os.path.dirname(__file__), "..", "shape_atrophy_gb300", "csrc", "sa_varifold.cu")


def test_exp2_table_correctly_rounded():
    src = open(SRC).read()
    body = re.search(r"c_exp2_256\[256\]\s*=\s*\{(.*?)\};", src, re.S).group(1)
    vals = [float.fromhex(t) for t in re.findall(r"0x[0-9a-fA-F.]+p[+-]\d+", body)]
    assert len(vals) == 256
    getcontext().prec = 60
    for j, v in enumerate(vals):
        exact = Decimal(2) ** (Decimal(j) / 256)
        assert v == float(exact), j                                # float(Decimal) rounds to nearest
        assert abs(Decimal(v) - exact) <= abs(Decimal(v) * Decimal(2) ** -53)


def test_ln2_split_constants():
    src = open(SRC).read()
    getcontext().prec = 60
    ln2_256 = Decimal(2).ln() / 256
    hi = float.fromhex(re.search(r"fma\(-Nd, (0x[0-9a-f.]+p-9), x\)", src).group(1))
    lo = float.fromhex(re.search(r"fma\(-Nd, (0x[0-9a-f.]+p-64), r\)", src).group(1))
    assert hi == float(ln2_256) and lo == float(ln2_256 - Decimal(hi))
    inv = float.fromhex(re.search(r"fma\(x, (0x[0-9a-f.]+p\+8), 0x1.8p52\)", src).group(1))
    assert inv == float(256 / Decimal(2).ln())


# --- the device algorithms emulated with exact fused multiply-adds ----------------------------------------

def _fma(a, b, c):
    from fractions import Fraction
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def _ulp_err(y, exact):
    import math
    return abs(Decimal(y) - exact) / Decimal(math.ulp(float(exact)))


def _exp_tab(x, tab, inv, l1, l2):
    """exp_tab of csrc/sa_varifold.cu, operation by operation."""
    import math
    magic = float.fromhex("0x1.8p52")
    t = _fma(x, inv, magic)
    nd = t - magic
    n = int(nd)
    r = _fma(-nd, l1, x)
    r = _fma(-nd, l2, r)
    p = _fma(r, 1.0 / 24.0, 1.0 / 6.0)
    p = _fma(p, r, 0.5)
    p = _fma(p, r, 1.0)
    p = p * r
    s = tab[n & 255]
    y = _fma(s, p, s)
    return math.ldexp(y, n >> 8)


def test_exp_algorithm_within_1_5_ulp_in_exact_arithmetic():
    """Table rounding (1/2 ulp of 2^(j/256)) plus the final rounding: about 1 ulp."""
    import numpy as np
    src = open(SRC).read()
    body = re.search(r"c_exp2_256\[256\]\s*=\s*\{(.*?)\};", src, re.S).group(1)
    tab = [float.fromhex(t) for t in re.findall(r"0x[0-9a-fA-F.]+p[+-]\d+", body)]
    l1 = float.fromhex(re.search(r"fma\(-Nd, (0x[0-9a-f.]+p-9), x\)", src).group(1))
    l2 = float.fromhex(re.search(r"fma\(-Nd, (0x[0-9a-f.]+p-64), r\)", src).group(1))
    inv = float.fromhex(re.search(r"fma\(x, (0x[0-9a-f.]+p\+8), 0x1.8p52\)", src).group(1))
    rng = np.random.default_rng(11)
    xs = list(-rng.uniform(0.0, 40.0, 1500)) + list(rng.uniform(-699.0, 699.0, 500))
    xs += [k * math_ln2_256() + d for k in range(-800, 800, 29) for d in (0.0, math_ln2_256() / 2)]
    getcontext().prec = 50
    worst = max(_ulp_err(_exp_tab(float(x), tab, inv, l1, l2), Decimal(float(x)).exp()) for x in xs)
    assert worst <= 1.5, worst


def math_ln2_256():
    import math
    return math.log(2.0) / 256


def _sqrt_nr(a, seed):
    """sqrt_nr of csrc/sa_varifold.cu from a given FP32 reciprocal-square-root seed."""
    y = float(seed)
    h = 0.5 * y
    s = a * y
    s = _fma(_fma(-s, s, a), h, s)
    s = _fma(_fma(-s, s, a), h, s)
    return s


def test_sqrt_algorithm_correct_to_one_ulp_from_a_perturbed_fp32_seed():
    import math
    import numpy as np
    rng = np.random.default_rng(12)
    xs = list(rng.uniform(0.0, 4.0, 800)) + list(10.0 ** rng.uniform(-28.0, 28.0, 800))
    getcontext().prec = 50
    for a in xs:
        a = float(a)
        if a == 0.0:
            continue
        y32 = np.float32(1.0) / np.sqrt(np.float32(a))
        for k in (-4, 0, 4):                   # the hardware reciprocal square root is within a few FP32 ulps
            seed = y32 + np.float32(k) * np.spacing(y32)
            s = _sqrt_nr(a, seed)
            exact = Decimal(a).sqrt()
            assert _ulp_err(s, exact) <= 1, (a, k)
            assert abs(s - math.sqrt(a)) <= math.ulp(math.sqrt(a))
