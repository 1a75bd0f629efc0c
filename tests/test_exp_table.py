"""The 2^(j/64) table of the varifold's FP64 exponential (csrc/sa_varifold.cu
c_exp2_64) against 60-digit decimal arithmetic: every entry is the double
nearest to 2^(j/64)."""
import os
import re
from decimal import Decimal, getcontext

SRC = os.path.join(os.path.dirname(__file__), "..", "shape_atrophy_gb300", "csrc", "sa_varifold.cu")


def test_exp2_table_correctly_rounded():
    src = open(SRC).read()
    body = re.search(r"c_exp2_64\[64\]\s*=\s*\{(.*?)\};", src, re.S).group(1)
    vals = [float.fromhex(t) for t in re.findall(r"0x[0-9a-fA-F.]+p[+-]\d+", body)]
    assert len(vals) == 64
    getcontext().prec = 60
    for j, v in enumerate(vals):
        exact = Decimal(2) ** (Decimal(j) / 64)
        assert v == float(exact), j                                # float(Decimal) rounds to nearest
        assert abs(Decimal(v) - exact) <= abs(Decimal(v) * Decimal(2) ** -53)


def test_ln2_split_constants():
    src = open(SRC).read()
    getcontext().prec = 60
    ln2_64 = Decimal(2).ln() / 64
    hi = float.fromhex(re.search(r"fma\(-Nd, (0x[0-9a-f.]+p-7), x\)", src).group(1))
    lo = float.fromhex(re.search(r"fma\(-Nd, (0x[0-9a-f.]+p-62), r\)", src).group(1))
    assert hi == float(ln2_64) and lo == float(ln2_64 - Decimal(hi))
    inv = float.fromhex(re.search(r"fma\(x, (0x[0-9a-f.]+p\+6), 0x1.8p52\)", src).group(1))
    assert inv == float(64 / Decimal(2).ln())
