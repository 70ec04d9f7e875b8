"""The table-driven log(1 + u) of the NFW halo (potentials.cuh, log1p_pos):
the committed table matches its generator, and the algorithm, replayed here
with exactly rounded fused multiply-adds, stays within one unit in the last
place of a 40-digit reference over the radii the potentials meet."""

from __future__ import annotations

import math
import re
import struct
import sys
from decimal import Decimal, getcontext
from fractions import Fraction
from pathlib import Path

import numpy as np

CSRC = Path(__file__).resolve().parents[1] / "galax_gb300" / "csrc"
sys.path.insert(0, str(CSRC))
import gen_log_table  # noqa: E402


def _d2l(x):
    return struct.unpack("<q", struct.pack("<d", x))[0]


def _l2d(i):
    return struct.unpack("<d", struct.pack("<q", i))[0]


def _fma(a, b, c):
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def _log1p_pos(u, T):
    x = 1.0 + u
    c = u - (x - 1.0) if u <= 1.0 else 1.0 - (x - u)
    bits = _d2l(x)
    k = (bits >> 52) - 1023
    mant = bits & 0x000FFFFFFFFFFFFF
    m = _l2d(mant | 0x3FF0000000000000)
    j = (mant + (1 << 44)) >> 45
    F = 1.0 + j * 0.0078125
    r = _fma(c, _l2d((1023 - k) << 52), m - F) * T[j][0]
    q = _fma(0.14285714285714285, r, -0.16666666666666666)
    for cc in (0.2, -0.25, 0.3333333333333333, -0.5):
        q = _fma(q, r, cc)
    p = _fma(r * r, q, r)
    hi = _fma(float(k), 0.6931471805599453, T[j][1])
    lo = _fma(float(k), 2.3190468138462996e-17, T[j][2])
    return hi + (lo + p)


def test_committed_table_matches_generator():
    text = (CSRC / "log_table.h").read_text()
    rows = re.findall(r"\{(-?0x[^,]+), (-?0x[^,]+), (-?0x[^}]+)\}", text)
    got = [tuple(float.fromhex(v) for v in r) for r in rows]
    assert got == gen_log_table.table()


def test_log1p_within_one_ulp():
    T = gen_log_table.table()
    getcontext().prec = 40
    rng = np.random.default_rng(0)
    us = np.concatenate([np.exp(rng.uniform(np.log(1e-12), np.log(1e4), 2000)),
                         [1e-300, 0.5, 1.0, 2.0, 1 - 2**-53, 3.0, 255 / 256, 1 / 256, 1023.9]])
    assert _log1p_pos(0.0, T) == 0.0
    for u in us:
        ud = Decimal(float(u))
        ref = (ud + 1).ln() if u > 1e-8 else ud - ud * ud / 2 + ud**3 / 3
        err = abs(Decimal(_log1p_pos(float(u), T)) - ref) / Decimal(math.ulp(float(ref)))
        assert err <= 1.0, (u, float(err))
