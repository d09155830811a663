"""Python restatement of the pieces of the J -> M transform that can be
checked in isolation — TEST INFRASTRUCTURE ONLY.

* ``antoine_shells`` / ``jt_basis``  the Antoine shell order and coupled
  basis (src/Neptune/bases/shells.c:72-130, src/Neptune/bases/jt_basis.c:70-101,
  130-166, 250-287), with the configuration count of the interaction file.
* ``cg_exact``  Clebsch-Gordan coefficients from the Racah formula in exact
  rational arithmetic (the square of the coefficient is rational), as the
  reference defines them through the 3j symbol
  (src/Neptune/clebsch_gordan/clebsch_gordan.c:31-42).  Arguments doubled.
* ``read_antoine``  the three Fortran records of an Antoine file
  (src/Neptune/input/read_2nf_antoine_format.c:131-236).
"""
import math
import struct
from fractions import Fraction

import numpy as np


def antoine_shells(emax):
    out = []
    for e in range(emax + 1):
        for l in range(e & 1, e + 1, 2):
            for j in range(abs(2 * l - 1), 2 * l + 2, 2):
                out.append((e, (e - l) // 2, l, j))
    return out


def jt_basis(emax1, emax2):
    """States (a, b, J, T, parity) in file order and the number of configurations."""
    sh = antoine_shells(emax1)
    states = []
    for idx in range(4 * (emax2 + 2)):
        parity, T, J = idx & 1, (idx >> 1) & 1, idx >> 2
        for a, sa in enumerate(sh):
            if 2 * sa[0] > emax2:
                break
            for b in range(a, len(sh)):
                sb = sh[b]
                if sa[0] + sb[0] > emax2:
                    break
                if not (sa[3] + sb[3] >= 2 * J and abs(sa[3] - sb[3]) <= 2 * J):
                    continue
                if (sa[2] + sb[2]) & 1 != parity:
                    continue
                if a == b and (J + T) % 2 == 0:
                    continue
                states.append((a, b, J, T, parity))
    nconf = 0
    for i, s in enumerate(states):
        k = i
        while k < len(states) and states[k][2:] == s[2:]:
            k += 1
        nconf += k - i
    return states, nconf


def _f(n):
    return math.factorial(n)


def three_j_squared_sign(j1, j2, j3, m1, m2, m3):
    """(sign, exact square) of the 3j symbol; doubled arguments."""
    if m1 + m2 + m3 != 0 or min(j1, j2, j3) < 0:
        return 0, Fraction(0)
    if abs(m1) > j1 or abs(m2) > j2 or abs(m3) > j3:
        return 0, Fraction(0)
    if (j1 + m1) % 2 or (j2 + m2) % 2 or (j3 + m3) % 2 or (j1 + j2 + j3) % 2:
        return 0, Fraction(0)
    a, b, c = j1 + j2 - j3, j1 - j2 + j3, -j1 + j2 + j3
    if min(a, b, c) < 0:
        return 0, Fraction(0)
    delta = Fraction(_f(a // 2) * _f(b // 2) * _f(c // 2), _f((j1 + j2 + j3) // 2 + 1))
    pre = delta * _f((j1 + m1) // 2) * _f((j1 - m1) // 2) * _f((j2 + m2) // 2) * _f((j2 - m2) // 2) \
        * _f((j3 + m3) // 2) * _f((j3 - m3) // 2)
    s = Fraction(0)
    for k in range(0, 200):
        x = [2 * k, j3 - j2 + 2 * k + m1, j3 - j1 + 2 * k - m2, j1 + j2 - j3 - 2 * k, j1 - 2 * k - m1, j2 - 2 * k + m2]
        if x[3] < 0 or x[4] < 0 or x[5] < 0:
            break
        if min(x) < 0:
            continue
        d = 1
        for v in x:
            d *= _f(v // 2)
        s += Fraction((-1) ** k, d)
    if s == 0:
        return 0, Fraction(0)
    sign = (1 if s > 0 else -1) * (-1 if ((j1 - j2 - m3) // 2) % 2 else 1)
    return sign, pre * s * s


def cg_exact(j1, j2, j3, m1, m2, m3):
    """<j1 m1 j2 m2 | j3 m3> as a float rounded from the exact value."""
    sign, sq = three_j_squared_sign(j1, j2, j3, m1, m2, -m3)
    if sign == 0:
        return 0.0
    sq = sq * (j3 + 1)
    ph = ((j1 - j2 + m3) // 2) % 2
    v = math.sqrt(sq.numerator) / math.sqrt(sq.denominator)
    return -sign * v if ph else sign * v


def read_antoine(path):
    """(title bytes, ncol, hw, nrow, float32 array [nrow, ncol])."""
    raw = open(path, "rb").read()
    recs, pos = [], 0
    for _ in range(3):
        (n,) = struct.unpack_from("<i", raw, pos)
        recs.append(raw[pos + 4:pos + 4 + n])
        (n2,) = struct.unpack_from("<i", raw, pos + 4 + n)
        assert n == n2, "not a Fortran record"
        pos += 8 + n
    ncol, hw, nrow = struct.unpack("<ifi", recs[1])
    data = np.frombuffer(recs[2], dtype=np.float32).reshape(nrow, ncol)
    return recs[0], ncol, hw, nrow, data
