"""Oracle restatement of the scaling techniques' automatic rescaling — TEST INFRASTRUCTURE ONLY.

Follows the reference's CPU-side logic step for step on oracle ciphertexts (numpy u64[2][t][N] plus the noise
degree and the scaling factor):
  * scaling tables per technique (what RawParams carries from OpenFHE's CryptoParametersCKKSRNS, read by
    src/CKKS/openfhe-interface/RawCiphertext.cu:260-272, indexed here like FIDESlib by towers - 1);
  * ContextData::ElemForEvalMult (src/CKKS/Context.cu:366-458): a real constant encoded at sf[level];
  * Ciphertext::adjustScaleAndLevel / adjustForAddOrSub / adjustForMult (src/CKKS/Ciphertext.cpp:1376-1518) and the
    retry with the roles swapped in Ciphertext::add / sub / mult (:164-240, 458-477);
  * the FIXEDMANUAL tower cut of Ciphertext::add (:186-197).
Only tests/ use it, as the checker of the engine's fideslib_gb300/csrc/autoscale.cu.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

FIXEDMANUAL, FIXEDAUTO, FLEXIBLEAUTO, FLEXIBLEAUTOEXT = 0, 1, 2, 3


def scaling_tables(q: list[int], technique: int, default_scale: float = 0.0):
    """(sf, big, mrf) for Q primes q (nq entries each, index = towers - 1)."""
    nq = len(q)
    L = nq - 1
    mrf = [float(x) for x in q]
    if technique in (FIXEDMANUAL, FIXEDAUTO):
        d = default_scale if default_scale > 0 else math.ldexp(1.0, round(math.log2(float(q[L]))))
        sf = [d] * nq
    else:
        sf = [0.0] * nq
        if technique == FLEXIBLEAUTO:
            sf[L] = float(q[L])
            top = L
        else:
            sf[L] = float(q[L - 1]) if nq >= 2 else float(q[L])
            if L >= 1:
                sf[L - 1] = float(q[L - 1])
            top = L - 1
        for lv in range(top - 1, -1, -1):
            sf[lv] = sf[lv + 1] * sf[lv + 1] / float(q[lv + 1])
    big = [x * x for x in sf]
    if technique == FLEXIBLEAUTOEXT and nq >= 2:
        big[L] = sf[L] * sf[L - 1]
    return sf, big, mrf


def eval_mult_constants(q: list[int], sf: list[float], t: int, operand: float) -> list[int]:
    """Residues mod q_0..q_{t-1} of operand encoded at sf[t-1] (ElemForEvalMult with level_in = -1)."""
    scf = sf[t - 1]
    log_approx = 0
    res = abs(operand * scf)
    if res > 0:
        log_sf = int(math.ceil(math.log2(res)))
        log_approx = log_sf - min(log_sf, 125)
    approx = 2.0 ** log_approx
    large = int(operand / approx * scf + 0.5)  # truncation toward zero, like the reference's cast
    return [(large % qi) * pow(2, log_approx, qi) % qi for qi in q[:t]]


@dataclass
class Ct:
    data: np.ndarray  # u64[2][t][N]
    deg: int
    scale: float

    @property
    def t(self) -> int:
        return self.data.shape[1]


class Scaler:
    """The reference's operand alignment over an oracle context `orc` (oracle.Ctx)."""

    def __init__(self, orc, technique: int, sf, big, mrf, rlk=None):
        self.orc, self.tech = orc, technique
        self.sf, self.big, self.mrf = list(sf), list(big), list(mrf)
        self.q = [int(x) for x in orc.moduli[:orc.nq]]
        self.rlk = rlk

    # primitive steps
    def rescale(self, x: Ct) -> Ct:
        return Ct(self.orc.rescale(x.data), x.deg - 1, x.scale / self.mrf[x.t - 1])

    def drop(self, x: Ct, t: int) -> Ct:
        if t >= x.t:
            return x
        return Ct(np.ascontiguousarray(x.data[:, :t]), x.deg, x.scale)

    def mult_const(self, x: Ct, operand: float) -> Ct:
        k = eval_mult_constants(self.q, self.sf, x.t, operand)
        return Ct(self.orc.scalar_op(x.data, k, [0] * x.t), x.deg + 1, x.scale * self.sf[x.t - 1])

    # Ciphertext::adjustScaleAndLevel
    def scale_and_level(self, x: Ct, deg2: int, t2: int, scale2: float):
        l1, l2, d1 = x.t - 1, t2 - 1, x.deg
        sf, big, mrf = self.sf, self.big, self.mrf
        if l1 > l2:
            if d1 == 2:
                if deg2 == 2:
                    x = self.mult_const(x, scale2 * mrf[l2 + 1] / x.scale / sf[l1])
                    if x.t - 1 > l2 + 1:
                        x = self.drop(x, l2 + 2)
                    x.scale = big[l2] * mrf[l2 + 1]
                    x = self.rescale(x)
                    x.scale = scale2
                elif l1 - 1 == l2:
                    x = self.rescale(x)
                else:
                    x = self.mult_const(x, big[l2 + 1] / x.scale * mrf[l1] / sf[l1])
                    x.scale = big[x.t - 2] * mrf[l1]
                    x = self.rescale(x)
                    if x.t - 2 > l2:
                        x = self.drop(x, l2 + 2)
                    x.scale = big[x.t - 1]
                    x = self.rescale(x)
                    x.scale = scale2
            else:
                if deg2 == 2:
                    x = self.mult_const(x, scale2 / x.scale / sf[l1])
                    x = self.drop(x, l2 + 1)
                    x.scale = scale2
                else:
                    scf1, scf2, scf = x.scale, big[l2 + 1], sf[l1]
                    x = self.mult_const(x, scf2 / scf1 / scf)
                    if l1 - 1 > l2:
                        x = self.drop(x, l2 + 2)
                    x.scale *= scf2 / scf1 / scf
                    x = self.rescale(x)
                    x.scale = scale2
            return x, True
        if l1 < l2:
            return x, False
        if d1 < deg2:
            return self.mult_const(x, 1.0), True
        return x, not (deg2 < d1)

    # Ciphertext::adjustForAddOrSub
    def for_add(self, x: Ct, y: Ct):
        if self.tech in (FLEXIBLEAUTO, FLEXIBLEAUTOEXT):
            return self.scale_and_level(x, y.deg, y.t, y.scale)
        if (x.t - 1) - x.deg > (y.t - 1) - y.deg:
            if y.deg == 1 and x.deg == 2:
                x = self.rescale(x)
            elif y.deg == 2 and x.deg == 1:
                x = self.mult_const(x, 1.0)
            return x, True
        if y.deg == 1 and x.deg == 2:
            return self.rescale(x), True
        return x, not (x.deg == 1 and y.deg == 2)

    # Ciphertext::adjustForMult
    def for_mult(self, x: Ct, y: Ct):
        x, ok = self.for_add(x, y)
        if x.deg == 2:
            x = self.rescale(x)
        return x, ok and y.deg != 2

    def align(self, a: Ct, b: Ct, mult: bool):
        if self.tech != FIXEDMANUAL:
            f = self.for_mult if mult else self.for_add
            for _ in range(4):
                a, ok = f(a, b)
                if ok:
                    break
                b, ok_b = f(b, a)
                assert ok_b
        if a.t > b.t:
            a = self.drop(a, b.t)
        elif b.t > a.t:
            b = self.drop(b, a.t)
        return a, b

    # the ops
    def add(self, a: Ct, b: Ct, sub: bool = False) -> Ct:
        a, b = self.align(a, b, False)
        d = self.orc.sub(a.data, b.data) if sub else self.orc.add(a.data, b.data)
        return Ct(d, max(a.deg, b.deg), a.scale)

    def mult(self, a: Ct, b: Ct) -> Ct:
        a, b = self.align(a, b, True)
        return Ct(self.orc.mult(a.data, b.data, self.rlk), a.deg + b.deg, a.scale * b.scale)

    def square(self, a: Ct) -> Ct:
        if self.tech != FIXEDMANUAL and a.deg >= 2:
            a = self.rescale(a)
        return Ct(self.orc.mult(a.data, a.data, self.rlk), 2 * a.deg, a.scale * a.scale)
