"""Oracle replay of composite engine ops (test helper, not a test module).

Mirrors the engine's metadata rules: a rescale divides the scale by the dropped prime, a product multiplies the
scales, scalar constants are round(v * scale) residues (round half to even, as the engine's nearbyint)."""
import numpy as np


def double_residue(v: float, q: int) -> int:
    a = round(abs(v))
    r = a % q
    return (q - r) % q if v < 0 else r


class Sim:
    """Oracle replay with the engine's metadata rules (scale after rescale = scale / dropped prime)."""

    def __init__(self, orc, mods, rlk):
        self.orc, self.mods, self.rlk = orc, mods, rlk

    def t(self, a):
        return a[0].shape[1]

    def mult(self, a, b):
        return (self.orc.mult(a[0], b[0], self.rlk), a[1] * b[1])

    def rescale(self, a):
        return (self.orc.rescale(a[0]), a[1] / self.mods[self.t(a) - 1])

    def mult_int(self, a, k):
        return (self.orc.scalar_op(a[0], [k % q for q in self.mods[:self.t(a)]], [0] * self.t(a)), a[1])

    def add_scalar(self, a, v):
        add = [double_residue(v * a[1], q) for q in self.mods[:self.t(a)]]
        return (self.orc.scalar_op(a[0], [1] * self.t(a), add), a[1])

    def mult_scalar(self, a, v, cs):
        mul = [double_residue(v * cs, q) for q in self.mods[:self.t(a)]]
        return (self.orc.scalar_op(a[0], mul, [0] * self.t(a)), a[1] * cs)

    def drop(self, a, t):
        return (np.ascontiguousarray(a[0][:, :t]), a[1]) if self.t(a) != t else a

    def add(self, a, b):
        return (self.orc.add(a[0], b[0]), a[1])

    def sub(self, a, b):
        return (self.orc.sub(a[0], b[0]), a[1])

    def chebyshev(self, x, c, lo, hi, cs):
        d = len(c) - 1
        T = [None] * (d + 1)
        if lo == -1.0 and hi == 1.0:
            T[1] = x
        else:
            u = self.rescale(self.mult_scalar(x, 2.0 / (hi - lo), cs))
            T[1] = self.add_scalar(u, -(hi + lo) / (hi - lo))
        for k in range(2, d + 1):
            if k % 2 == 0:
                m2 = self.mult_int(self.rescale(self.mult(T[k // 2], T[k // 2])), 2)
                T[k] = self.add_scalar(m2, -1.0)
            else:
                A, B = T[(k - 1) // 2], T[(k + 1) // 2]
                t = min(self.t(A), self.t(B))
                m2 = self.mult_int(self.rescale(self.mult(self.drop(A, t), self.drop(B, t))), 2)
                T[k] = self.sub(m2, self.drop(T[1], self.t(m2)))
        tmin = min(self.t(T[k]) for k in range(1, d + 1) if c[k] != 0)
        acc = None
        for k in range(1, d + 1):
            if c[k] == 0:
                continue
            term = self.mult_scalar(self.drop(T[k], tmin), c[k], cs)
            acc = term if acc is None else self.add(acc, term)
        return self.add_scalar(self.rescale(acc), c[0])
