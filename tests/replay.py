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

    def _align(self, a, b):
        t = min(self.t(a), self.t(b))
        return self.drop(a, t), self.drop(b, t)

    def _next_t(self, T, k):
        if k % 2 == 0:
            return self.add_scalar(self.mult_int(self.rescale(self.mult(T[k // 2], T[k // 2])), 2), -1.0)
        A, B = self._align(T[(k - 1) // 2], T[(k + 1) // 2])
        m2 = self.mult_int(self.rescale(self.mult(A, B)), 2)
        t1 = self.drop(T[1], self.t(m2) + 1)
        f = m2[1] * float(self.mods[self.t(m2)]) / t1[1]
        return self.sub(m2, self.rescale(self.mult_scalar(t1, 1.0, f)))

    def _leaf_towers(self, T, c):
        ks = [k for k in range(1, len(c)) if c[k] != 0]
        return min(self.t(T[k]) for k in ks) - 1 if ks else None

    @staticmethod
    def _split(c):
        M = len(c) // 2
        q, r = [0.0] * M, list(c[:M])
        q[0] = c[M]
        for j in range(1, M):
            q[j] = 2.0 * c[M + j]
            r[M - j] -= c[M + j]
        return q, r

    def _node_towers(self, T, G, c, i):
        if i == 0:
            return self._leaf_towers(T, c)
        q, r = self._split(c)
        tq, tr = self._node_towers(T, G, q, i - 1), self._node_towers(T, G, r, i - 1)
        tg = self.t(G[i - 1])
        tp = min(tq, tg) - 1 if tq is not None else (tg - 1 if q[0] != 0.0 else None)
        if tp is None:
            return tr
        return tp if tr is None else min(tp, tr)

    def _leaf(self, T, c, target):
        tl = self._leaf_towers(T, c)
        acc = None
        for k in range(1, len(c)):
            if c[k] == 0:
                continue
            X = self.drop(T[k], tl + 1)
            term = self.mult_scalar(X, c[k], target * float(self.mods[tl]) / X[1])
            acc = term if acc is None else self.add(acc, term)
        return (self.rescale(acc) if acc is not None else None), c[0]

    def _node(self, T, G, c, i, target):
        if i == 0:
            return self._leaf(T, c, target)
        q, r = self._split(c)
        Gm = G[i - 1]
        tg, sg = self.t(Gm), Gm[1]
        prod = None
        if any(x != 0.0 for x in q[1:]):
            tq = self._node_towers(T, G, q, i - 1)
            Qct, Qc = self._node(T, G, q, i - 1, target * float(self.mods[min(tq, tg) - 1]) / sg)
            X = self.add_scalar(Qct, Qc) if Qc != 0.0 else Qct
            X, Gd = self._align(X, Gm)
            prod = self.rescale(self.mult(X, Gd))
        elif q[0] != 0.0:
            prod = self.rescale(self.mult_scalar(Gm, q[0], target * float(self.mods[tg - 1]) / sg))
        Rct, Rc = self._node(T, G, r, i - 1, target)
        if prod is None:
            return Rct, Rc
        if Rct is None:
            return prod, Rc
        pd, rd = self._align(prod, Rct)
        return self.add(pd, rd), Rc

    def chebyshev(self, x, c, lo, hi, cs):
        """Baby-step/giant-step Chebyshev evaluation in the engine's op order (fideslib_gb300/csrc/poly_eval.cu)."""
        d = len(c) - 1
        if lo == -1.0 and hi == 1.0:
            t1 = x
        else:
            u = self.rescale(self.mult_scalar(x, 2.0 / (hi - lo), cs))
            t1 = self.add_scalar(u, -(hi + lo) / (hi - lo))
        lb = max(1, int(np.floor(np.log2(d + 1) / 2.0 + 0.5)))
        bs = 1 << lb
        m = 0
        while (bs << m) <= d:
            m += 1
        top = bs if m > 0 else bs - 1
        T = [None, t1] + [None] * (top - 1)
        for k in range(2, top + 1):
            T[k] = self._next_t(T, k)
        G = [T[bs]] if m > 0 else []
        for i in range(1, m):
            G.append(self.add_scalar(self.mult_int(self.rescale(self.mult(G[i - 1], G[i - 1])), 2), -1.0))
        cc = list(c) + [0.0] * ((bs << m) - len(c))
        ct, c0 = self._node(T, G, cc, m, t1[1])
        assert ct is not None
        return self.add_scalar(ct, c0)
