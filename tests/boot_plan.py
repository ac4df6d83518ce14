"""Encoded bootstrap factors for the tests (test helper, not a test module).

The reference receives its CoeffsToSlots / SlotsToCoeffs plaintexts from OpenFHE; here the factors come from
fideslib_gb300.bootplan and their diagonals are encoded by the oracle.  `Factor.replay` evaluates one factor on
the oracle in the engine's op order (`replay_ext` for a double-hoisted factor, whose diagonals carry the special
primes)."""
import numpy as np

from fideslib_gb300.bootplan import (  # noqa: F401  (re-exported for the tests)
    apply, bitrev_perm, bsgs_layout, compose, eval_layout, factors, rotation_indices, slot_matrix, split, stage)


class Factor:
    """One encoded factor: layout plus the oracle-encoded diagonals [bs*gs][towers (+ np when ext)][N]."""

    def __init__(self, orc, M, n, stride, r, towers, delta_pt, ext=False, bs=None):
        self.bs, self.gs, self.base, self.slots = bsgs_layout(M, n, stride, r, bs=bs)
        self.stride = stride
        self.ext = ext
        self.towers_q = towers
        self.present = np.array([s is not None for s in self.slots])
        ids = orc.ext_ids(towers) if ext else list(range(towers))
        self.diags = np.zeros((self.bs * self.gs, len(ids), orc.N), dtype=np.uint64)
        for k, s in enumerate(self.slots):
            if s is not None:
                self.diags[k] = orc.encode(s, delta_pt, len(ids), tower_ids=ids)

    def rotations(self, n, N):
        return rotation_indices(n, N, self.stride, self.bs, self.gs, self.base, self.slots)

    def create(self, gpu, delta_pt) -> int:
        return gpu.lt_create(self.bs, self.gs, self.diags, self.present, delta_pt, stride=self.stride,
                             base=self.base, ext=self.ext)

    def replay(self, orc, ct, keys, N):
        """Oracle replay in the engine's op order (keys: rotation index mod N/2 -> (galois, key))."""
        if self.ext:
            return self.replay_ext(orc, ct, keys, N)
        h = N // 2
        baby = [ct]
        for b in range(1, self.bs):
            r = (b * self.stride) % h
            baby.append(ct if r == 0 else orc.rotate(ct, *keys[r]))
        total = None
        for g in range(self.gs):
            inner = None
            for b in range(self.bs):
                k = g * self.bs + b
                if not self.present[k]:
                    continue
                term = orc.plain_op(baby[b], self.diags[k], 0)
                inner = term if inner is None else orc.add(inner, term)
            if inner is None:
                continue
            r = (self.base + g * self.bs * self.stride) % h
            if r:
                inner = orc.rotate(inner, *keys[r])
            total = inner if total is None else orc.add(total, inner)
        return total

    def replay_ext(self, orc, ct, keys, N):
        """The double-hoisted evaluation (Context::linear_transform_ext_batch) on the oracle: baby-step rotations
        kept in the extended basis Q_t ∪ P, inner sums there, each giant-step sum ModDowned in c1 only and rotated
        without ModDown, one ModDown of the total."""
        h, t = N // 2, ct.shape[1]
        ids = orc.ext_ids(t)
        P = 1
        for p in orc.moduli[orc.nq:]:
            P *= int(p)
        lifted = np.zeros((2, len(ids), N), dtype=np.uint64)
        lifted[:, :t] = orc.scalar_op(ct, [P % int(q) for q in orc.moduli[:t]], [0] * t)
        digits = orc.modup(np.ascontiguousarray(ct[1]), t)
        baby = [lifted]
        for b in range(1, self.bs):
            r = (b * self.stride) % h
            if r == 0:
                baby.append(lifted)
                continue
            g, key = keys[r]
            x = orc.ks_inner(digits, t, key)
            x[0] = orc.ew(x[0], lifted[0], ids, 1)
            baby.append(orc.automorph(x, g))
        total = None
        for gi in range(self.gs):
            inner = None
            for b in range(self.bs):
                k = gi * self.bs + b
                if not self.present[k]:
                    continue
                term = orc.ew(baby[b], self.pt_rows(k, t), ids, 0)
                inner = term if inner is None else orc.ew(inner, term, ids, 1)
            if inner is None:
                continue
            r = (self.base + gi * self.bs * self.stride) % h
            if r:
                g, key = keys[r]
                c1 = orc.moddown(np.ascontiguousarray(inner[1]), t)
                x = orc.ks_inner(orc.modup(c1, t), t, key)
                x[0] = orc.ew(x[0], inner[0], ids, 1)
                inner = orc.automorph(x, g)
            total = inner if total is None else orc.ew(total, inner, ids, 1)
        return np.stack([orc.moddown(np.ascontiguousarray(total[0]), t),
                         orc.moddown(np.ascontiguousarray(total[1]), t)])

    def pt_rows(self, k, t):
        """Diagonal k's rows for a ciphertext of t towers: Q rows 0..t-1, then the special rows."""
        return np.ascontiguousarray(np.concatenate([self.diags[k][:t], self.diags[k][self.towers_q:]]))
