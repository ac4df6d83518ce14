"""Encoded bootstrap factors for the tests (test helper, not a test module).

The reference receives its CoeffsToSlots / SlotsToCoeffs plaintexts from OpenFHE; here the factors come from
fideslib_gb300.bootplan and their diagonals are encoded by the oracle.  `Factor.replay` evaluates one factor on
the oracle in the engine's op order."""
import numpy as np

from fideslib_gb300.bootplan import (  # noqa: F401  (re-exported for the tests)
    apply, bitrev_perm, bsgs_layout, compose, eval_layout, factors, rotation_indices, slot_matrix, split, stage)


class Factor:
    """One encoded factor: layout plus the oracle-encoded diagonals [bs*gs][towers][N]."""

    def __init__(self, orc, M, n, stride, r, towers, delta_pt):
        self.bs, self.gs, self.base, self.slots = bsgs_layout(M, n, stride, r)
        self.stride = stride
        self.present = np.array([s is not None for s in self.slots])
        self.diags = np.zeros((self.bs * self.gs, towers, orc.N), dtype=np.uint64)
        for k, s in enumerate(self.slots):
            if s is not None:
                self.diags[k] = orc.encode(s, delta_pt, towers)

    def rotations(self, n, N):
        return rotation_indices(n, N, self.stride, self.bs, self.gs, self.base, self.slots)

    def create(self, gpu, delta_pt) -> int:
        return gpu.lt_create(self.bs, self.gs, self.diags, self.present, delta_pt, stride=self.stride,
                             base=self.base)

    def replay(self, orc, ct, keys, N):
        """Oracle replay in the engine's op order (keys: rotation index mod N/2 -> (galois, key))."""
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
