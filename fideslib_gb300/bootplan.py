"""Bootstrap precomputation (host side, FP64): the level-budget factors of CoeffsToSlots / SlotsToCoeffs and
their baby-step/giant-step layout for fides_lt_create_strided.

OpenFHE computes these for the reference (EvalBootstrapSetup; FIDESlib receives the encoded plaintexts through
RawCiphertext.cu AddBootstrapPrecomputation and evaluates them in src/CKKS/CoeffsToSlots.cu:77-151).  Here they
come from the factored special FFT; encoding the diagonals into plaintexts is left to the caller's CKKS
encoder.  Conventions (the engine's):

* slots z = U_n w, U_n[j][k] = xi^(5^j k), xi = exp(i pi / 2n), w = packed coefficients;
* U_n = S_n ... S_4 S_2 P with P the bit-reversal permutation and S_len the butterfly stage of length len
  (three diagonals: 0, +len/2, -len/2);
* a slot-linear map M acts as (M v)[x] = sum_o d_o[x] v[(x + o) mod n] ("diagonal o");
* a factor is evaluated as out = sum_g rot_{base + g bs s}( sum_b D[g bs + b] (.) rot_{b s}(x) ), D[k] the
  diagonal of offset base + k s pre-rotated by -(base + g bs s), rot_r(v)[x] = v[(x + r) mod n].
"""
import numpy as np


def slot_matrix(n: int) -> np.ndarray:
    xi = np.exp(1j * np.pi / (2 * n))
    return np.array([[xi ** ((pow(5, j, 4 * n) * k) % (4 * n)) for k in range(n)] for j in range(n)])


def bitrev_perm(n: int) -> np.ndarray:
    m = n.bit_length() - 1
    return np.array([int(format(i, f"0{m}b")[::-1], 2) if m else 0 for i in range(n)])


def stage(n: int, ln: int, inverse: bool = False) -> dict:
    """Diagonals of S_len (or its inverse): on each block of len slots, top position j < len/2 and bottom
    position j + len/2 hold (u + w_j v, u - w_j v), w_j = exp(2 pi i (5^j mod 4 len) / (4 len))."""
    h = ln // 2
    p5 = np.empty(h, dtype=np.int64)
    acc = 1
    for j in range(h):
        p5[j] = acc
        acc = acc * 5 % (4 * ln)
    x = np.arange(n)
    j = x % ln
    top = j < h
    w = np.exp(2j * np.pi * p5[np.where(top, j, j - h)] / (4 * ln))
    if not inverse:  # (a, b) = (u + w v, u - w v)
        d0 = np.where(top, 1.0 + 0j, -w)
        dp = np.where(top, w, 0j)
        dm = np.where(top, 0j, 1.0 + 0j)
    else:  # u = (a + b) / 2, v = (a - b) / (2 w)
        d0 = np.where(top, 0.5 + 0j, -0.5 / w)
        dp = np.where(top, 0.5 + 0j, 0j)
        dm = np.where(top, 0j, 0.5 / w)
    out = {}
    for o, d in ((0, d0), (h % n, dp), ((-h) % n, dm)):
        out[o] = out.get(o, 0) + d
    return out


def compose(A: dict, B: dict, n: int) -> dict:
    """Diagonals of A @ B."""
    out = {}
    for a, da in A.items():
        for b, db in B.items():
            o = (a + b) % n
            out[o] = out.get(o, 0) + da * np.roll(db, -a)
    return out


def apply(M: dict, v: np.ndarray) -> np.ndarray:
    return sum(d * np.roll(v, -o) for o, d in M.items())


def split(m: int, budget: int) -> list:
    """m stages into `budget` consecutive groups, sizes as even as possible (larger groups first)."""
    q, r = divmod(m, budget)
    return [q + (1 if i < r else 0) for i in range(budget)]


def factors(n: int, budget: int, inverse: bool, scale: complex = 1.0):
    """Level-budget factors in application order, each (diagonals, stride, r = stages in the group).

    inverse=False (SlotsToCoeffs): S_2 first, ..., S_n last (product U_n P).
    inverse=True (CoeffsToSlots): S_n^-1 first, ..., S_2^-1 last (product P U_n^-1), times `scale`."""
    m = n.bit_length() - 1
    lens = [1 << (i + 1) for i in range(m)]  # 2, 4, ..., n
    sizes = split(m, budget)
    groups, pos = [], 0
    for sz in sizes:
        groups.append(lens[pos:pos + sz])
        pos += sz
    if inverse:
        groups = [list(reversed(g)) for g in reversed(groups)]
    out = []
    for gi, g in enumerate(groups):
        M = {0: np.ones(n, complex)}
        for ln in g:  # later stages multiply on the left
            M = compose(stage(n, ln, inverse), M, n)
        if inverse and gi == 0:
            M = {o: d * scale for o, d in M.items()}
        out.append((M, min(g) // 2, len(g)))
    return out


def bsgs_layout(M: dict, n: int, stride: int, r: int, bs: int | None = None):
    """(bs, gs, base, D list of length bs*gs with None for absent diagonals) for diagonals at multiples of stride
    within +-(2^r - 1) stride.  bs defaults to 2^ceil((r+1)/2) (at most 16, the engine's limit); a double-hoisted
    transform, whose baby steps cost no NTT, runs faster with more baby steps (ext_baby_steps)."""
    D = 2 ** (r + 1) - 1
    base = -(2 ** r - 1) * stride
    if bs is None:
        bs = min(16, 1 << ((r + 2) // 2))
    gs = -(-D // bs)
    slots = [None] * (bs * gs)
    for o, d in M.items():
        if not np.any(np.abs(d) > 1e-13):
            continue
        for k in range(bs * gs):
            if (base + k * stride - o) % n == 0:
                break
        else:
            raise ValueError(f"offset {o} not on the stride-{stride} grid")
        g = k // bs
        rot = np.roll(d, base + g * bs * stride)  # rot_{-(base + g bs s)}
        slots[k] = rot if slots[k] is None else slots[k] + rot
    return bs, gs, base, slots


def ext_baby_steps(r: int) -> int:
    """Baby-step count for a double-hoisted factor of 2^(r+1) - 1 diagonals: twice the default (gs about halves),
    at most 16."""
    return min(16, 1 << ((r + 2) // 2 + 1))


def eval_layout(v: np.ndarray, n: int, stride: int, bs: int, gs: int, base: int, slots) -> np.ndarray:
    """Plain-vector evaluation of the baby-step/giant-step form (the engine's op order)."""
    rot = lambda x, r: np.roll(x, -(r % n))  # noqa: E731
    out = np.zeros(n, complex)
    for g in range(gs):
        inner = np.zeros(n, complex)
        for b in range(bs):
            if slots[g * bs + b] is not None:
                inner += slots[g * bs + b] * rot(v, b * stride)
        out += rot(inner, base + g * bs * stride)
    return out


def rotation_indices(n: int, N: int, stride: int, bs: int, gs: int, base: int, slots) -> set:
    """Slot-rotation indices (mod N/2, nonzero) a factor needs keys for."""
    h = N // 2
    need = {(b * stride) % h for b in range(1, bs)}
    for g in range(gs):
        if any(slots[g * bs + b] is not None for b in range(bs)):
            need.add((base + g * bs * stride) % h)
    need.discard(0)
    return need
