"""Bootstrapping at the config-5 shape: N = 2^16, 32768 full slots, level budget {3, 3}, sparse-secret
encapsulation (main secret of Hamming weight 192, encapsulated under weight 32).

Moduli: q_0 of 60 bits and 24 towers of 55 bits (the scaling factor 2^55 sits on the towers, q_0 / scale = 32),
5 special primes of 60 bits (P above each 5-tower digit), dnum 5.  Keys come from the oracle; the CoeffsToSlots /
SlotsToCoeffs diagonals are encoded on the GPU at the special primes too (fides_lt_create_slots_ext: double-hoisted
factors with twice the default baby steps, as in the config-5 benchmark).  Residue-exact replay at this size is too
slow for the oracle (the N = 2^12 tests replay the same recipe op for op); this test states the decrypted
precision."""
import numpy as np
import numpy.polynomial.chebyshev as C
import pytest

import oracle as O
from fideslib_gb300 import bootplan as BP

pytestmark = pytest.mark.gpu

LOGN = 16
N = 1 << LOGN
NQ, NP, DNUM = 25, 5, 5
DELTA = 2.0 ** 55
R_DOUBLE, CHEB_DEG, B_RANGE = 3, 47, 12.5


def test_bootstrap_full_slots_n16(engine_lib):
    import fideslib_gb300 as F
    n = N // 2
    mods = O.make_moduli(LOGN, [60] + [55] * (NQ - 1), [60] * NP)
    gpu = F.CryptoContext(LOGN, mods, NP, DNUM)
    orc = O.Ctx(N, NQ, NP, DNUM, mods, threads=16)
    s = orc.secret(0x5EED0051, hamming_weight=192)
    s_sparse = orc.secret(0x5EED0052, hamming_weight=32)
    gpu.load_eval_mult_key(orc.relin_key(1, s))
    gpu.load_switch_key(1, orc.switch_key(2, s, s_sparse))
    gpu.load_switch_key(2, orc.switch_key(3, s_sparse, s))
    gpu.load_rotation_key(2 * N - 1, orc.rot_key(4, s, 2 * N - 1))
    lts = {True: [], False: []}
    need = set()
    for inverse in (True, False):
        for M, stride, r in BP.factors(n, 3, inverse, scale=n / N if inverse else 1.0):
            bs, gs, base, slots = BP.bsgs_layout(M, n, stride, r, bs=BP.ext_baby_steps(r))
            need |= BP.rotation_indices(n, N, stride, bs, gs, base, slots)
            present = np.array([x is not None for x in slots])
            diag = np.array([x if x is not None else np.zeros(n) for x in slots])
            lts[inverse].append(gpu.lt_create_slots(bs, gs, diag, present, DELTA, NQ, stride=stride, base=base,
                                                    ext=True))
    for i, idx in enumerate(sorted(need)):
        g = orc.galois(idx)
        gpu.load_rotation_key(g, orc.rot_key(100 + i, s, g))
    K = mods[0] / DELTA
    lo, hi = -B_RANGE * K, B_RANGE * K
    f = lambda r: np.cos(2 * np.pi * (r / K - 0.25) / 2 ** R_DOUBLE)  # noqa: E731
    coeffs = C.chebinterpolate(lambda u: f(lo + (u + 1) * (hi - lo) / 2), CHEB_DEG)
    plan = F.BootstrapPlan.make(n, NQ, lts[True], lts[False], coeffs, R_DOUBLE, lo, hi, DELTA, sse_keys=(1, 2))
    rng = np.random.default_rng(0x5EED0053)
    z = (rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)) * 0.5
    ct = orc.encrypt(5, s, orc.encode(z, DELTA, 1))
    out = gpu.eval_bootstrap(gpu.load_ciphertext(ct, DELTA), plan)
    meta = gpu.meta(out)
    dec = orc.decode(orc.decrypt(s, gpu.store_ciphertext(out)), meta.scale, n)
    err = np.abs(dec - z).max()
    print(f"bootstrap N=2^16, {n} slots: {meta.towers} towers left, max slot error {err:.3e} "
          f"({-np.log2(err):.1f} bits)")
    assert meta.towers >= 4
    assert err < 1e-4, err
