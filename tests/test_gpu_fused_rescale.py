"""The rescale fused into the forward NTT (switch of the dropped tower on load, (x_i - .) * q_l^-1 on the way out),
against the oracle, on every forward-kernel variant.

The engine runs a rescale as INTT of the top tower -> one NTT launch per batch that switches that tower into every
q_i as it loads it and writes (x_i - NTT(.)) * q_l^-1 instead of the transform.  For N >= 2^13 each forward
variant (radix-16 with 8192 or 4096 residues per CTA, radix-32/16) is forced in turn; rescale at the top level and
at 3 towers, and for the same variants rotation, hoisted rotation and HMult + relinearisation (the separate ModDown
epilogue), are checked residue for residue.  Inputs carry the largest residues (q - 1) in their first
coefficients so the lazy bounds are exercised.
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

NQ, NP, DNUM = 6, 3, 2


@pytest.mark.parametrize("logN", [10, 11, 12, 13, 14, 15, 16])
def test_fused_rescale_every_variant(engine_lib, logN):
    import fideslib_gb300 as F
    N = 1 << logN
    mods = O.make_moduli(logN, [60] + [45] * (NQ - 1), [60] * NP)
    ctx = F.CryptoContext(logN, mods, NP, DNUM)
    orc = O.Ctx(N, NQ, NP, DNUM, mods, threads=16)
    idx = [1, -3]
    keys = {}
    for k, i in enumerate(idx):
        keys[i] = np.stack([[orc.uniform(300 + 10 * k + 2 * a + d, NQ + NP) for d in range(DNUM)] for a in range(2)])
        ctx.load_rotation_key(orc.galois(i), keys[i])
    rlk = np.stack([[orc.uniform(400 + 2 * a + d, NQ + NP) for d in range(DNUM)] for a in range(2)])
    ctx.load_eval_mult_key(rlk)
    cts = []
    for s in (1, 2):
        ct = np.stack([orc.uniform(10 * s, NQ), orc.uniform(10 * s + 1, NQ)])
        for j in range(NQ):
            ct[:, j, :5] = np.uint64(mods[j] - 1)
        cts.append(ct)
    want_rot = {i: orc.rotate(cts[0], orc.galois(i), keys[i]) for i in idx}
    want_hoist = orc.rotate_hoisted(cts[0], [orc.galois(i) for i in idx], [keys[i] for i in idx])
    want_mult = orc.mult(cts[0], cts[1], rlk)
    want_rs = orc.rescale(cts[0])
    want_rs3 = orc.rescale(np.ascontiguousarray(cts[1][:, :3]))
    for v in ((0, 1, 2) if logN >= 13 else (1,)):
        ctx.set_ntt_variant(v, 0)
        h = ctx.load_ciphertext(cts[0], 2.0 ** 45)
        h2 = ctx.load_ciphertext(cts[1], 2.0 ** 45)
        for i in idx:
            assert np.array_equal(ctx.store_ciphertext(ctx.eval_rotate(h, i)), want_rot[i]), (logN, v, i)
        for o, w in zip(ctx.eval_fast_rotation(h, idx), want_hoist):
            assert np.array_equal(ctx.store_ciphertext(o), w), (logN, v, "hoisted")
        assert np.array_equal(ctx.store_ciphertext(ctx.eval_mult(h, h2)), want_mult), (logN, v, "mult")
        assert np.array_equal(ctx.store_ciphertext(ctx.rescale(h)), want_rs), (logN, v, "rescale")
        h3 = ctx.load_ciphertext(np.ascontiguousarray(cts[1][:, :3]), 2.0 ** 45)
        assert np.array_equal(ctx.store_ciphertext(ctx.rescale(h3)), want_rs3), (logN, v, "rescale at 3 towers")
    ctx.close()


@pytest.mark.parametrize("logN", [13, 16])
def test_fused_rescale_mixed_prime_sizes(engine_lib, logN):
    """A chain whose base prime is far smaller than the others (40 against 58 bits): rescaling drops a 58-bit tower,
    which enters the 40-bit tower's transform through the full reduction (q_top >= 15 q_0) and the other towers'
    unreduced; both, and a rescale down to the base prime, equal the oracle on every forward variant, with the
    largest residues in the first coefficients."""
    import fideslib_gb300 as F
    N = 1 << logN
    mods = O.make_moduli(logN, [40] + [58] * (NQ - 1), [60] * NP)
    assert max(mods[1:NQ]) >= 15 * mods[0]
    ctx = F.CryptoContext(logN, mods, NP, DNUM)
    orc = O.Ctx(N, NQ, NP, DNUM, mods, threads=16)
    ct = np.stack([orc.uniform(71, NQ), orc.uniform(72, NQ)])
    for j in range(NQ):
        ct[:, j, :5] = np.uint64(mods[j] - 1)
    want = orc.rescale(ct)
    want2 = orc.rescale(np.ascontiguousarray(ct[:, :2]))
    for v in (0, 1, 2):
        ctx.set_ntt_variant(v, 0)
        h = ctx.load_ciphertext(ct, 2.0 ** 58)
        assert np.array_equal(ctx.store_ciphertext(ctx.rescale(h)), want), (logN, v)
        h2 = ctx.load_ciphertext(np.ascontiguousarray(ct[:, :2]), 2.0 ** 58)
        assert np.array_equal(ctx.store_ciphertext(ctx.rescale(h2)), want2), (logN, v, "to the base prime")
    ctx.close()
