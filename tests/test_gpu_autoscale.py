"""Scaling techniques at the boundary: FIXEDMANUAL's tower cut and the automatic rescaling of FIXEDAUTO,
FLEXIBLEAUTO and FLEXIBLEAUTOEXT (the reference's adjustForAddOrSub / adjustForMult, src/CKKS/Ciphertext.cpp:
1376-1518), replayed op for op by the oracle (oracle/autoscale.py) and checked residue for residue, with the
decrypted result against the plaintext computation; and the slot-aware rotation-key search of
src/CKKS/Context.cu:591-619."""
import numpy as np
import pytest

import oracle as O
from oracle import autoscale as A

pytestmark = pytest.mark.gpu

LOGN = 12
N = 1 << LOGN
NQ, NP, DNUM = 8, 3, 3


@pytest.fixture(scope="module")
def base(engine_lib):
    mods = O.make_moduli(LOGN, [60] + [45] * (NQ - 1), [60] * NP)
    orc = O.Ctx(N, NQ, NP, DNUM, mods, threads=8)
    s = orc.secret(5)
    rlk = orc.relin_key(6, s)
    return dict(mods=mods, orc=orc, s=s, rlk=rlk)


def _ctx(F, base, tech):
    ctx = F.CryptoContext(LOGN, base["mods"], NP, DNUM, scaling_technique=tech)
    ctx.load_eval_mult_key(base["rlk"])
    return ctx


def _load(ctx, c: A.Ct, slots=0):
    return ctx.load_ciphertext(c.data, c.scale, c.deg, slots)


def _check(ctx, h, want: A.Ct, what):
    m = ctx.meta(h)
    assert (m.towers, m.noise_deg) == (want.t, want.deg), what
    assert m.scale == pytest.approx(want.scale, rel=1e-12), what
    assert np.array_equal(ctx.store_ciphertext(h), want.data), what


def _decrypt(base, c: A.Ct):
    return base["orc"].decode(base["orc"].decrypt(base["s"], c.data), c.scale, N // 2)


@pytest.mark.parametrize("tech", [A.FLEXIBLEAUTO, A.FLEXIBLEAUTOEXT, A.FIXEDAUTO])
def test_automatic_chain_matches_replay(base, tech):
    """mult at mismatched levels, then add / sub / square against operands at other levels and degrees: every
    intermediate the reference would rescale, scale-correct or cut is replayed by the oracle, bit for bit."""
    import fideslib_gb300 as F
    orc = base["orc"]
    ctx = _ctx(F, base, tech)
    t_, sf, big, mrf = ctx.scaling()
    q = [int(x) for x in base["mods"][:NQ]]
    want = A.scaling_tables(q, tech)
    assert t_ == tech
    for got, exp in zip((sf, big, mrf), want):
        assert np.array_equal(got, np.array(exp)), "scaling tables differ from the technique's definition"
    S = A.Scaler(orc, tech, sf, big, mrf, base["rlk"])
    rng = np.random.default_rng(tech)
    z = [rng.uniform(-1, 1, N // 2) + 1j * rng.uniform(-1, 1, N // 2) for _ in range(3)]
    cts = []
    for k, t in enumerate((8, 5, 3)):
        cts.append(A.Ct(orc.encrypt(50 + k, base["s"], orc.encode(z[k], sf[t - 1], t)), 1, sf[t - 1]))
    h = [_load(ctx, c) for c in cts]

    m = S.mult(cts[0], cts[1])
    hm = ctx.eval_mult(h[0], h[1])
    _check(ctx, hm, m, "mult of 8 and 5 towers")
    r = S.add(m, cts[2])
    hr = ctx.eval_add(hm, h[2])
    _check(ctx, hr, r, "add of a degree-2 product to 3 towers")
    d = S.add(cts[2], m, sub=True)
    hd = ctx.eval_sub(h[2], hm)
    _check(ctx, hd, d, "sub with the roles swapped")
    sq = S.square(m)
    hsq = ctx.eval_square(hm)
    _check(ctx, hsq, sq, "square of a degree-2 ciphertext")
    # the same requests through one batch
    hb = ctx.eval_batch([(F.OP_MULT, h[0], h[1], 0), (F.OP_ADD, hm, h[2], 0), (F.OP_SUB, h[2], hm, 0),
                         (F.OP_SQUARE, hm, 0, 0)])
    for hh, want_ct in zip(hb, (m, r, d, sq)):
        _check(ctx, hh, want_ct, "batched")
    # and the values are the plaintext computation's
    assert np.abs(_decrypt(base, r) - (z[0] * z[1] + z[2])).max() < 1e-5
    assert np.abs(_decrypt(base, d) - (z[2] - z[0] * z[1])).max() < 1e-5
    assert np.abs(_decrypt(base, sq) - (z[0] * z[1]) ** 2).max() < 1e-5
    ctx.close()


def test_fixedmanual_cuts_to_the_lower_level(base):
    import fideslib_gb300 as F
    orc = base["orc"]
    ctx = _ctx(F, base, A.FIXEDMANUAL)
    rng = np.random.default_rng(3)
    sc = 2.0 ** 45
    z = [rng.uniform(-1, 1, N // 2) for _ in range(2)]
    c8 = orc.encrypt(60, base["s"], orc.encode(z[0], sc, 8))
    c3 = orc.encrypt(61, base["s"], orc.encode(z[1], sc, 3))
    h8, h3 = ctx.load_ciphertext(c8, sc), ctx.load_ciphertext(c3, sc)
    got = ctx.store_ciphertext(ctx.eval_add(h3, h8))
    assert np.array_equal(got, orc.add(c3, np.ascontiguousarray(c8[:, :3])))
    got = ctx.store_ciphertext(ctx.eval_mult(h8, h3))
    assert np.array_equal(got, orc.mult(np.ascontiguousarray(c8[:, :3]), c3, base["rlk"]))
    ctx.close()


def test_sparse_slot_rotation_uses_a_congruent_key(base):
    """A ciphertext packing 16 slots rotated by 3 with only the key of 19 loaded (19 = 3 mod 16), and by -3 with
    only the key of 13: the reference's normalised index and congruent-key search pick those keys; a full-slot
    ciphertext finds none."""
    import fideslib_gb300 as F
    orc, s = base["orc"], base["s"]
    ctx = _ctx(F, base, A.FIXEDMANUAL)
    keys = {}
    for idx in (19, 13):
        g = orc.galois(idx)
        keys[idx] = orc.rot_key(70 + idx, s, g)
        ctx.load_rotation_key(g, keys[idx])
    rng = np.random.default_rng(8)
    z16 = rng.uniform(-1, 1, 16) + 1j * rng.uniform(-1, 1, 16)
    ct = orc.encrypt(80, s, orc.encode(np.tile(z16, N // 2 // 16), 2.0 ** 45, 6))
    h = ctx.load_ciphertext(ct, 2.0 ** 45, 1, 16)
    for index, used in ((3, 19), (-3, 13)):
        got = ctx.store_ciphertext(ctx.eval_rotate(h, index))
        assert np.array_equal(got, orc.rotate(ct, orc.galois(used), keys[used])), index
        vals = orc.decode(orc.decrypt(s, got), 2.0 ** 45, N // 2)[:16]
        assert np.abs(vals - np.roll(z16, -index)).max() < 1e-6, index
    hf = ctx.load_ciphertext(ct, 2.0 ** 45, 1, 0)  # slots unknown: full packing, no congruent search
    with pytest.raises(F.FidesError) as ei:
        ctx.eval_rotate(hf, 3)
    assert ei.value.code == F.FIDES_ENOKEY
    ctx.close()


def test_composites_do_not_depend_on_the_technique(base):
    """The engine's composites (here EvalMod's double-angle iterations and a Chebyshev series) keep their own exact
    level and scale bookkeeping: under FLEXIBLEAUTO they return the residues they return under FIXEDMANUAL."""
    import fideslib_gb300 as F
    orc = base["orc"]
    rng = np.random.default_rng(12)
    z = rng.uniform(-1, 1, N // 2)
    ct = orc.encrypt(90, base["s"], orc.encode(z, 2.0 ** 45, 8))
    outs = []
    for tech in (A.FIXEDMANUAL, A.FLEXIBLEAUTO):
        ctx = _ctx(F, base, tech)
        h = ctx.load_ciphertext(ct, 2.0 ** 45)
        outs.append((ctx.store_ciphertext(ctx.eval_double_angle(h, 2)),
                     ctx.store_ciphertext(ctx.eval_chebyshev(h, [0.1, -0.4, 0.25, 0.05, -0.02], -1.0, 1.0, 2.0 ** 45))))
        ctx.close()
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])
