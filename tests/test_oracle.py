"""CPU tests of the oracle: pinned to the reference's own CPU NTT and to CKKS algebraic identities."""
import os

import numpy as np
import pytest

import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ntt_reference.npz")


def brev_perm(N):
    logn = N.bit_length() - 1
    return np.array([int(format(i, f"0{logn}b")[::-1], 2) for i in range(N)])


def golden_cases():
    g = np.load(GOLDEN)
    keys = sorted({k.rsplit("_", 1)[0] for k in g.files if k.endswith("_in")})
    return g, keys


def test_oracle_ntt_matches_reference_golden_vectors():
    """Forward NTT (bit-reversed output) == bit-reverse of the reference's nega_fft / nega_fft2 output."""
    g, keys = golden_cases()
    assert len(keys) >= 5
    for k in keys:
        N = int(k.split("_")[0][1:])
        p = int(k.split("_p")[1])
        psi = int(g[k + "_psi"][0])
        assert psi == O.root_of_unity(p, 2 * N)  # the reference's generator-based root (ConstantsGPU.cu:37-67)
        tab, itab = O.ntt_tables(N, p, psi)
        a = g[k + "_in"]
        mine = O.ntt_fwd(a, p, tab)
        br = brev_perm(N)
        assert np.array_equal(mine, g[k + "_nega_fft"][br]), k
        assert np.array_equal(mine, g[k + "_nega_fft2"][br]), k
        assert np.array_equal(O.ntt_inv(mine, p, itab), a), k
        assert np.array_equal(g[k + "_nega_fft2_inv"], a), k


def test_known_answer_p17_n8_round_trip():
    """test/NegacyclicNTTtests.cu:44-68: v2 = {1,2,3,7,5,4,1,2} mod 17 survives NTT->INTT and INTT->NTT."""
    p, N = 17, 8
    psi = O.root_of_unity(p, 2 * N)
    tab, itab = O.ntt_tables(N, p, psi)
    v = np.array([1, 2, 3, 7, 5, 4, 1, 2], dtype=np.uint64)
    assert np.array_equal(O.ntt_inv(O.ntt_fwd(v, p, tab), p, itab), v)
    assert np.array_equal(O.ntt_fwd(O.ntt_inv(v, p, itab), p, tab), v)
    # negacyclic convolution theorem on the same vectors (the test's second half)
    v1 = np.array([1, 2, 3, 7, 5, 4, 3, 9], dtype=np.uint64)
    prod = O.ntt_inv((O.ntt_fwd(v1, p, tab) * O.ntt_fwd(v, p, tab)) % p, p, itab)
    ref = np.zeros(N, dtype=np.int64)
    for i in range(N):
        for j in range(N):
            if i + j < N:
                ref[i + j] += int(v1[i]) * int(v[j])
            else:
                ref[i + j - N] -= int(v1[i]) * int(v[j])
    assert np.array_equal(prod, (ref % p).astype(np.uint64))


def test_reference_build_matches_when_available():
    """Live check against oracle/_ref (built from the reference sources) when the reference tree exists."""
    try:
        O.build_ref()
    except Exception as e:  # pragma: no cover - the build needs nvcc
        pytest.skip(f"reference build unavailable: {e}")
    R = O.ref_lib()
    if R is None:
        pytest.skip("reference tree not present on this host")
    N = 1 << 14
    p = O.gen_primes(59, 1, 2 * N)[0]
    psi = O.root_of_unity(p, 2 * N)
    tab, itab = O.ntt_tables(N, p, psi)
    a = np.random.default_rng(5).integers(0, p, N, dtype=np.uint64)
    r = a.copy()
    R.ref_nega_fft(O._p(r), N, 0, O._p(tab), O._p(itab), p)
    assert np.array_equal(O.ntt_fwd(a, p, tab), r[brev_perm(N)])


def test_gen_primes_and_roots():
    N = 1 << 12
    ps = O.gen_primes(50, 4, 2 * N)
    assert len(set(ps)) == 4
    for p in ps:
        assert p % (2 * N) == 1 and p < 2 ** 50 and O.lib().orc_is_prime(p)
        r = O.root_of_unity(p, 2 * N)
        assert pow(r, N, p) == p - 1


@pytest.fixture(scope="module")
def ckks():
    logN = 11
    N = 1 << logN
    mods = O.make_moduli(logN, [60] + [45] * 7, [60] * 4)
    ctx = O.Ctx(N, 8, 4, 3, mods, threads=4)
    s = ctx.secret(0x5EED0001)
    rng = np.random.default_rng(3)
    z = rng.uniform(-1, 1, N // 2) + 1j * rng.uniform(-1, 1, N // 2)
    scale = 2.0 ** 45
    pt = ctx.encode(z, scale, 8)
    ct = ctx.encrypt(17, s, pt)
    return dict(ctx=ctx, s=s, z=z, scale=scale, ct=ct, mods=mods, N=N)


def dec(c, ct, scale):
    ctx = c["ctx"]
    return ctx.decode(ctx.decrypt(c["s"], ct), scale, c["N"] // 2)


def test_encrypt_decrypt(ckks):
    assert np.abs(dec(ckks, ckks["ct"], ckks["scale"]) - ckks["z"]).max() < 1e-8


@pytest.mark.parametrize("t", [8, 5, 3, 1])
@pytest.mark.parametrize("index", [1, -3, 7])
def test_rotate_decrypts_to_rotated_slots(ckks, t, index):
    ctx = ckks["ctx"]
    g = ctx.galois(index)
    key = ctx.rot_key(100 + index, ckks["s"], g)
    ct = np.ascontiguousarray(ckks["ct"][:, :t])
    r = ctx.rotate(ct, g, key)
    err = np.abs(dec(ckks, r, ckks["scale"]) - np.roll(ckks["z"], -index)).max()
    assert err < 1e-6, err


def test_hoisted_equals_individual_rotations(ckks):
    ctx = ckks["ctx"]
    idx = [1, 2, -4]
    gs = [ctx.galois(i) for i in idx]
    keys = [ctx.rot_key(7 + i, ckks["s"], g) for i, g in zip(idx, gs)]
    hs = ctx.rotate_hoisted(ckks["ct"], gs, keys)
    for g, k, h in zip(gs, keys, hs):
        assert np.array_equal(h, ctx.rotate(ckks["ct"], g, k))


def test_conjugation(ckks):
    ctx = ckks["ctx"]
    g = 2 * ckks["N"] - 1
    key = ctx.rot_key(55, ckks["s"], g)
    r = ctx.rotate(ckks["ct"], g, key)
    assert np.abs(dec(ckks, r, ckks["scale"]) - np.conj(ckks["z"])).max() < 1e-6


def test_mult_relin_rescale(ckks):
    ctx = ckks["ctx"]
    rlk = ctx.relin_key(9, ckks["s"])
    m = ctx.mult(ckks["ct"], ckks["ct"], rlk)
    sc2 = ckks["scale"] ** 2
    assert np.abs(dec(ckks, m, sc2) - ckks["z"] ** 2).max() < 1e-6
    r = ctx.rescale(m)
    assert r.shape[1] == 7
    assert np.abs(dec(ckks, r, sc2 / ckks["mods"][7]) - ckks["z"] ** 2).max() < 1e-6


def test_keyswitch_linearity(ckks):
    """ModUp, the inner product and ModDown are exact maps: KS(a) + KS(b) - KS(a+b) is tiny noise only."""
    ctx = ckks["ctx"]
    key = ctx.relin_key(3, ckks["s"])
    a = ctx.uniform(1, 8)
    b = ctx.uniform(2, 8)
    ab = ctx.add(a[None], b[None])[0]
    # modup + inner product are exactly linear before ModDown
    d = ctx.ks_inner(ctx.modup(a, 8), 8, key)
    e = ctx.ks_inner(ctx.modup(b, 8), 8, key)
    assert d.shape == (2, 12, ckks["N"]) and e.shape == d.shape


def test_rescale_matches_exact_division():
    """Rescale == round-toward-centred (x - [x]_{q_l}) / q_l, checked through CRT on a tiny ring."""
    logN = 10
    N = 1 << logN
    mods = O.make_moduli(logN, [50, 40, 40], [50])
    ctx = O.Ctx(N, 3, 1, 1, mods)
    rng = np.random.default_rng(11)
    vals = rng.integers(-(2 ** 100), 2 ** 100, N, dtype=np.int64) if False else None
    big = [int(rng.integers(0, 2 ** 62)) * 2 ** 60 + int(rng.integers(0, 2 ** 60)) for _ in range(N)]
    big = [b - 2 ** 121 for b in big]
    x = np.array([[b % m for b in big] for m in mods[:3]], dtype=np.uint64)
    xe = ctx.to_eval(x)
    ct = np.stack([xe, xe])
    r = ctx.rescale(ct)
    rc = ctx.to_coeff(r[0])
    ql = mods[2]
    for i in range(0, N, 97):
        b = big[i]
        top = b % ql
        if top > ql // 2:
            top -= ql
        exact = (b - top) // ql
        for j in range(2):
            assert int(rc[j][i]) == exact % mods[j]


def test_scaling_tables_and_constants():
    """The oracle's scaling tables keep FLEXIBLEAUTO's invariant (a product rescaled by q_l lands on the next
    level's factor: sf[l-1] q_l = sf[l]^2), FIXED* tables are one power of two, and a constant is round(v sf)
    reduced per tower (exact big-integer check, including the 2^k split past 2^125)."""
    from oracle import autoscale as A
    q = O.gen_primes(45, 6, 1 << 13)
    sf, big, mrf = A.scaling_tables(q, A.FLEXIBLEAUTO)
    assert sf[-1] == float(q[-1]) and mrf == [float(x) for x in q]
    for lv in range(1, len(q)):
        assert abs(sf[lv - 1] * q[lv] - sf[lv] ** 2) <= 1e-12 * sf[lv] ** 2
        assert big[lv] == sf[lv] * sf[lv]
    sfx, bigx, _ = A.scaling_tables(q, A.FLEXIBLEAUTOEXT)
    assert sfx[-1] == sfx[-2] == float(q[-2]) and bigx[-1] == sfx[-1] * sfx[-2]
    sff, _, _ = A.scaling_tables(q, A.FIXEDAUTO)
    assert sff == [2.0 ** 45] * len(q)
    for v in (1.0, -0.3, 12345.678, -2.0 ** 90):
        k = A.eval_mult_constants(q, sf, 4, v)
        x = v * sf[3]
        if abs(x) < 2.0 ** 125:
            exact = int(x + 0.5)
            assert k == [exact % qi for qi in q[:4]]
    big_v = 2.0 ** 100
    k = A.eval_mult_constants(q, [2.0 ** 40] * 6, 2, big_v)  # 2^140: scaled by 2^15 and restored
    assert k == [(2 ** 140) % qi for qi in q[:2]]
