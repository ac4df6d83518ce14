"""GPU parity of the CKKS evaluation ops against the oracle: every residue bit-identical, through the C ABI.

Inputs are real encryptions under oracle-generated keys, so each case also states decrypted precision."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

PARAMS = {
    # ring, Q bits, P bits, dnum
    "cfg1_n13": (13, [60] + [40] * 5, [60] * 3, 2),
    "cfg3_small": (12, [60] + [50] * 29, [60] * 10, 3),
    "dnum4": (11, [60] + [45] * 7, [60] * 3, 4),
}


class Env:
    def __init__(self, name):
        import fideslib_gb300 as F
        logN, qb, pb, dnum = PARAMS[name]
        self.N = N = 1 << logN
        self.mods = O.make_moduli(logN, qb, pb)
        self.nq, self.np = len(qb), len(pb)
        self.orc = O.Ctx(N, self.nq, self.np, dnum, self.mods, threads=8)
        self.gpu = F.CryptoContext(logN, self.mods, self.np, dnum, roots=None)
        assert self.gpu.roots == [O.root_of_unity(p, 2 * N) for p in self.mods]
        self.s = self.orc.secret(0x5EED0003)
        rng = np.random.default_rng(7)
        self.z = rng.uniform(-1, 1, N // 2) + 1j * rng.uniform(-1, 1, N // 2)
        self.scale = 2.0 ** 40
        self.pt = self.orc.encode(self.z, self.scale, self.nq)
        self.ct = self.orc.encrypt(21, self.s, self.pt)
        self.rlk = self.orc.relin_key(5, self.s)
        self.gpu.load_eval_mult_key(self.rlk)
        self.rot = {}

    def rot_key(self, index):
        g = self.orc.galois(index)
        if g not in self.rot:
            self.rot[g] = self.orc.rot_key(1000 + g, self.s, g)
            self.gpu.load_rotation_key(g, self.rot[g])
        return g, self.rot[g]

    def at(self, t):
        return np.ascontiguousarray(self.ct[:, :t])

    def decode(self, ct, scale):
        return self.orc.decode(self.orc.decrypt(self.s, ct), scale, self.N // 2)


@pytest.fixture(scope="module", params=list(PARAMS))
def env(request, engine_lib):
    return Env(request.param)


def test_rotate_bit_exact(env):
    for t in sorted({env.nq, max(1, env.nq // 2), 1}):
        for index in (1, -5):
            g, key = env.rot_key(index)
            ct = env.at(t)
            h = env.gpu.load_ciphertext(ct, env.scale)
            r = env.gpu.eval_rotate(h, index)
            got = env.gpu.store_ciphertext(r)
            exp = env.orc.rotate(ct, g, key)
            assert np.array_equal(got, exp), (t, index)
            err = np.abs(env.decode(got, env.scale) - np.roll(env.z, -index)).max()
            assert err < 1e-5, err


def test_fast_rotation_bit_exact(env):
    t = env.nq
    idx = [1, 2, -3, 4]
    gk = [env.rot_key(i) for i in idx]
    ct = env.at(t)
    h = env.gpu.load_ciphertext(ct, env.scale)
    outs = env.gpu.eval_fast_rotation(h, idx)
    exps = env.orc.rotate_hoisted(ct, [g for g, _ in gk], [k for _, k in gk])
    for o, e in zip(outs, exps):
        assert np.array_equal(env.gpu.store_ciphertext(o), e)


def test_precomputed_fast_rotation(env):
    """EvalFastRotationPrecompute, then rotations by several indices from the kept digits (after the source
    handle is freed): bit-identical to plain rotations and to the oracle."""
    for t in sorted({env.nq, 2}):
        ct = env.at(t)
        h = env.gpu.load_ciphertext(ct, env.scale)
        pre = env.gpu.fast_rotation_precompute(h)
        outs = {}
        for index in (1, -5, 3):
            g, key = env.rot_key(index)
            outs[index] = env.gpu.store_ciphertext(env.gpu.eval_fast_rotation_precomputed(h, pre, index))
            assert np.array_equal(outs[index], env.orc.rotate(ct, g, key)), (t, index)
        h2 = env.gpu.load_ciphertext(ct, env.scale)  # the same residues under another handle
        env.gpu.free(h)
        assert np.array_equal(env.gpu.store_ciphertext(env.gpu.eval_fast_rotation_precomputed(h2, pre, 1)), outs[1])
        env.gpu.precompute_free(pre)


def test_mult_square_rescale_bit_exact(env):
    for t in sorted({env.nq, max(2, env.nq // 2 + 1), 2}):
        ct = env.at(t)
        h = env.gpu.load_ciphertext(ct, env.scale)
        m = env.gpu.eval_mult(h, h)
        got = env.gpu.store_ciphertext(m)
        exp = env.orc.mult(ct, ct, env.rlk)
        assert np.array_equal(got, exp), t
        sq = env.gpu.store_ciphertext(env.gpu.eval_square(h))
        assert np.array_equal(sq, exp)
        r = env.gpu.rescale(m)
        gr = env.gpu.store_ciphertext(r)
        er = env.orc.rescale(exp)
        assert np.array_equal(gr, er), t
        err = np.abs(env.decode(gr, env.scale ** 2 / env.mods[t - 1]) - env.z ** 2).max()
        assert err < 1e-4, err
        meta = env.gpu.meta(r)
        assert meta.towers == t - 1 and meta.noise_deg == 1


def test_mult_square_rotate_at_every_level(env):
    """Mult, Square and Rotate at every tower count (the reference's all-levels cases, test/OpenFheInterfaceTests.cu
    Mult/Square/Rotate all levels): bit-identical to the oracle."""
    levels = range(1, env.nq + 1) if env.nq <= 8 else sorted({1, 2, 3, env.nq // 3, env.nq // 2, env.nq - 1, env.nq})
    g, key = env.rot_key(2)
    for t in levels:
        ct = env.at(t)
        h = env.gpu.load_ciphertext(ct, env.scale)
        expect_mult = env.orc.mult(ct, ct, env.rlk)
        assert np.array_equal(env.gpu.store_ciphertext(env.gpu.eval_mult(h, h)), expect_mult), t
        assert np.array_equal(env.gpu.store_ciphertext(env.gpu.eval_square(h)), expect_mult), t
        assert np.array_equal(env.gpu.store_ciphertext(env.gpu.eval_rotate(h, 2)), env.orc.rotate(ct, g, key)), t
        env.gpu.free(h)


def test_add_sub_bit_exact(env):
    t = env.nq
    a = env.at(t)
    b = env.orc.encrypt(99, env.s, env.pt)
    ha, hb = env.gpu.load_ciphertext(a), env.gpu.load_ciphertext(b)
    assert np.array_equal(env.gpu.store_ciphertext(env.gpu.eval_add(ha, hb)), env.orc.add(a, b))
    assert np.array_equal(env.gpu.store_ciphertext(env.gpu.eval_sub(ha, hb)), env.orc.sub(a, b))


def test_errors_are_status_codes(env):
    import fideslib_gb300 as F
    h = env.gpu.load_ciphertext(env.at(env.nq))
    with pytest.raises(F.FidesError) as e:
        env.gpu.eval_automorphism(h, 3)  # no key for Galois element 3
    assert e.value.code == F.FIDES_ENOKEY
    with pytest.raises(F.FidesError):
        env.gpu.eval_add(h, 123456)
    h1 = env.gpu.load_ciphertext(env.at(1))
    with pytest.raises(F.FidesError):
        env.gpu.rescale(h1)


def test_batch_mixed_ops_same_alone_and_in_mix(env):
    """fides_eval_batch over rotations (two sharing one input), mults, squares, rescales and adds at ragged
    levels: every output equals the oracle and the same request issued alone."""
    import fideslib_gb300 as F
    rng = np.random.default_rng(17)
    nq = env.nq
    levels = [nq, max(2, nq - 1), max(2, nq // 2), 2, max(2, nq - 3), nq]
    hs = {t: env.gpu.load_ciphertext(env.at(t), env.scale) for t in set(levels)}
    g1, k1 = env.rot_key(1)
    g2, k2 = env.rot_key(-5)
    ops, expect = [], []
    for i, t in enumerate(levels):
        ct = env.at(t)
        kind = i % 4
        if kind == 0:
            ops.append((F.OP_ROTATE, hs[t], 0, 1))
            expect.append(env.orc.rotate(ct, g1, k1))
            ops.append((F.OP_ROTATE, hs[t], 0, -5))  # same input: shared ModUp
            expect.append(env.orc.rotate(ct, g2, k2))
        elif kind == 1:
            ops.append((F.OP_MULT, hs[t], hs[t], 0))
            expect.append(env.orc.mult(ct, ct, env.rlk))
        elif kind == 2:
            ops.append((F.OP_RESCALE, hs[t], 0, 0))
            expect.append(env.orc.rescale(ct))
        else:
            ops.append((F.OP_ADD, hs[t], hs[t], 0))
            expect.append(env.orc.add(ct, ct))
        ops.append((F.OP_SQUARE, hs[t], 0, 0))
        expect.append(env.orc.mult(ct, ct, env.rlk))
    outs = env.gpu.eval_batch(ops)
    for o, e, op in zip(outs, expect, ops):
        got = env.gpu.store_ciphertext(o)
        assert np.array_equal(got, e), op
        alone = env.gpu.store_ciphertext(env.gpu.eval_batch([op])[0])
        assert np.array_equal(alone, got), op


@pytest.mark.parametrize("chunk", [0, 1, 3])
def test_host_batch_pipelined_equals_oracle(env, chunk):
    """fides_eval_batch_host (inputs and outputs in host memory, chunks pipelined across copy and compute
    streams): every output equals the oracle's, for any chunking."""
    import fideslib_gb300 as F
    nq = env.nq
    levels = [nq, max(2, nq // 2), 2, nq, max(2, nq - 1)]
    g1, k1 = env.rot_key(1)
    ops, expect = [], []
    for i, t in enumerate(levels):
        ct = env.at(t)
        if i % 3 == 0:
            out = np.zeros_like(ct)
            ops.append((F.OP_ROTATE, ct, None, 1, out, env.scale))
            expect.append(env.orc.rotate(ct, g1, k1))
        elif i % 3 == 1:
            out = np.zeros_like(ct)
            ops.append((F.OP_MULT, ct, ct, 0, out, env.scale))
            expect.append(env.orc.mult(ct, ct, env.rlk))
        else:
            out = np.zeros((2, t - 1, env.N), dtype=np.uint64)
            ops.append((F.OP_RESCALE, ct, None, 0, out, env.scale))
            expect.append(env.orc.rescale(ct))
    metas = env.gpu.eval_batch_host(ops, chunk)
    for (code, a, b, idx, out, _), e, m in zip(ops, expect, metas):
        assert np.array_equal(out, e), code
        assert m.towers == e.shape[1]


def test_host_batch_automatic_chunks(env):
    """chunk = 0 with 21 requests runs chunks of 4, 8, 5 and 4 (the automatic schedule): every output equals the
    oracle's."""
    import fideslib_gb300 as F
    nq = env.nq
    g1, k1 = env.rot_key(1)
    ops, expect = [], []
    for i in range(21):
        t = 2 + i % (nq - 1)
        ct = env.at(t)
        out = np.zeros_like(ct)
        if i % 2:
            ops.append((F.OP_ROTATE, ct, None, 1, out, env.scale))
            expect.append(env.orc.rotate(ct, g1, k1))
        else:
            ops.append((F.OP_ADD, ct, ct, 0, out, env.scale))
            expect.append(env.orc.add(ct, ct))
    env.gpu.eval_batch_host(ops, 0)
    for (code, a, b, idx, out, _), e in zip(ops, expect):
        assert np.array_equal(out, e), code


def test_batched_rotations_full_ring_cfg3(engine_lib):
    """Config-3 shape at full size: N=2^16, 30 Q towers (60 + 29x50 bits), 10 special 60-bit primes, dnum=3.
    Four ciphertexts at levels 0, 13, 21, 28 rotated in one batch (two of them twice, sharing a ModUp):
    every residue bit-identical to the oracle."""
    import fideslib_gb300 as F
    logN = 16
    N = 1 << logN
    mods = O.make_moduli(logN, [60] + [50] * 29, [60] * 10)
    gpu = F.CryptoContext(logN, mods, 10, 3)
    orc = O.Ctx(N, 30, 10, 3, mods, threads=16)
    rng = np.random.default_rng(0x5EED0003)
    keys = {}
    for idx in (1, -16, 1024):
        g = orc.galois(idx)
        k = np.zeros(orc.key_shape(), dtype=np.uint64)
        for j in range(40):
            k[:, :, j] = rng.integers(0, mods[j], (2, 3, N), dtype=np.uint64)
        keys[idx] = (g, k)
        gpu.load_rotation_key(g, k)
    cts, ops = {}, []
    for t in (30, 17, 9, 2):
        ct = np.stack([np.stack([rng.integers(0, mods[j], N, dtype=np.uint64) for j in range(t)]) for _ in range(2)])
        cts[t] = (ct, gpu.load_ciphertext(ct))
    plan = [(30, 1), (30, -16), (17, 1024), (9, 1), (2, -16), (2, 1024)]
    outs = gpu.eval_batch([(F.OP_ROTATE, cts[t][1], 0, idx) for t, idx in plan])
    for (t, idx), o in zip(plan, outs):
        g, k = keys[idx]
        assert np.array_equal(gpu.store_ciphertext(o), orc.rotate(cts[t][0], g, k)), (t, idx)
    gpu.close()


def test_every_inner_product_tile_bit_exact(env):
    """The key inner product's tile (coefficient pairs per thread), tuned on the first key-switch launch of at least
    16 ciphertexts: every tile the ring allows gives the oracle's residues for a batch of rotations at ragged levels
    (a dnum-4 ring takes the three-product accumulation, the others the four-product one)."""
    import fideslib_gb300 as F
    ts = [env.nq, max(1, env.nq // 2), 1, max(1, env.nq - 1)]
    cases = []
    for k in range(16):
        t, index = ts[k % 4], (1, -5)[k % 2]
        g, key = env.rot_key(index)
        ct = np.ascontiguousarray(env.orc.encrypt(500 + k, env.s, env.pt)[:, :t])
        cases.append((env.gpu.load_ciphertext(ct, env.scale), index, env.orc.rotate(ct, g, key)))
    ops = [(F.OP_ROTATE, h, 0, index) for h, index, _ in cases]

    def check(tag):
        outs = env.gpu.eval_batch(ops)
        for o, (_, index, exp) in zip(outs, cases):
            assert np.array_equal(env.gpu.store_ciphertext(o), exp), (tag, index)
            env.gpu.free(o)

    check("first batch")  # 16 jobs: tunes the tile if no earlier batch did
    tun = env.gpu.ks_tuning()
    allowed = [i for i in (1, 2, 4, 8, 16) if i <= env.N // 512]
    assert tun["pairs_per_thread"] in allowed, tun
    assert all(tun["ms_1_2_4_8_16"][k] > 0 for k, i in enumerate((1, 2, 4, 8, 16)) if i in allowed), tun
    try:
        for iters in (1, 2, 4, 8, 16):
            if iters not in allowed:
                with pytest.raises(F.FidesError):
                    env.gpu.set_ks_tile(iters)
                continue
            env.gpu.set_ks_tile(iters)
            check(iters)
    finally:
        env.gpu.set_ks_tile(tun["pairs_per_thread"])
    for h, _, _ in cases:
        env.gpu.free(h)
