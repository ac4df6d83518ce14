"""Bootstrap building blocks on the GPU: plaintext and scalar ops, level reduction, ModRaise and the
baby-step/giant-step linear transform — bit-identical to the oracle, with decrypted precision stated."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def double_residue(v: float, q: int) -> int:
    """round(v) mod q for the double value v (round half to even, as nearbyint)."""
    a = round(abs(v))
    r = a % q
    return (q - r) % q if v < 0 else r


@pytest.fixture(scope="module")
def env(engine_lib):
    import fideslib_gb300 as F
    logN = 12
    N = 1 << logN
    mods = O.make_moduli(logN, [60] + [45] * 7, [60] * 4)  # P (240 bits) well above a digit (<= 150 bits)
    gpu = F.CryptoContext(logN, mods, 4, 3)
    orc = O.Ctx(N, 8, 4, 3, mods, threads=8)
    s = orc.secret(5)
    rng = np.random.default_rng(21)
    z = rng.uniform(-1, 1, N // 2) + 1j * rng.uniform(-1, 1, N // 2)
    scale = 2.0 ** 45
    ct = orc.encrypt(9, s, orc.encode(z, scale, 8))
    return dict(F=F, gpu=gpu, orc=orc, s=s, z=z, scale=scale, ct=ct, mods=mods, N=N, rng=rng)


def dec(e, ct, scale):
    return e["orc"].decode(e["orc"].decrypt(e["s"], ct), scale, e["N"] // 2)


def test_plain_ops_bit_exact(env):
    gpu, orc = env["gpu"], env["orc"]
    w = env["rng"].uniform(-1, 1, env["N"] // 2)
    pt = orc.encode(w, env["scale"], 8)
    h = gpu.load_ciphertext(env["ct"], env["scale"])
    hp = gpu.load_plaintext(pt, env["scale"])
    for mode, fn in ((0, gpu.eval_mult_plain), (1, gpu.eval_add_plain), (2, gpu.eval_sub_plain)):
        got = gpu.store_ciphertext(fn(h, hp))
        assert np.array_equal(got, orc.plain_op(env["ct"], pt, mode)), mode
    m = gpu.store_ciphertext(gpu.eval_mult_plain(h, hp))
    err = np.abs(dec(env, m, env["scale"] ** 2) - env["z"] * w).max()
    assert err < 1e-6, err


@pytest.mark.parametrize("k", [3, -7, 1 << 55, -(1 << 57) + 11])
def test_mult_int_bit_exact(env, k):
    gpu, orc, mods = env["gpu"], env["orc"], env["mods"]
    h = gpu.load_ciphertext(env["ct"], env["scale"])
    got = gpu.store_ciphertext(gpu.eval_mult_int(h, k))
    mul = [k % q for q in mods[:8]]
    assert np.array_equal(got, orc.scalar_op(env["ct"], mul, [0] * 8))


def test_mult_and_add_scalar_bit_exact_and_precise(env):
    gpu, orc, mods, sc = env["gpu"], env["orc"], env["mods"], env["scale"]
    h = gpu.load_ciphertext(env["ct"], sc)
    v, cscale = 0.3701, 2.0 ** 40
    got = gpu.store_ciphertext(gpu.eval_mult_scalar(h, v, cscale))
    mul = [double_residue(v * cscale, q) for q in mods[:8]]
    assert np.array_equal(got, orc.scalar_op(env["ct"], mul, [0] * 8))
    assert np.abs(dec(env, got, sc * cscale) - v * env["z"]).max() < 1e-7
    got = gpu.store_ciphertext(gpu.eval_add_scalar(h, -0.5))
    add = [double_residue(-0.5 * sc, q) for q in mods[:8]]
    assert np.array_equal(got, orc.scalar_op(env["ct"], [1] * 8, add))
    assert np.abs(dec(env, got, sc) - (env["z"] - 0.5)).max() < 1e-7


def test_level_reduce_and_mod_raise(env):
    gpu, orc = env["gpu"], env["orc"]
    h = gpu.load_ciphertext(env["ct"], env["scale"])
    low = gpu.level_reduce(h, 1)
    got_low = gpu.store_ciphertext(low)
    assert np.array_equal(got_low, env["ct"][:, :1])
    raised = gpu.store_ciphertext(gpu.mod_raise(low, 8))
    assert np.array_equal(raised, orc.mod_raise(np.ascontiguousarray(env["ct"][:, :1]), 8))
    # the raised ciphertext decrypts, modulo q_0, to the same plaintext as the level-0 one
    d_low = orc.to_coeff(orc.decrypt(env["s"], np.ascontiguousarray(got_low)))[0]
    d_hi = orc.to_coeff(orc.decrypt(env["s"], raised))
    assert np.array_equal(d_hi[0], d_low)


def test_linear_transform_bsgs(env):
    """y = sum_{i < bs*gs} d_i (.) rot_i(z) for a banded slot matrix: bit-exact against the oracle replay of
    the same baby-step/giant-step order, and within 1e-5 of the numpy matrix-vector product."""
    F, gpu, orc, N = env["F"], env["gpu"], env["orc"], env["N"]
    n = N // 2
    bs, gs, sc = 4, 3, env["scale"]
    rng = np.random.default_rng(4)
    d = rng.uniform(-1, 1, (bs * gs, n))
    present = np.ones(bs * gs, dtype=bool)
    present[5] = False  # a zero diagonal
    diags = np.zeros((bs * gs, 8, N), dtype=np.uint64)
    for g in range(gs):
        for b in range(bs):
            i = g * bs + b
            if present[i]:
                diags[i] = orc.encode(np.roll(d[i], g * bs), sc, 8)  # pre-rotated by -g*bs
    keys = {}
    for idx in list(range(1, bs)) + [g * bs for g in range(1, gs)]:
        gl = orc.galois(idx)
        keys[idx] = (gl, orc.rot_key(300 + idx, env["s"], gl))
        gpu.load_rotation_key(gl, keys[idx][1])
    lt = gpu.lt_create(bs, gs, diags, present, sc)
    h = gpu.load_ciphertext(env["ct"], sc)
    got = gpu.store_ciphertext(gpu.eval_linear_transform(h, lt))
    # oracle replay: baby steps, inner sums, giant steps, sum
    ct = env["ct"]
    baby = [ct] + [orc.rotate(ct, keys[b][0], keys[b][1]) for b in range(1, bs)]
    total = None
    for g in range(gs):
        inner = None
        for b in range(bs):
            i = g * bs + b
            if not present[i]:
                continue
            term = orc.plain_op(baby[b], diags[i], 0)
            inner = term if inner is None else orc.add(inner, term)
        if g > 0:
            inner = orc.rotate(inner, keys[g * bs][0], keys[g * bs][1])
        total = inner if total is None else orc.add(total, inner)
    assert np.array_equal(got, total)
    z = env["z"]
    expect = sum(d[i] * np.roll(z, -i) for i in range(bs * gs) if present[i])
    err = np.abs(dec(env, got, sc * sc) - expect).max()
    assert err < 1e-5, err
    gpu.lt_free(lt)


@pytest.mark.parametrize("towers", [8, 5])
def test_linear_transform_double_hoisted(env, towers):
    """A strided SlotsToCoeffs factor whose diagonals carry the special primes (fides_lt_create_strided_ext): the
    double-hoisted evaluation (baby steps and inner sums in the extended basis, giant-step sums ModDowned in c1
    only, one final ModDown) is bit-exact against its oracle replay for a batch of three ciphertexts, also below
    the transform's top level, and decrypts to the factor's matrix-vector product."""
    from fideslib_gb300 import bootplan as B
    from tests import boot_plan as BP
    gpu, orc, N, s = env["gpu"], env["orc"], env["N"], env["s"]
    n, sc = N // 2, env["scale"]
    M, stride, r = BP.factors(n, 3, inverse=False)[1]
    f = BP.Factor(orc, M, n, stride, r, 8, sc, ext=True, bs=B.ext_baby_steps(r))
    assert f.diags.shape[1] == 8 + 4
    keys = {}
    for i, idx in enumerate(sorted(f.rotations(n, N))):
        g = orc.galois(idx)
        keys[idx] = (g, orc.rot_key(500 + i, s, g))
        gpu.load_rotation_key(g, keys[idx][1])
    lt = f.create(gpu, sc)
    rng = np.random.default_rng(31 + towers)
    zs = [(rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)) * 0.5 for _ in range(3)]
    cts = [orc.encrypt(40 + k, s, orc.encode(z, sc, towers)) for k, z in enumerate(zs)]
    outs = gpu.eval_linear_transform_batch([gpu.load_ciphertext(c, sc) for c in cts], lt)
    for c, z, o in zip(cts, zs, outs):
        got = gpu.store_ciphertext(o)
        assert np.array_equal(got, f.replay(orc, c, keys, N))
        err = np.abs(dec(env, got, sc * sc) - B.apply(M, z)).max()
        assert err < 1e-6, err
    gpu.lt_free(lt)
