"""Extended-basis ciphertexts on the GPU: EvalFastRotationExt, products with extended plaintexts, sums and
KeySwitchDown (fides_eval_fast_rotation_ext, fides_ext_mult_plain, fides_ext_add, fides_key_switch_down) —
every residue bit-identical to the oracle replay, and the decrypted result equal to the plain linear map.

The hoisted linear map sum_i v_i (.) rot_{r_i}(z) is the pattern OpenFHE's users (and the reference's
LinearTransform, src/CKKS/LinearTransform.cu:63-190) build from these calls: one ModUp, one extended-basis inner
product per index, one ModDown at the end."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

LOGN = 12
N = 1 << LOGN
QB, PB, DNUM = [60] + [45] * 7, [60] * 4, 3  # P (240 bits) above every digit (<= 150 bits)
NQ, NP = len(QB), len(PB)
SCALE = 2.0 ** 45
INDICES = [1, 3, -2, 0]


@pytest.fixture(scope="module")
def env(engine_lib):
    import fideslib_gb300 as F
    mods = O.make_moduli(LOGN, QB, PB)
    gpu = F.CryptoContext(LOGN, mods, NP, DNUM)
    orc = O.Ctx(N, NQ, NP, DNUM, mods, threads=8)
    s = orc.secret(0x5EED0041)
    keys = {}
    for i, idx in enumerate(INDICES):
        if idx:
            g = orc.galois(idx)
            keys[idx] = (g, orc.rot_key(700 + i, s, g))
            gpu.load_rotation_key(g, keys[idx][1])
    return dict(F=F, gpu=gpu, orc=orc, s=s, keys=keys, mods=mods)


def replay_rotation_ext(e, ct, idx, add_first):
    orc, t = e["orc"], ct.shape[1]
    ids = orc.ext_ids(t)
    P = 1
    for p in e["mods"][NQ:]:
        P *= int(p)
    lifted = np.zeros((2, t + NP, N), dtype=np.uint64)
    lifted[:, :t] = orc.scalar_op(ct, [P % int(q) for q in e["mods"][:t]], [0] * t)
    if idx == 0:
        out = lifted.copy()
        if not add_first:
            out[0] = 0
        return out
    g, key = e["keys"][idx]
    x = orc.ks_inner(orc.modup(np.ascontiguousarray(ct[1]), t), t, key)
    if add_first:
        x[0] = orc.ew(x[0], lifted[0], ids, 1)
    return orc.automorph(x, g)


@pytest.mark.parametrize("towers", [NQ, 5])
def test_hoisted_linear_map_extended_basis(env, towers):
    gpu, orc, s = env["gpu"], env["orc"], env["s"]
    rng = np.random.default_rng(towers)
    z = (rng.uniform(-1, 1, N // 2) + 1j * rng.uniform(-1, 1, N // 2)) * 0.5
    ct = orc.encrypt(33 + towers, s, orc.encode(z, SCALE, towers))
    h = gpu.load_ciphertext(ct, SCALE)
    ids = orc.ext_ids(towers)
    pre = gpu.fast_rotation_precompute(h)
    exts = gpu.eval_fast_rotation_ext(h, INDICES, add_first=True, pre=pre)
    exts_here = gpu.eval_fast_rotation_ext(h, INDICES, add_first=True)  # ModUp inside the call
    vs, pts, total, total_ref = [], [], None, None
    for k, (idx, x, y) in enumerate(zip(INDICES, exts, exts_here)):
        ref = replay_rotation_ext(env, ct, idx, True)
        got = gpu.store_ext(x, towers)
        assert np.array_equal(got, ref), idx
        assert np.array_equal(gpu.store_ext(y, towers), ref), idx
        v = rng.uniform(-1, 1, N // 2)
        pt = orc.encode(v, SCALE, len(ids), tower_ids=ids)
        m = gpu.ext_mult_plain(x, gpu.load_plaintext_ext(pt, towers, SCALE))
        m_ref = orc.ew(ref, pt, ids, 0)
        assert np.array_equal(gpu.store_ext(m, towers), m_ref), idx
        total = m if total is None else gpu.ext_add(total, m)
        total_ref = m_ref if total_ref is None else orc.ew(total_ref, m_ref, ids, 1)
        vs.append((idx, v))
    assert np.array_equal(gpu.store_ext(total, towers), total_ref)
    down = gpu.key_switch_down(total)
    got = gpu.store_ciphertext(down)
    ref = np.stack([orc.moddown(np.ascontiguousarray(total_ref[p]), towers) for p in range(2)])
    assert np.array_equal(got, ref)
    assert abs(gpu.meta(down).scale / SCALE ** 2 - 1) < 1e-12
    expect = sum(v * np.roll(z, -idx) for idx, v in vs)
    dec = orc.decode(orc.decrypt(s, got), SCALE ** 2, N // 2)
    err = np.abs(dec - expect).max()
    print(f"hoisted extended-basis map at {towers} towers: max slot error {err:.2e}")
    assert err < 1e-6, err
    gpu.precompute_free(pre)


def test_rotation_ext_without_first_term(env):
    """add_first = 0 leaves c0 out (the caller adds P * c0 once for a sum of rotations); KeySwitchDown of the sum
    of the extended rotation and the lifted c0 decrypts to the rotation."""
    gpu, orc, s = env["gpu"], env["orc"], env["s"]
    rng = np.random.default_rng(5)
    z = rng.uniform(-1, 1, N // 2) + 1j * rng.uniform(-1, 1, N // 2)
    ct = orc.encrypt(51, s, orc.encode(z, SCALE, NQ))
    h = gpu.load_ciphertext(ct, SCALE)
    for idx in (3, 0):
        x = gpu.eval_fast_rotation_ext(h, [idx], add_first=False)[0]
        assert np.array_equal(gpu.store_ext(x, NQ), replay_rotation_ext(env, ct, idx, False))
    x = gpu.eval_fast_rotation_ext(h, [1], add_first=True)[0]
    dec = orc.decode(orc.decrypt(s, gpu.store_ciphertext(gpu.key_switch_down(x))), SCALE, N // 2)
    assert np.abs(dec - np.roll(z, -1)).max() < 1e-6


def test_extended_handles_are_separate(env):
    import fideslib_gb300 as F
    gpu, orc, s = env["gpu"], env["orc"], env["s"]
    ct = orc.encrypt(52, s, orc.encode(np.zeros(N // 2), SCALE, 3))
    h = gpu.load_ciphertext(ct, SCALE)
    x = gpu.eval_fast_rotation_ext(h, [1])[0]
    with pytest.raises(F.FidesError):  # a regular op does not take an extended-basis ciphertext
        gpu.rescale(x)
    with pytest.raises(F.FidesError):  # and the extended ops do not take a regular one
        gpu.key_switch_down(h)
    pt = gpu.load_plaintext(orc.encode(np.ones(N // 2), SCALE, 3), SCALE)
    with pytest.raises(F.FidesError):  # a plaintext without special rows
        gpu.ext_mult_plain(x, pt)
    gpu.free(x)
    with pytest.raises(F.FidesError):
        gpu.free(x)
