"""CKKS encoding / decoding on the GPU (fides_pt_encode, fides_pt_decode, fides_lt_create_slots) against the
oracle's encoder (a different FFT: the 2N-point canonical embedding), within floating-point tolerance."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

LOGN = 12
N = 1 << LOGN


@pytest.fixture(scope="module")
def env(engine_lib):
    import fideslib_gb300 as F
    mods = O.make_moduli(LOGN, [60] + [45] * 5, [60] * 2)
    gpu = F.CryptoContext(LOGN, mods, 2, 3)
    orc = O.Ctx(N, 6, 2, 3, mods, threads=8)
    return dict(F=F, gpu=gpu, orc=orc, mods=mods)


def centred(orc, pt, q):
    """Centred integer coefficients of tower 0 (Python ints: exact beyond 2^53)."""
    c = orc.to_coeff(np.ascontiguousarray(pt[:1]))[0]
    return [int(x) - q if int(x) > q // 2 else int(x) for x in c]


@pytest.mark.parametrize("slots,scale", [(1, 2.0 ** 40), (16, 2.0 ** 40), (N // 2, 2.0 ** 40), (N // 2, 2.0 ** 55)])
def test_encode_matches_oracle_and_decodes(env, slots, scale):
    gpu, orc, mods = env["gpu"], env["orc"], env["mods"]
    rng = np.random.default_rng(slots)
    z = rng.uniform(-1, 1, slots) + 1j * rng.uniform(-1, 1, slots)
    h = gpu.encode(z, scale, 4)
    got = gpu.store_plaintext(h, 4)
    ref = orc.encode(z, scale, 4)
    # the two FFTs differ in rounding only: coefficients agree to a few units in the last place of scale * m
    c0, r0 = centred(orc, got, mods[0]), centred(orc, ref, mods[0])
    diff = max(abs(a - b) for a, b in zip(c0, r0))
    assert diff <= max(1.0, scale * 2.0 ** -48), diff
    # every tower carries the same integer coefficient vector
    for j in range(1, 4):
        cj = orc.to_coeff(np.ascontiguousarray(got[j:j + 1]), [j])[0]
        assert [int(x) for x in cj] == [v % mods[j] for v in c0]
    dec = gpu.decode(h, slots)
    assert np.abs(dec - z).max() < 1e-9
    assert np.abs(orc.decode(got, scale, slots) - z).max() < 1e-9
    gpu.free_plaintext(h)


def test_encode_rejects_overflow(env):
    F, gpu = env["F"], env["gpu"]
    with pytest.raises(F.FidesError):
        gpu.encode(np.ones(8), 2.0 ** 70, 2)


def test_linear_transform_from_slot_diagonals(env):
    """A transform whose diagonals are encoded on the GPU gives the same slots as one built from the oracle's
    encodings (residues may differ by rounding, so the comparison is on decrypted slots)."""
    from tests import boot_plan as BP
    gpu, orc = env["gpu"], env["orc"]
    n, sc = 64, 2.0 ** 45
    s = orc.secret(3)
    (M, stride, r), = BP.factors(n, 1, inverse=False)
    bs, gs, base, slots = BP.bsgs_layout(M, n, stride, r)
    present = np.array([x is not None for x in slots])
    diag = np.array([x if x is not None else np.zeros(n) for x in slots])
    fac = BP.Factor(orc, M, n, stride, r, 6, sc)
    need = fac.rotations(n, N)
    for i, idx in enumerate(sorted(need)):
        g = orc.galois(idx)
        gpu.load_rotation_key(g, orc.rot_key(40 + i, s, g))
    lt_gpu = gpu.lt_create_slots(bs, gs, diag, present, sc, 6, stride=stride, base=base)
    lt_orc = fac.create(gpu, sc)
    rng = np.random.default_rng(5)
    z = rng.uniform(-1, 1, n) + 1j * rng.uniform(-1, 1, n)
    ct = orc.encrypt(6, s, orc.encode(z, sc, 6))
    h = gpu.load_ciphertext(ct, sc)
    a = orc.decode(orc.decrypt(s, gpu.store_ciphertext(gpu.eval_linear_transform(h, lt_gpu))), sc * sc, n)
    b = orc.decode(orc.decrypt(s, gpu.store_ciphertext(gpu.eval_linear_transform(h, lt_orc))), sc * sc, n)
    expect = BP.apply(M, z)
    assert np.abs(a - expect).max() < 1e-6
    assert np.abs(a - b).max() < 1e-9
