"""EvalChebyshevSeries and the double-angle iterations (the EvalMod core) on the GPU: bit-identical to an
op-for-op oracle replay of the recipe documented in fideslib_gb300/csrc/poly_eval.cu, and within the stated
precision of numpy's Chebyshev evaluation of the decrypted slots."""
import numpy as np
import numpy.polynomial.chebyshev as C
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


from tests.replay import Sim  # noqa: E402


@pytest.fixture(scope="module")
def env(engine_lib):
    import fideslib_gb300 as F
    logN = 12
    N = 1 << logN
    nq = 12
    mods = O.make_moduli(logN, [60] + [45] * (nq - 1), [60] * 4)
    gpu = F.CryptoContext(logN, mods, 4, 3)
    orc = O.Ctx(N, nq, 4, 3, mods, threads=8)
    s = orc.secret(8)
    rlk = orc.relin_key(9, s)
    gpu.load_eval_mult_key(rlk)
    rng = np.random.default_rng(13)
    return dict(gpu=gpu, orc=orc, s=s, N=N, nq=nq, mods=mods, rng=rng, sim=Sim(orc, mods, rlk))


@pytest.mark.parametrize("lo,hi,fn,deg", [(-1.0, 1.0, lambda x: np.exp(x) / 3, 12),
                                           (-2.0, 2.0, lambda x: np.cos(np.pi * x / 4), 9)])
def test_chebyshev_series(env, lo, hi, fn, deg):
    gpu, orc, N = env["gpu"], env["orc"], env["N"]
    x = env["rng"].uniform(lo, hi, N // 2)
    sc = 2.0 ** 45
    ct = orc.encrypt(3, env["s"], orc.encode(x + 0j, sc, env["nq"]))
    coeffs = C.chebinterpolate(lambda u: fn(lo + (u + 1) * (hi - lo) / 2), deg)
    h = gpu.load_ciphertext(ct, sc)
    out = gpu.eval_chebyshev(h, coeffs, lo, hi, sc)
    got = gpu.store_ciphertext(out)
    ref, ref_scale = env["sim"].chebyshev((ct, sc), list(coeffs), lo, hi, sc)
    assert np.array_equal(got, ref)
    meta = gpu.meta(out)
    assert abs(meta.scale / ref_scale - 1) < 1e-12
    val = orc.decode(orc.decrypt(env["s"], got), meta.scale, N // 2).real
    expect = C.chebval((2 * x - lo - hi) / (hi - lo), coeffs)
    err = np.abs(val - expect).max()
    assert err < 1e-5, err
    assert np.abs(val - fn(x)).max() < 1e-4


def test_double_angle(env):
    gpu, orc, N = env["gpu"], env["orc"], env["N"]
    x = env["rng"].uniform(-1, 1, N // 2)
    sc = 2.0 ** 45
    ct = orc.encrypt(4, env["s"], orc.encode(x + 0j, sc, env["nq"]))
    h = gpu.load_ciphertext(ct, sc)
    out = gpu.eval_double_angle(h, 2)
    got = gpu.store_ciphertext(out)
    sim = env["sim"]
    y = (ct, sc)
    for _ in range(2):
        y = sim.add_scalar(sim.mult_int(sim.rescale(sim.mult(y, y)), 2), -1.0)
    assert np.array_equal(got, y[0])
    val = orc.decode(orc.decrypt(env["s"], got), gpu.meta(out).scale, N // 2).real
    assert np.abs(val - np.cos(4 * np.arccos(x))).max() < 1e-5
