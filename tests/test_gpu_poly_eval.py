"""EvalChebyshevSeries and the double-angle iterations (the EvalMod core) on the GPU: bit-identical to an
op-for-op oracle replay of the recipe documented in fideslib_gb300/csrc/poly_eval.cu, and within the stated
precision of numpy's Chebyshev evaluation of the decrypted slots."""
import numpy as np
import numpy.polynomial.chebyshev as C
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def double_residue(v: float, q: int) -> int:
    a = round(abs(v))
    r = a % q
    return (q - r) % q if v < 0 else r


class Sim:
    """Oracle replay with the engine's metadata rules (scale after rescale = scale / dropped prime)."""

    def __init__(self, orc, mods, rlk):
        self.orc, self.mods, self.rlk = orc, mods, rlk

    def t(self, a):
        return a[0].shape[1]

    def mult(self, a, b):
        return (self.orc.mult(a[0], b[0], self.rlk), a[1] * b[1])

    def rescale(self, a):
        return (self.orc.rescale(a[0]), a[1] / self.mods[self.t(a) - 1])

    def mult_int(self, a, k):
        return (self.orc.scalar_op(a[0], [k % q for q in self.mods[:self.t(a)]], [0] * self.t(a)), a[1])

    def add_scalar(self, a, v):
        add = [double_residue(v * a[1], q) for q in self.mods[:self.t(a)]]
        return (self.orc.scalar_op(a[0], [1] * self.t(a), add), a[1])

    def mult_scalar(self, a, v, cs):
        mul = [double_residue(v * cs, q) for q in self.mods[:self.t(a)]]
        return (self.orc.scalar_op(a[0], mul, [0] * self.t(a)), a[1] * cs)

    def drop(self, a, t):
        return (np.ascontiguousarray(a[0][:, :t]), a[1]) if self.t(a) != t else a

    def add(self, a, b):
        return (self.orc.add(a[0], b[0]), a[1])

    def sub(self, a, b):
        return (self.orc.sub(a[0], b[0]), a[1])

    def chebyshev(self, x, c, lo, hi, cs):
        d = len(c) - 1
        T = [None] * (d + 1)
        if lo == -1.0 and hi == 1.0:
            T[1] = x
        else:
            u = self.rescale(self.mult_scalar(x, 2.0 / (hi - lo), cs))
            T[1] = self.add_scalar(u, -(hi + lo) / (hi - lo))
        for k in range(2, d + 1):
            if k % 2 == 0:
                m2 = self.mult_int(self.rescale(self.mult(T[k // 2], T[k // 2])), 2)
                T[k] = self.add_scalar(m2, -1.0)
            else:
                A, B = T[(k - 1) // 2], T[(k + 1) // 2]
                t = min(self.t(A), self.t(B))
                m2 = self.mult_int(self.rescale(self.mult(self.drop(A, t), self.drop(B, t))), 2)
                T[k] = self.sub(m2, self.drop(T[1], self.t(m2)))
        tmin = min(self.t(T[k]) for k in range(1, d + 1) if c[k] != 0)
        acc = None
        for k in range(1, d + 1):
            if c[k] == 0:
                continue
            term = self.mult_scalar(self.drop(T[k], tmin), c[k], cs)
            acc = term if acc is None else self.add(acc, term)
        return self.add_scalar(self.rescale(acc), c[0])


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
