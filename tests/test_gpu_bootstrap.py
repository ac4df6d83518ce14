"""End-to-end CKKS bootstrapping on the GPU (fides_eval_bootstrap / fides_eval_bootstrap_batch).

Ring N=2^12, q_0 of 60 bits and 55-bit towers, 4 special primes of 60 bits (P above every digit's modulus).
Two shapes: 16 sparse slots with a one-factor level budget, and 2048 full slots with the level budget {3, 3}
and sparse-secret encapsulation (main secret of Hamming weight 192, encapsulated under weight 32).  The
CoeffsToSlots / SlotsToCoeffs factors come from the factored special FFT (tests/boot_plan.py) and are encoded by
the oracle, the way the reference receives its bootstrap plaintexts from OpenFHE; the full-slot shape uses
double-hoisted factors (diagonals also at the special primes), the sparse one the ModDown-per-rotation form.  Every output residue is
checked against an op-for-op oracle replay of the recipe documented in fideslib_gb300/csrc/bootstrap.cu, and
the decrypted slots against the input message (precision stated).  A batch of bootstraps in flight together
must give exactly the single-call results."""
import numpy as np
import numpy.polynomial.chebyshev as C
import pytest

import oracle as O
from tests import boot_plan as BP
from tests.replay import Sim

pytestmark = pytest.mark.gpu

LOGN = 12
N = 1 << LOGN
NQ, NP, DNUM = 22, 4, 6  # digits of 4 towers (<= 220 bits) under P = 240 bits
DELTA_M = DELTA_PT = 2.0 ** 55  # q_0 / DELTA_M = 32 keeps the EvalMod gain small
R_DOUBLE = 3
CHEB_DEG = 47
B_RANGE = 12.5


class Setup:
    def __init__(self, slots, budget, sse, seed, ext=False):
        import fideslib_gb300 as F
        from fideslib_gb300.bootplan import ext_baby_steps
        self.F, self.slots = F, slots
        self.mods = O.make_moduli(LOGN, [60] + [55] * (NQ - 1), [60] * NP)
        self.gpu = F.CryptoContext(LOGN, self.mods, NP, DNUM)
        self.orc = orc = O.Ctx(N, NQ, NP, DNUM, self.mods, threads=16)
        self.s = orc.secret(seed, hamming_weight=192 if sse else 32)
        self.rlk = orc.relin_key(seed + 1, self.s)
        self.gpu.load_eval_mult_key(self.rlk)
        self.sse = None
        if sse:
            s_sparse = orc.secret(seed + 2, hamming_weight=32)
            self.sse = (orc.switch_key(seed + 3, self.s, s_sparse), orc.switch_key(seed + 4, s_sparse, self.s))
            self.gpu.load_switch_key(10, self.sse[0])
            self.gpu.load_switch_key(11, self.sse[1])
        bs = ext_baby_steps if ext else (lambda r: None)  # noqa: E731
        self.cts = [BP.Factor(orc, M, slots, stride, r, NQ, DELTA_PT, ext=ext, bs=bs(r))
                    for M, stride, r in BP.factors(slots, budget[0], inverse=True, scale=slots / N)]
        self.stc = [BP.Factor(orc, M, slots, stride, r, NQ, DELTA_PT, ext=ext, bs=bs(r))
                    for M, stride, r in BP.factors(slots, budget[1], inverse=False)]
        need = set()
        for f in self.cts + self.stc:
            need |= f.rotations(slots, N)
        r = slots
        while r < N // 2:
            need.add(r)
            r <<= 1
        self.keys = {}
        for i, idx in enumerate(sorted(need)):
            g = orc.galois(idx)
            self.keys[idx] = (g, orc.rot_key(seed + 100 + i, self.s, g))
            self.gpu.load_rotation_key(g, self.keys[idx][1])
        self.conj = (2 * N - 1, orc.rot_key(seed + 7, self.s, 2 * N - 1))
        self.gpu.load_rotation_key(*self.conj)
        self.K = self.mods[0] / DELTA_M
        self.lo, self.hi = -B_RANGE * self.K, B_RANGE * self.K
        f = lambda r: np.cos(2 * np.pi * (r / self.K - 0.25) / 2 ** R_DOUBLE)  # noqa: E731
        lo, hi = self.lo, self.hi
        self.coeffs = C.chebinterpolate(lambda u: f(lo + (u + 1) * (hi - lo) / 2), CHEB_DEG)
        self.plan = F.BootstrapPlan.make(slots, NQ, [f.create(self.gpu, DELTA_PT) for f in self.cts],
                                         [f.create(self.gpu, DELTA_PT) for f in self.stc], self.coeffs, R_DOUBLE,
                                         self.lo, self.hi, DELTA_PT, sse_keys=(10, 11) if sse else None)

    def message(self, seed):
        rng = np.random.default_rng(seed)
        z = (rng.uniform(-1, 1, self.slots) + 1j * rng.uniform(-1, 1, self.slots)) * 0.5
        return z, self.orc.encrypt(seed, self.s, self.orc.encode(z, DELTA_M, 1))

    def replay(self, ct, prescale=0.0):
        """The recipe of fideslib_gb300/csrc/bootstrap.cu on the oracle, op for op."""
        orc, sim = self.orc, Sim(self.orc, self.mods, self.rlk)
        scale_in = DELTA_M
        if prescale:
            ct, scale_in = sim.rescale(sim.mult_scalar((ct, DELTA_M), prescale, float(self.mods[ct.shape[1] - 1])))
        K = self.mods[0] / scale_in
        x = ct
        if self.sse:
            x = orc.key_switch(np.ascontiguousarray(x[:, :1]), self.sse[0])
        x = orc.mod_raise(x, NQ)
        if self.sse:
            x = orc.key_switch(x, self.sse[1])
        r = self.slots
        while r < N // 2:
            x = orc.add(x, orc.rotate(x, *self.keys[r]))
            r <<= 1
        v = (x, scale_in)
        for f in self.cts:
            v = sim.rescale((f.replay(orc, v[0], self.keys, N), v[1] * DELTA_PT))
        c = orc.rotate(v[0], *self.conj)
        halves = [(orc.add(v[0], c), v[1]), (orc.mult_monomial(orc.sub(v[0], c), 3 * N // 2), v[1])]
        modded = []
        for h in halves:
            y = sim.chebyshev(h, list(self.coeffs), self.lo, self.hi, DELTA_PT)
            for _ in range(R_DOUBLE):
                y = sim.add_scalar(sim.mult_int(sim.rescale(sim.mult(y, y)), 2), -1.0)
            modded.append(sim.rescale(sim.mult_scalar(y, K / (2 * np.pi), DELTA_PT)))
        w = (orc.add(modded[0][0], orc.mult_monomial(modded[1][0], N // 2)), modded[0][1])
        for f in self.stc:
            w = sim.rescale((f.replay(orc, w[0], self.keys, N), w[1] * DELTA_PT))
        return w

    def precision(self, got, scale, z):
        dec = self.orc.decode(self.orc.decrypt(self.s, got), scale, self.slots)
        err = np.abs(dec - z).max()
        return err, -np.log2(err)


def check(setup, z, ct, tol):
    gpu = setup.gpu
    out = gpu.eval_bootstrap(gpu.load_ciphertext(ct, DELTA_M), setup.plan)
    got = gpu.store_ciphertext(out)
    meta = gpu.meta(out)
    ref, ref_scale = setup.replay(ct)
    assert np.array_equal(got, ref)
    assert abs(meta.scale / ref_scale - 1) < 1e-9
    err, bits = setup.precision(got, meta.scale, z)
    print(f"bootstrap n={setup.slots}: {meta.towers} towers left, max slot error {err:.3e} ({bits:.1f} bits)")
    assert err < tol, err
    return got, meta


def test_bootstrap_sparse_slots():
    st = Setup(slots=16, budget=(1, 1), sse=False, seed=0x5EED0005)
    z, ct = st.message(77)
    _, meta = check(st, z, ct, 1e-3)
    assert meta.towers >= 2


def test_bootstrap_with_prescale():
    """plan.prescale != 0 (the reference's ModRaise without `prescaled`): a two-tower input is multiplied by the
    factor encoded at its top prime and rescaled first; the result is bit-exact against the replay and decrypts to
    factor * message."""
    st = Setup(slots=16, budget=(1, 1), sse=False, seed=0x5EED0006)
    F, gpu, orc = st.F, st.gpu, st.orc
    rng = np.random.default_rng(81)
    z = (rng.uniform(-1, 1, st.slots) + 1j * rng.uniform(-1, 1, st.slots)) * 0.5
    ct = orc.encrypt(81, st.s, orc.encode(z, DELTA_M, 2))
    plan = F.BootstrapPlan.make(st.slots, NQ, list(st.plan.lt_cts[:st.plan.cts_count]),
                                list(st.plan.lt_stc[:st.plan.stc_count]), st.coeffs, R_DOUBLE, st.lo, st.hi,
                                DELTA_PT, prescale=0.5)
    out = gpu.eval_bootstrap(gpu.load_ciphertext(ct, DELTA_M), plan)
    got = gpu.store_ciphertext(out)
    ref, ref_scale = st.replay(ct, prescale=0.5)
    assert np.array_equal(got, ref)
    err, bits = st.precision(got, gpu.meta(out).scale, 0.5 * z)
    print(f"prescaled bootstrap: max slot error {err:.3e} ({bits:.1f} bits)")
    assert err < 1e-3, err


def test_bootstrap_full_slots_level_budget_sse_and_batch():
    """Double-hoisted CoeffsToSlots / SlotsToCoeffs factors (diagonals at the special primes too)."""
    st = Setup(slots=N // 2, budget=(3, 3), sse=True, seed=0x5EED0015, ext=True)
    z, ct = st.message(78)
    got, meta = check(st, z, ct, 2e-5)
    assert meta.towers >= 2
    # three bootstraps in flight together: the first equals the single call, the others decrypt to their inputs
    z2, ct2 = st.message(79)
    z3, ct3 = st.message(80)
    gpu = st.gpu
    hs = [gpu.load_ciphertext(c, DELTA_M) for c in (ct, ct2, ct3)]
    outs = gpu.eval_bootstrap_batch(hs, st.plan)
    assert np.array_equal(gpu.store_ciphertext(outs[0]), got)
    for o, zz in zip(outs[1:], (z2, z3)):
        err, bits = st.precision(gpu.store_ciphertext(o), gpu.meta(o).scale, zz)
        assert err < 2e-5, err


def test_bootstrap_requests_through_the_server():
    """Bootstrap requests submitted to the continuous-batching server run in flight together and give exactly the
    single-call results."""
    st = Setup(slots=N // 2, budget=(3, 3), sse=True, seed=0x5EED0025, ext=True)
    gpu, F = st.gpu, st.F
    msgs = [st.message(90 + i) for i in range(3)]
    hs = [gpu.load_ciphertext(ct, DELTA_M) for _, ct in msgs]
    singles = [gpu.store_ciphertext(gpu.eval_bootstrap(h, st.plan)) for h in hs]
    srv = F.Server(gpu, max_batch=8, max_inflight=1, mem_budget=64 << 30)
    srv.set_bootstrap_plan(st.plan)
    tickets = [srv.submit(F.OP_BOOTSTRAP, h) for h in hs]
    outs = [srv.wait(t)[0] for t in tickets]
    stats = srv.stats()
    srv.close()  # unreleased results stay in the context, owned by the caller
    got = [gpu.store_ciphertext(o) for o in outs]
    for g, ref in zip(got, singles):
        assert np.array_equal(g, ref)
    assert stats["completed"] == 3
