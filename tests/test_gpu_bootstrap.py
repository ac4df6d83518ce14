"""End-to-end CKKS bootstrapping on the GPU (fides_eval_bootstrap).

Ring N=2^12 with 16 sparse slots, sparse ternary secret (Hamming weight 32), q_0 of 60 bits and 19 further
45-bit towers, 4 special primes, dnum 5.  The CoeffsToSlots / SlotsToCoeffs diagonals are computed here for the
slot order of the encoder (slot j <-> zeta^(5^j)) and encoded by the oracle, the way the reference receives its
bootstrap plaintexts from OpenFHE.  The output is checked residue-for-residue against an op-for-op oracle replay
of the documented bootstrap recipe, and its decrypted slots against the input message."""
import numpy as np
import numpy.polynomial.chebyshev as C
import pytest

import oracle as O
from tests.replay import Sim

pytestmark = pytest.mark.gpu

LOGN, NQ, NP, DNUM, SLOTS = 12, 20, 4, 5, 16
DELTA_M, DELTA_PT = 2.0 ** 55, 2.0 ** 55  # towers of 55 bits; q_0 / DELTA_M = 32 keeps the EvalMod gain small
BS = GS = 4
R_DOUBLE = 3
CHEB_DEG = 47
B_RANGE = 12.5


def slot_matrix(n):
    zeta = np.exp(1j * np.pi / (2 * n))
    rows = [pow(5, j, 4 * n) for j in range(n)]
    return np.array([[zeta ** ((r * i) % (4 * n)) for i in range(n)] for r in rows])


def diagonals(M):
    n = M.shape[0]
    return np.array([[M[j, (j + i) % n] for j in range(n)] for i in range(n)])


def encode_lt(orc, M, towers):
    d = diagonals(M)
    out = np.zeros((BS * GS, towers, 1 << LOGN), dtype=np.uint64)
    for g in range(GS):
        for b in range(BS):
            i = g * BS + b
            out[i] = orc.encode(np.roll(d[i], g * BS), DELTA_PT, towers)
    return out


def lt_replay(orc, keys, ct, diags):
    baby = [ct] + [orc.rotate(ct, *keys[b]) for b in range(1, BS)]
    total = None
    for g in range(GS):
        inner = None
        for b in range(BS):
            term = orc.plain_op(baby[b], diags[g * BS + b], 0)
            inner = term if inner is None else orc.add(inner, term)
        if g > 0:
            inner = orc.rotate(inner, *keys[g * BS])
        total = inner if total is None else orc.add(total, inner)
    return total


def test_bootstrap_end_to_end(engine_lib):
    import fideslib_gb300 as F
    N = 1 << LOGN
    mods = O.make_moduli(LOGN, [60] + [55] * (NQ - 1), [60] * NP)
    gpu = F.CryptoContext(LOGN, mods, NP, DNUM)
    orc = O.Ctx(N, NQ, NP, DNUM, mods, threads=16)
    s = orc.secret(0x5EED0005, hamming_weight=32)
    rlk = orc.relin_key(1, s)
    gpu.load_eval_mult_key(rlk)
    keys = {}
    for idx in [1, 2, 3, 4, 8, 12] + [SLOTS << k for k in range(20) if (SLOTS << k) < N // 2]:
        g = orc.galois(idx)
        keys[idx] = (g, orc.rot_key(100 + idx, s, g))
        gpu.load_rotation_key(g, keys[idx][1])
    conj = (2 * N - 1, orc.rot_key(7, s, 2 * N - 1))
    gpu.load_rotation_key(*conj)

    U = slot_matrix(SLOTS)
    A = np.linalg.inv(U) / (N // (2 * SLOTS))
    mats = {"cts_re": A / 2, "cts_im": -0.5j * A, "stc_re": U, "stc_im": 1j * U}
    enc = {k: encode_lt(orc, M, NQ) for k, M in mats.items()}
    lts = {k: gpu.lt_create(BS, GS, v, np.ones(BS * GS, dtype=bool), DELTA_PT) for k, v in enc.items()}

    K = mods[0] / DELTA_M
    lo, hi = -B_RANGE * K, B_RANGE * K
    f = lambda r: np.cos(2 * np.pi * (r / K - 0.25) / 2 ** R_DOUBLE)  # noqa: E731
    coeffs = C.chebinterpolate(lambda u: f(lo + (u + 1) * (hi - lo) / 2), CHEB_DEG)
    cbuf = np.ascontiguousarray(coeffs)
    plan = F.BootstrapPlan(SLOTS, NQ, lts["cts_re"], lts["cts_im"], lts["stc_re"], lts["stc_im"],
                           cbuf.ctypes.data_as(F.C.POINTER(F.C.c_double)), len(cbuf), R_DOUBLE, lo, hi, DELTA_PT)

    rng = np.random.default_rng(77)
    z = (rng.uniform(-1, 1, SLOTS) + 1j * rng.uniform(-1, 1, SLOTS)) * 0.5
    ct = orc.encrypt(5, s, orc.encode(z, DELTA_M, 1))
    h = gpu.load_ciphertext(ct, DELTA_M)
    out = gpu.eval_bootstrap(h, plan)
    got = gpu.store_ciphertext(out)
    meta = gpu.meta(out)

    # op-for-op oracle replay of the recipe in fideslib_gb300/csrc/bootstrap.cu
    sim = Sim(orc, mods, rlk)
    x = orc.mod_raise(ct, NQ)
    r = SLOTS
    while r < N // 2:
        x = orc.add(x, orc.rotate(x, *keys[r]))
        r <<= 1
    halves = []
    for name in ("cts_re", "cts_im"):
        y = lt_replay(orc, keys, x, enc[name])
        y = orc.add(y, orc.rotate(y, *conj))
        halves.append(sim.rescale((y, DELTA_M * DELTA_PT)))
    mods_out = []
    for v in halves:
        c = sim.chebyshev(v, list(coeffs), lo, hi, DELTA_PT)
        for _ in range(R_DOUBLE):
            c = sim.add_scalar(sim.mult_int(sim.rescale(sim.mult(c, c)), 2), -1.0)
        mods_out.append(sim.rescale(sim.mult_scalar(c, K / (2 * np.pi), DELTA_PT)))
    a = lt_replay(orc, keys, mods_out[0][0], enc["stc_re"])
    b = lt_replay(orc, keys, mods_out[1][0], enc["stc_im"])
    ref, ref_scale = sim.rescale((orc.add(a, b), mods_out[0][1] * DELTA_PT))
    assert np.array_equal(got, ref)
    assert abs(meta.scale / ref_scale - 1) < 1e-9

    dec = orc.decode(orc.decrypt(s, got), meta.scale, SLOTS)
    err = np.abs(dec - z).max()
    print(f"bootstrap: {meta.towers} towers left, max slot error {err:.3e} ({-np.log2(err):.1f} bits)")
    assert meta.towers == NQ - 14
    assert err < 1e-3, err
