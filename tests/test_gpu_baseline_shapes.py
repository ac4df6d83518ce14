"""Residue checks at the benchmark's own shapes (N = 2^16), against the oracle or the engine's single-request path.

  config 3a  one ciphertext at 30 towers rotated by the 32 indices +-2^k through EvalFastRotation (one shared
             ModUp), 30 + 10 towers, dnum 3: four outputs against the oracle;
  config 3b  the benchmarked batch itself: 64 ciphertexts at levels drawn as the benchmark draws them (U{1..29}),
             one rotation each, in one fides_eval_batch: a seeded sample of eight outputs against the oracle;
  config 4   one request server over both rings (N = 2^15 and 2^16 on the config-3 moduli) with one admission loop
             and one memory budget, requests submitted from several threads: every served result equals the same
             request evaluated alone;
  config 5   one double-hoisted CoeffsToSlots factor of the level-budget {3, 3} bootstrap (n = 2^15 slots, 60 +
             24 x 55-bit towers, 5 special primes, dnum 5) and one EvalMod double-angle step, replayed op for op by
             the oracle.
Keys and ciphertexts are seeded uniform residues of the real shapes (a key switch computes the same function of
any residues); the checks are residue-exact.
"""
import threading

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

LOGN = 16
N = 1 << LOGN
INDICES = [s * (1 << k) for k in range(16) for s in (1, -1)]


def _rand(gen, shape, mods, tower_axis):
    import torch
    m = torch.tensor([int(x) for x in mods], dtype=torch.int64, device="cuda")
    view = [1] * len(shape)
    view[tower_axis] = -1
    x = torch.randint(0, 1 << 62, shape, dtype=torch.int64, device="cuda", generator=gen)
    return x % m.view(*view)


def _host(x):
    return x.cpu().numpy().view(np.uint64)


@pytest.fixture(scope="module")
def cfg3(engine_lib):
    import torch

    import fideslib_gb300 as F
    nq, np_, dnum = 30, 10, 3
    mods = O.make_moduli(LOGN, [60] + [50] * (nq - 1), [60] * np_)
    ctx = F.CryptoContext(LOGN, mods, np_, dnum)
    orc = O.Ctx(N, nq, np_, dnum, mods, threads=16)
    gen = torch.Generator(device="cuda")
    gen.manual_seed(0x5EED0003)
    keys = {}
    for idx in INDICES:
        k = _rand(gen, (2, dnum, nq + np_, N), mods, 2)
        ctx.load_rotation_key_device(ctx.galois(idx), k.data_ptr())
        keys[idx] = k
    torch.cuda.synchronize()
    yield dict(F=F, ctx=ctx, orc=orc, mods=mods, gen=gen, keys=keys, nq=nq)
    ctx.close()


def test_cfg3a_hoisted_32_rotations(cfg3):
    ctx, orc, mods = cfg3["ctx"], cfg3["orc"], cfg3["mods"]
    ct = _rand(cfg3["gen"], (2, 30, N), mods[:30], 1)
    h = ctx.load_ciphertext_device(ct.data_ptr(), 30)
    outs = ctx.eval_fast_rotation(h, INDICES)
    sample = [1, -(1 << 7), 1 << 12, -(1 << 15)]
    ct_h = _host(ct)
    want = orc.rotate_hoisted(ct_h, [orc.galois(i) for i in sample], [_host(cfg3["keys"][i]) for i in sample])
    for i, w in zip(sample, want):
        assert np.array_equal(ctx.store_ciphertext(outs[INDICES.index(i)]), w), f"index {i}"


def test_cfg3b_benchmarked_batch(cfg3):
    F, ctx, orc, mods = cfg3["F"], cfg3["ctx"], cfg3["orc"], cfg3["mods"]
    rng = np.random.default_rng(0x5EED0003)  # the benchmark's draws of levels and rotation indices
    levels = rng.integers(1, 30, 64)
    towers = [cfg3["nq"] - int(lv) for lv in levels]
    rot_idx = [INDICES[int(i)] for i in rng.integers(0, len(INDICES), 64)]
    cts = [_rand(cfg3["gen"], (2, t, N), mods[:t], 1) for t in towers]
    hs = [ctx.load_ciphertext_device(c.data_ptr(), t, scale=2.0 ** 50) for c, t in zip(cts, towers)]
    outs = ctx.eval_batch([(F.OP_ROTATE, h, 0, i) for h, i in zip(hs, rot_idx)])
    pick = np.random.default_rng(8).choice(64, 8, replace=False)
    for k in pick:
        want = orc.rotate(_host(cts[k]), orc.galois(rot_idx[k]), _host(cfg3["keys"][rot_idx[k]]))
        assert np.array_equal(ctx.store_ciphertext(outs[k]), want), f"request {k}: {towers[k]} towers"


def test_cfg4_two_rings_one_server(cfg3):
    """Requests to N = 2^15 and N = 2^16 interleaved through one server (one admission queue, one budget) by three
    client threads; each result equals the request evaluated alone on its ring."""
    import torch

    F = cfg3["F"]
    mods = cfg3["mods"]
    rings = []
    for logn in (15, 16):
        n = 1 << logn
        ctx = F.CryptoContext(logn, mods, 10, 3) if logn == 15 else cfg3["ctx"]
        gen = torch.Generator(device="cuda")
        gen.manual_seed(0x5EED0004 + logn)
        k = _rand(gen, (2, 3, 40, n), mods, 2) if logn == 15 else None
        if logn == 15:
            ctx.load_rotation_key_device(ctx.galois(1), k.data_ptr())
            ctx.load_rotation_key_device(ctx.galois(-2), k.data_ptr())
        rk = _rand(gen, (2, 3, 40, n), mods, 2)
        ctx.load_eval_mult_key_device(rk.data_ptr())
        cts = {}
        for t in (3, 11, 20, 30):
            cts[t] = [ctx.load_ciphertext_device(_rand(gen, (2, t, n), mods[:t], 1).data_ptr(), t, scale=2.0 ** 50)
                      for _ in range(2)]
        torch.cuda.synchronize()
        rings.append((ctx, cts))
    rng = np.random.default_rng(41)
    reqs = []
    for _ in range(48):
        ring = int(rng.integers(0, 2))
        cts = rings[ring][1]
        t = [3, 11, 20, 30][int(rng.integers(0, 4))]
        a, b = cts[t]
        kind = int(rng.integers(0, 10))  # the config-4 mix: 40% mult, 40% rotate, 10% rescale, 10% add
        op = ((F.OP_MULT, a, b, 0) if kind < 4 else (F.OP_ROTATE, a, 0, [1, -2][kind % 2]) if kind < 8
              else (F.OP_RESCALE, a, 0, 0) if kind == 8 else (F.OP_ADD, a, b, 0))
        reqs.append((ring, op))
    alone = [rings[r][0].store_ciphertext(rings[r][0].eval_batch([op])[0]) for r, op in reqs]
    srv = F.Server([rings[0][0], rings[1][0]], max_batch=16, max_inflight=2, mem_budget=4 << 30)
    tickets = [None] * len(reqs)

    def client(lo, hi):
        for i in range(lo, hi):
            tickets[i] = srv.submit(*reqs[i][1], ring=reqs[i][0])

    th = [threading.Thread(target=client, args=(k * 16, (k + 1) * 16)) for k in range(3)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    outs = [srv.wait(tk)[0] for tk in tickets]
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs) and st["mean_batch"] > 1, st
    for (r, op), o, e in zip(reqs, outs, alone):
        assert np.array_equal(rings[r][0].store_ciphertext(o), e), (r, op)
    rings[0][0].close()


def test_cfg5_coeffs_to_slots_factor_and_evalmod_step(engine_lib):
    """The first CoeffsToSlots factor of the config-5 bootstrap, double-hoisted as the benchmark runs it, and one
    double-angle step of EvalMod on its rescaled output, residue for residue against the oracle."""
    import fideslib_gb300 as F
    from fideslib_gb300 import bootplan as B
    from tests import boot_plan as BP
    from tests.replay import Sim
    nq, np_, dnum = 25, 5, 5
    n, delta = N // 2, 2.0 ** 55
    mods = O.make_moduli(LOGN, [60] + [55] * (nq - 1), [60] * np_)
    ctx = F.CryptoContext(LOGN, mods, np_, dnum)
    orc = O.Ctx(N, nq, np_, dnum, mods, threads=16)
    M, stride, r = BP.factors(n, 3, inverse=True, scale=n / N)[0]
    f = BP.Factor(orc, M, n, stride, r, nq, delta, ext=True, bs=B.ext_baby_steps(r))
    keys = {}
    for i, idx in enumerate(sorted(f.rotations(n, N))):
        g = orc.galois(idx)
        keys[idx] = (g, np.stack([[orc.uniform(7000 + 10 * i + 2 * a + d, nq + np_) for d in range(dnum)]
                                  for a in range(2)]))
        ctx.load_rotation_key(g, keys[idx][1])
    rlk = np.stack([[orc.uniform(9000 + 2 * a + d, nq + np_) for d in range(dnum)] for a in range(2)])
    ctx.load_eval_mult_key(rlk)
    lt = f.create(ctx, delta)
    ct = np.stack([orc.uniform(11, nq), orc.uniform(12, nq)])
    h = ctx.load_ciphertext(ct, delta)
    out = ctx.eval_linear_transform(h, lt)
    want = f.replay(orc, ct, keys, N)
    assert np.array_equal(ctx.store_ciphertext(out), want)
    # one EvalMod double angle (x <- 2x^2 - 1) on the rescaled transform output
    x = ctx.rescale(out)
    got = ctx.store_ciphertext(ctx.eval_double_angle(x, 1))
    sim = Sim(orc, mods, rlk)
    y = sim.rescale((want, delta * delta))
    y = sim.add_scalar(sim.mult_int(sim.rescale(sim.mult(y, y)), 2), -1.0)
    assert np.array_equal(got, y[0])
    ctx.lt_free(lt)
    ctx.close()
