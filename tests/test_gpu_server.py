"""The continuous-batching server: every served result equals the same request evaluated alone, whatever batch
it landed in; requests from several client threads at ragged levels; admission under a tight memory budget."""
import threading

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("max_batch,budget", [(16, 16 << 30), (64, 24 << 20)])
def test_served_results_equal_alone_results(engine_lib, max_batch, budget):
    import fideslib_gb300 as F
    logN = 12
    N = 1 << logN
    mods = O.make_moduli(logN, [60] + [50] * 11, [60] * 4)
    nq = 12
    ctx = F.CryptoContext(logN, mods, 4, 3)
    orc = O.Ctx(N, nq, 4, 3, mods, threads=4)
    s = orc.secret(1)
    ctx.load_eval_mult_key(orc.relin_key(2, s))
    for idx in (1, -2, 7):
        g = orc.galois(idx)
        ctx.load_rotation_key(g, orc.rot_key(3 + g, s, g))
    rng = np.random.default_rng(9)
    handles = {}
    for t in range(2, nq + 1):
        handles[t] = [ctx.load_ciphertext(np.stack([orc.uniform(100 * t + k, t), orc.uniform(7 + 100 * t + k, t)]))
                      for k in range(2)]
    reqs = []
    for _ in range(48):
        t = int(rng.integers(2, nq + 1))
        a, b = handles[t]
        kind = int(rng.integers(0, 4))
        if kind == 0:
            reqs.append((F.OP_MULT, a, b, 0))
        elif kind == 1:
            reqs.append((F.OP_ROTATE, a, 0, int(rng.choice([1, -2, 7]))))
        elif kind == 2:
            reqs.append((F.OP_RESCALE, a, 0, 0))
        else:
            reqs.append((F.OP_ADD, a, b, 0))
    alone = [ctx.store_ciphertext(ctx.eval_batch([r])[0]) for r in reqs]
    srv = F.Server(ctx, max_batch=max_batch, max_inflight=2, mem_budget=budget)
    tickets = [None] * len(reqs)

    def client(lo, hi):
        for i in range(lo, hi):
            tickets[i] = srv.submit(*reqs[i])

    th = [threading.Thread(target=client, args=(k * 16, (k + 1) * 16)) for k in range(3)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    outs = [srv.wait(tk)[0] for tk in tickets]
    st = srv.stats()
    assert st["completed"] == len(reqs)
    srv.close()  # results stay in the context after the server stops
    for r, o, e in zip(reqs, outs, alone):
        assert np.array_equal(ctx.store_ciphertext(o), e), r
    if budget == 16 << 30:  # a roomy budget: 48 requests submitted at once cannot all run one by one
        assert st["mean_batch"] > 1 and st["batches"] < len(reqs), st
    ctx.close()


def test_released_results_are_freed_safely_while_batches_run(engine_lib):
    """Three lanes.  A client thread keeps submitting requests on resident ciphertexts while a second thread waits
    for each result, submits a rotation of that result and releases the result at once, while the rotation is
    pending or in flight on another lane; the server must keep the released ciphertext until no request reads it.
    Every rotation of a result equals the same two requests evaluated alone, read after the server stops."""
    import fideslib_gb300 as F
    logN = 12
    N = 1 << logN
    mods = O.make_moduli(logN, [60] + [50] * 11, [60] * 4)
    nq = 12
    ctx = F.CryptoContext(logN, mods, 4, 3)
    orc = O.Ctx(N, nq, 4, 3, mods, threads=4)
    s = orc.secret(5)
    ctx.load_eval_mult_key(orc.relin_key(6, s))
    for idx in (1, -3):
        g = orc.galois(idx)
        ctx.load_rotation_key(g, orc.rot_key(7 + g, s, g))
    rng = np.random.default_rng(21)
    handles = {t: [ctx.load_ciphertext(np.stack([orc.uniform(300 * t + k, t), orc.uniform(11 + 300 * t + k, t)]))
                   for k in range(2)] for t in range(2, nq + 1)}
    reqs = []
    for _ in range(64):
        t = int(rng.integers(2, nq + 1))
        a, b = handles[t]
        kind = int(rng.integers(0, 3))
        reqs.append((F.OP_MULT, a, b, 0) if kind == 0 else
                    (F.OP_ROTATE, a, 0, int(rng.choice([1, -3]))) if kind == 1 else (F.OP_ADD, a, b, 0))
    second = [int(rng.choice([1, -3])) for _ in reqs]
    alone = []
    for r, i in zip(reqs, second):
        first = ctx.eval_batch([r])[0]
        alone.append(ctx.store_ciphertext(ctx.eval_batch([(F.OP_ROTATE, first, 0, i)])[0]))
    srv = F.Server(ctx, max_batch=8, max_inflight=3, mem_budget=16 << 30)
    tickets = [None] * len(reqs)
    ready = [threading.Event() for _ in reqs]
    chained = [None] * len(reqs)

    def submitter():
        for i, r in enumerate(reqs):
            tickets[i] = srv.submit(*r)
            ready[i].set()

    def chainer():
        for i in range(len(reqs)):
            ready[i].wait()
            out, _ = srv.wait(tickets[i])
            chained[i] = srv.submit(F.OP_ROTATE, out, 0, second[i])
            srv.release(tickets[i])  # the rotation just submitted still reads this result

    th = [threading.Thread(target=submitter), threading.Thread(target=chainer)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    outs = [srv.wait(tk)[0] for tk in chained]
    st = srv.stats()
    srv.close()
    assert st["completed"] == 2 * len(reqs)
    for r, o, e in zip(reqs, outs, alone):
        assert np.array_equal(ctx.store_ciphertext(o), e), r
    ctx.close()
