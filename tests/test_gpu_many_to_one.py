"""Batched plaintext and scalar ops on the GPU (fides_eval_many_to_one and the *_PLAIN requests of
fides_eval_batch) against the oracle: every residue bit-identical.

The many-to-one form follows the reference's LimbPartition::addBatchManyToOne / multPtBatchManyToOne /
addScalarBatchManyToOne / multScalarBatchManyToOne (src/CKKS/LimbPartitionBatch.cu:20-266): operand i applies to
the `stride` ciphertexts a[i*stride .. i*stride + stride - 1], which may sit at different levels.  Group sizes
are chosen so that one call spans several launches (more than 64 ciphertexts, more than 8 scalar constant
sets)."""
import numpy as np
import pytest

import oracle as O
from tests.replay import double_residue

pytestmark = pytest.mark.gpu

LOGN = 12
N = 1 << LOGN
QB, PB, DNUM = [60] + [45] * 7, [60] * 3, 2
NQ = len(QB)
SCALE = 2.0 ** 45


class Env:
    def __init__(self):
        import fideslib_gb300 as F
        self.F = F
        self.mods = O.make_moduli(LOGN, QB, PB)
        self.orc = O.Ctx(N, NQ, len(PB), DNUM, self.mods, threads=8)
        self.gpu = F.CryptoContext(LOGN, self.mods, len(PB), DNUM)
        self.rng = np.random.default_rng(0x5EED0031)

    def cts(self, towers):
        """Uniform ciphertexts at the given tower counts (residues are all the element-wise ops look at)."""
        arrs = [np.stack([self.orc.uniform(int(self.rng.integers(1 << 30)), t) for _ in range(2)]) for t in towers]
        hs = [self.gpu.load_ciphertext(a, SCALE) for a in arrs]
        return arrs, hs

    def pts(self, n, towers=NQ):
        arrs = [self.orc.uniform(int(self.rng.integers(1 << 30)), towers) for _ in range(n)]
        return arrs, [self.gpu.load_plaintext(p, 2.0 ** 40) for p in arrs]


@pytest.fixture(scope="module")
def env(engine_lib):
    return Env()


def ragged(nb, stride, rng):
    return [int(rng.integers(1, NQ + 1)) for _ in range(nb * stride)]


@pytest.mark.parametrize("op", ["MULT_PLAIN", "ADD_PLAIN", "SUB_PLAIN"])
@pytest.mark.parametrize("nb,stride", [(1, 1), (3, 4), (5, 15)])
def test_plaintext_many_to_one(env, op, nb, stride):
    F, gpu, orc = env.F, env.gpu, env.orc
    code = getattr(F, "OP_" + op)
    towers = ragged(nb, stride, env.rng)
    arrs, hs = env.cts(towers)
    parr, ph = env.pts(nb)
    outs = gpu.eval_many_to_one(code, hs, ph, stride=stride)
    mode = code - F.OP_MULT_PLAIN
    for k, (a, o) in enumerate(zip(arrs, outs)):
        i = k // stride
        expect = orc.plain_op(a, np.ascontiguousarray(parr[i][:a.shape[1]]), mode)
        assert np.array_equal(gpu.store_ciphertext(o), expect), (op, k)
        m = gpu.meta(o)
        assert m.towers == a.shape[1]
        assert m.scale == (SCALE * 2.0 ** 40 if mode == 0 else SCALE)
        # the single op gives the same ciphertext
        single = gpu.store_ciphertext([gpu.eval_mult_plain, gpu.eval_add_plain, gpu.eval_sub_plain][mode](hs[k], ph[i]))
        assert np.array_equal(single, expect)
    # in place: the a handles now hold the results
    gpu.eval_many_to_one(code, hs, ph, stride=stride, in_place=True)
    for h, o in zip(hs, outs):
        assert np.array_equal(gpu.store_ciphertext(h), gpu.store_ciphertext(o))
        assert gpu.meta(h).scale == gpu.meta(o).scale


@pytest.mark.parametrize("op", ["ADD", "SUB"])
def test_ciphertext_many_to_one(env, op):
    F, gpu, orc = env.F, env.gpu, env.orc
    nb, stride = 4, 17  # 68 ciphertexts: two launches
    gt = [int(env.rng.integers(1, NQ + 1)) for _ in range(nb)]
    towers = [gt[k // stride] for k in range(nb * stride)]
    arrs, hs = env.cts(towers)
    barr, bh = env.cts(gt)
    code = getattr(F, "OP_" + op)
    outs = gpu.eval_many_to_one(code, hs, bh, stride=stride)
    fn = orc.add if op == "ADD" else orc.sub
    for k, (a, o) in enumerate(zip(arrs, outs)):
        assert np.array_equal(gpu.store_ciphertext(o), fn(a, barr[k // stride])), k
    gpu.eval_many_to_one(code, hs, bh, stride=stride, in_place=True)
    for h, o in zip(hs, outs):
        assert np.array_equal(gpu.store_ciphertext(h), gpu.store_ciphertext(o))


@pytest.mark.parametrize("op", ["MULT_SCALAR", "ADD_SCALAR", "MULT_INT"])
def test_scalar_many_to_one(env, op):
    """Ten groups of seven (70 ciphertexts, 10 constant sets: launches split by job count and by set count)."""
    F, gpu, orc = env.F, env.gpu, env.orc
    nb, stride = 10, 7
    towers = ragged(nb, stride, env.rng)
    arrs, hs = env.cts(towers)
    if op == "MULT_INT":
        values = [float(v) for v in env.rng.integers(-(1 << 40), 1 << 40, nb)]
        scales = None
    else:
        values = list(env.rng.uniform(-3, 3, nb))
        scales = [2.0 ** int(e) for e in env.rng.integers(20, 50, nb)] if op == "MULT_SCALAR" else None
    code = getattr(F, "OP_" + op)
    outs = gpu.eval_many_to_one(code, hs, values=values, scales=scales, stride=stride)
    for k, (a, o) in enumerate(zip(arrs, outs)):
        i, t = k // stride, a.shape[1]
        mods = env.mods[:t]
        if op == "MULT_SCALAR":
            expect = orc.scalar_op(a, [double_residue(values[i] * scales[i], q) for q in mods], [0] * t)
            exp_scale = SCALE * scales[i]
        elif op == "ADD_SCALAR":
            expect = orc.scalar_op(a, [1] * t, [double_residue(values[i] * SCALE, q) for q in mods])
            exp_scale = SCALE
        else:
            expect = orc.scalar_op(a, [int(values[i]) % q for q in mods], [0] * t)
            exp_scale = SCALE
        assert np.array_equal(gpu.store_ciphertext(o), expect), (op, k)
        assert gpu.meta(o).scale == exp_scale
    # the single-ciphertext entry points agree
    k = nb * stride - 1
    i = k // stride
    single = {"MULT_SCALAR": lambda: gpu.eval_mult_scalar(hs[k], values[i], scales[i]) if scales else None,
              "ADD_SCALAR": lambda: gpu.eval_add_scalar(hs[k], values[i]),
              "MULT_INT": lambda: gpu.eval_mult_int(hs[k], int(values[i]))}[op]()
    assert np.array_equal(gpu.store_ciphertext(single), gpu.store_ciphertext(outs[k]))


def test_plaintext_requests_in_a_mixed_batch(env):
    """*_PLAIN requests join fides_eval_batch beside ciphertext adds and rescales."""
    F, gpu, orc = env.F, env.gpu, env.orc
    arrs, hs = env.cts([NQ, 3, 5, 1])
    parr, ph = env.pts(2)
    ops = [(F.OP_MULT_PLAIN, hs[0], ph[0], 0), (F.OP_ADD_PLAIN, hs[1], ph[1], 0), (F.OP_RESCALE, hs[2], 0, 0),
           (F.OP_SUB_PLAIN, hs[3], ph[0], 0), (F.OP_ADD, hs[2], hs[2], 0)]
    outs = gpu.eval_batch(ops)
    expect = [orc.plain_op(arrs[0], parr[0], 0), orc.plain_op(arrs[1], np.ascontiguousarray(parr[1][:3]), 1),
              orc.rescale(arrs[2]), orc.plain_op(arrs[3], np.ascontiguousarray(parr[0][:1]), 2),
              orc.add(arrs[2], arrs[2])]
    for o, e in zip(outs, expect):
        assert np.array_equal(gpu.store_ciphertext(o), e)


def test_many_to_one_errors(env):
    F, gpu = env.F, env.gpu
    arrs, hs = env.cts([4, 4, 2])
    parr, ph = env.pts(1, towers=3)
    with pytest.raises(F.FidesError):  # a handle twice, in place
        gpu.eval_many_to_one(F.OP_ADD_SCALAR, [hs[0], hs[0]], values=[1.0], stride=2, in_place=True)
    with pytest.raises(F.FidesError):  # in place reading one of its own outputs
        gpu.eval_many_to_one(F.OP_ADD, [hs[0]], [hs[0]], in_place=True)
    with pytest.raises(F.FidesError):  # plaintext with fewer towers than a ciphertext of its group
        gpu.eval_many_to_one(F.OP_MULT_PLAIN, [hs[2], hs[0]], [ph[0]], stride=2)
    with pytest.raises(F.FidesError):  # tower counts differ
        gpu.eval_many_to_one(F.OP_ADD, [hs[0]], [hs[2]])
    with pytest.raises(F.FidesError):  # not an integer
        gpu.eval_many_to_one(F.OP_MULT_INT, [hs[0]], values=[1.5])
    with pytest.raises(F.FidesError):  # no many-to-one form
        gpu.eval_many_to_one(F.OP_ROTATE, [hs[0]], values=[1.0])
    # a failed call leaves its inputs untouched
    assert np.array_equal(gpu.store_ciphertext(hs[0]), arrs[0])


def test_plaintext_requests_through_the_server(env):
    """*_PLAIN requests admitted by the continuous-batching server give the direct results."""
    F, gpu = env.F, env.gpu
    arrs, hs = env.cts([NQ, 4, 2, 6])
    parr, ph = env.pts(2)
    reqs = [(F.OP_MULT_PLAIN, hs[0], ph[0]), (F.OP_ADD_PLAIN, hs[1], ph[1]), (F.OP_SUB_PLAIN, hs[2], ph[0]),
            (F.OP_MULT_PLAIN, hs[3], ph[1])]
    direct = [gpu.store_ciphertext(gpu.eval_batch([(op, a, b, 0)])[0]) for op, a, b in reqs]
    srv = F.Server(gpu, max_batch=8, max_inflight=2, mem_budget=1 << 30)
    tickets = [srv.submit(op, a, b) for op, a, b in reqs]
    outs = [srv.wait(t)[0] for t in tickets]
    srv.close()
    for o, d in zip(outs, direct):
        assert np.array_equal(gpu.store_ciphertext(o), d)


@pytest.mark.parametrize("m,n_terms,shared", [(1, 1, True), (5, 7, True), (70, 3, True), (6, 11, False)])
def test_linear_wsum(env, m, n_terms, shared):
    """Weighted sums in lock step (fides_eval_linear_wsum, the reference's evalLinearWSumMutable): each sum equals
    the oracle's scalar products of its terms (constants round(w_k * scale_ki)) added up, on the smallest tower
    count of its terms.  70 sums split the launch by job count, 11 terms into two launches (the second
    accumulating), per-sum constant columns into one launch per column."""
    gpu, orc = env.gpu, env.orc
    towers = [[int(env.rng.integers(2, NQ + 1)) for _ in range(m)] for _ in range(n_terms)]
    terms = [env.cts(row) for row in towers]
    weights = list(env.rng.uniform(-2, 2, n_terms))
    if shared:
        col = [2.0 ** int(e) for e in env.rng.integers(10, 40, n_terms)]
        scales = [[col[k]] * m for k in range(n_terms)]
    else:
        scales = [[2.0 ** int(e) for e in env.rng.integers(10, 40, m)] for _ in range(n_terms)]
    outs = gpu.eval_linear_wsum([[h for h in terms[k][1]] for k in range(n_terms)], weights, scales)
    for i, o in enumerate(outs):
        t = min(towers[k][i] for k in range(n_terms))
        mods = env.mods[:t]
        acc = None
        for k in range(n_terms):
            a = np.ascontiguousarray(terms[k][0][i][:, :t])
            p = orc.scalar_op(a, [double_residue(weights[k] * scales[k][i], q) for q in mods], [0] * t)
            acc = p if acc is None else orc.add(acc, p)
        assert np.array_equal(gpu.store_ciphertext(o), acc), (m, n_terms, i)
        meta = gpu.meta(o)
        assert (meta.towers, meta.noise_deg) == (t, 2)
        assert meta.scale == SCALE * scales[0][i]
