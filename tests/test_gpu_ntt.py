"""GPU parity of the batched NTT / INTT against the oracle (bit-exact), through the C ABI."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def make_ctx(logN, nprimes, bits=59):
    import fideslib_gb300 as F
    N = 1 << logN
    mods = O.gen_primes(bits, nprimes + 1, 2 * N)
    ctx = F.CryptoContext(logN, mods, 1, 1)
    return ctx, mods


@pytest.mark.parametrize("logN", [10, 11, 12, 13, 14, 15, 16])
def test_ntt_matches_oracle(engine_lib, logN):
    N = 1 << logN
    ctx, mods = make_ctx(logN, 3)
    assert ctx.roots == [O.root_of_unity(p, 2 * N) for p in mods]
    rng = np.random.default_rng(logN)
    npolys, limbs = 2, 3
    data = np.stack([np.stack([rng.integers(0, mods[j], N, dtype=np.uint64) for j in range(limbs)])
                     for _ in range(npolys)])
    fwd = ctx.ntt_host(data.copy(), 0, inverse=False)
    for k in range(npolys):
        for j in range(limbs):
            tab, itab = O.ntt_tables(N, mods[j], ctx.roots[j])
            assert np.array_equal(fwd[k, j], O.ntt_fwd(data[k, j], mods[j], tab)), (logN, k, j)
    inv = ctx.ntt_host(fwd.copy(), 0, inverse=True)
    assert np.array_equal(inv, data)
    # inverse on arbitrary input vs oracle
    inv2 = ctx.ntt_host(data.copy(), 0, inverse=True)
    for j in range(limbs):
        tab, itab = O.ntt_tables(N, mods[j], ctx.roots[j])
        assert np.array_equal(inv2[0, j], O.ntt_inv(data[0, j], mods[j], itab))


def test_ntt_edge_values(engine_lib):
    """All-zero, all-(p-1) and single-spike limbs (largest residues exercise every lazy-reduction bound)."""
    logN = 16
    N = 1 << logN
    ctx, mods = make_ctx(logN, 2, bits=60)
    data = np.zeros((1, 2, N), dtype=np.uint64)
    data[0, 0, :] = mods[0] - 1
    data[0, 1, 12345] = mods[1] - 1
    fwd = ctx.ntt_host(data.copy(), 0, inverse=False)
    for j in range(2):
        tab, _ = O.ntt_tables(N, mods[j], ctx.roots[j])
        assert np.array_equal(fwd[0, j], O.ntt_fwd(data[0, j], mods[j], tab))
    assert np.array_equal(ctx.ntt_host(fwd, 0, inverse=True), data)
    z = np.zeros((1, 2, N), dtype=np.uint64)
    assert not ctx.ntt_host(z, 0).any()


def test_batched_ntt_full_size_config(engine_lib):
    """N=2^16, 40 primes < 2^60 with p = 1 mod 2^17, 16 polynomials (640 limbs): bit-exact vs the oracle on
    every limb, and INTT(NTT(x)) == x."""
    import fideslib_gb300 as F
    logN = 16
    N = 1 << logN
    mods = O.gen_primes(60, 41, 2 * N)
    ctx = F.CryptoContext(logN, mods, 1, 1)
    rng = np.random.default_rng(0x5EED0002)
    P = np.array(mods[:40], dtype=np.uint64)
    data = (rng.integers(0, 2 ** 63, (16, 40, N), dtype=np.uint64) % P[None, :, None]).astype(np.uint64)
    fwd = ctx.ntt_host(data.copy(), 0)
    tabs = np.zeros((40, N), dtype=np.uint64)
    itabs = np.zeros((40, N), dtype=np.uint64)
    for j in range(40):
        tabs[j], itabs[j] = O.ntt_tables(N, mods[j], ctx.roots[j])
    ref = data.reshape(640, N).copy()
    O.ntt_batch(ref, np.tile(np.arange(40), 16), P, tabs, inverse=False, nthreads=16)
    assert np.array_equal(fwd.reshape(640, N), ref)
    back = ctx.ntt_host(fwd, 0, inverse=True)
    assert np.array_equal(back, data)


@pytest.mark.parametrize("logN", [13, 14, 15, 16])
def test_all_ntt_variants_and_autotuner(engine_lib, logN):
    """The autotuner picked one kernel per direction and batch size with all of them timed; each variant,
    forced, gives the oracle's residues (edge values included) and inverts exactly."""
    N = 1 << logN
    ctx, mods = make_ctx(logN, 2, bits=60)
    tune = ctx.ntt_tuning()
    for cls in ("tiny", "small", "large"):
        assert tune[f"fwd_variant_{cls}"] in (0, 1, 2) and tune[f"inv_variant_{cls}"] in (0, 1, 2)
        assert min(tune[f"fwd_ms_{cls}"] + tune[f"inv_ms_{cls}"]) > 0
    rng = np.random.default_rng(logN + 100)
    data = np.stack([rng.integers(0, mods[j], N, dtype=np.uint64) for j in range(2)])[None]
    data[0, 0, :7] = mods[0] - 1
    for v in (0, 1, 2):
        ctx.set_ntt_variant(v, v)
        fwd = ctx.ntt_host(data.copy(), 0, inverse=False)
        for j in range(2):
            tab, _ = O.ntt_tables(N, mods[j], ctx.roots[j])
            assert np.array_equal(fwd[0, j], O.ntt_fwd(data[0, j], mods[j], tab)), (logN, v, j)
        assert np.array_equal(ctx.ntt_host(fwd.copy(), 0, inverse=True), data), (logN, v)


@pytest.mark.parametrize("logN", [12, 16])
def test_forward_ntt_accepts_lazy_inputs(engine_lib, logN):
    """The basis conversions hand the forward NTT residues in [0, 8p) (unreduced): the transform of x + k p,
    k < 8, equals the transform of x, for every kernel variant."""
    N = 1 << logN
    ctx, mods = make_ctx(logN, 2, bits=60)
    rng = np.random.default_rng(logN + 7)
    x = np.stack([rng.integers(0, mods[j], N, dtype=np.uint64) for j in range(2)])[None]
    lazy = x.copy()
    for j in range(2):
        k = rng.integers(0, 8, N, dtype=np.uint64)
        lazy[0, j] = x[0, j] + k * np.uint64(mods[j])
    assert lazy.max() >= max(mods[:2])
    for v in ((0, 1, 2) if logN >= 13 else (1,)):
        ctx.set_ntt_variant(v, 0)
        assert np.array_equal(ctx.ntt_host(lazy.copy(), 0, inverse=False), ctx.ntt_host(x.copy(), 0, inverse=False))


@pytest.mark.parametrize("logN", [10, 12, 13, 14, 16])
def test_inverse_ntt_accepts_lazy_inputs(engine_lib, logN):
    """The inverse takes residues in [0, 4p) (the key inner product's and other kernels' lazy outputs): the
    transform of x + k p, k < 4, equals the transform of x for every kernel variant, also with every residue at
    the top of the range (4p - 1), where the per-position bounds of the lazy butterflies are tightest."""
    N = 1 << logN
    ctx, mods = make_ctx(logN, 2, bits=60)
    rng = np.random.default_rng(logN + 11)
    x = np.stack([rng.integers(0, mods[j], N, dtype=np.uint64) for j in range(2)])[None]
    lazy = x.copy()
    for j in range(2):
        lazy[0, j] = x[0, j] + rng.integers(0, 4, N, dtype=np.uint64) * np.uint64(mods[j])
    top = np.stack([np.full(N, 4 * mods[j] - 1, dtype=np.uint64) for j in range(2)])[None]
    top_red = np.stack([np.full(N, mods[j] - 1, dtype=np.uint64) for j in range(2)])[None]
    for v in ((0, 1, 2) if logN >= 13 else (0,)):
        ctx.set_ntt_variant(1 if logN < 13 else 0, v)
        ref = ctx.ntt_host(x.copy(), 0, inverse=True)
        for j in range(2):
            _, itab = O.ntt_tables(N, mods[j], ctx.roots[j])
            assert np.array_equal(ref[0, j], O.ntt_inv(x[0, j], mods[j], itab)), (logN, v, j)
        assert np.array_equal(ctx.ntt_host(lazy.copy(), 0, inverse=True), ref), (logN, v)
        assert np.array_equal(ctx.ntt_host(top.copy(), 0, inverse=True),
                              ctx.ntt_host(top_red.copy(), 0, inverse=True)), (logN, v)
