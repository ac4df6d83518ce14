"""CPU checks of the bootstrap precomputation used by the GPU bootstrap tests: the special-FFT factorisation,
its level-budget grouping, and the baby-step/giant-step layout the engine evaluates."""
import numpy as np
import pytest

from tests import boot_plan as BP


@pytest.mark.parametrize("n", [4, 16, 64])
def test_special_fft_factorisation(n):
    P = np.eye(n)[BP.bitrev_perm(n)]
    prod = P.astype(complex)
    ln = 2
    while ln <= n:
        S = np.zeros((n, n), complex)
        for o, d in BP.stage(n, ln).items():
            for x in range(n):
                S[x, (x + o) % n] += d[x]
        prod = S @ prod
        ln *= 2
    assert np.abs(prod - BP.slot_matrix(n)).max() < 1e-12


@pytest.mark.parametrize("n,budget", [(16, 1), (16, 2), (64, 3), (256, 3), (256, 4)])
def test_factors_multiply_to_the_transforms(n, budget):
    rng = np.random.default_rng(n + budget)
    v = rng.normal(size=n) + 1j * rng.normal(size=n)
    U = BP.slot_matrix(n)
    perm = BP.bitrev_perm(n)
    x = v.copy()
    for M, _, _ in BP.factors(n, budget, inverse=True, scale=0.25):
        x = BP.apply(M, x)
    assert np.abs(x - 0.25 * np.linalg.solve(U, v)[perm]).max() < 1e-10  # P U^-1 v / 4
    y = v.copy()
    for M, _, _ in BP.factors(n, budget, inverse=False):
        y = BP.apply(M, y)
    assert np.abs(y - U @ v[perm]).max() < 1e-9  # U P v


@pytest.mark.parametrize("n,budget", [(16, 1), (64, 2), (2048, 3), (32768, 3)])
def test_bsgs_layout_matches_factor(n, budget):
    rng = np.random.default_rng(7)
    v = rng.normal(size=n) + 1j * rng.normal(size=n)
    for inverse in (True, False):
        for M, stride, r in BP.factors(n, budget, inverse):
            bs, gs, base, slots = BP.bsgs_layout(M, n, stride, r)
            assert bs * gs >= 2 ** (r + 1) - 1
            got = BP.eval_layout(v, n, stride, bs, gs, base, slots)
            assert np.abs(got - BP.apply(M, v)).max() < 1e-9
