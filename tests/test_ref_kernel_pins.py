"""The oracle against the reference's own GPU kernels (CPU test; fixtures from a GB300 run).

tests/golden/ref_kernel_pins.json holds digests of what the reference's kernels — NTT_ / INTT_, DecompAndModUpConv,
ModDown2 with the NTT_MODDOWN epilogue, the NTT_RESCALE rescale, the key inner product fusedDotKSK_2_ and the tensor
product binomialMult_, compiled from its src/NTT.cu, src/CKKS/Conv.cu and src/CKKS/ElemenwiseBatchKernels.cu and
launched as its LimbPartition launches them — return on seeded inputs (tests/golden/make_ref_kernel_pins.py).
Here the oracle recomputes every case on the same inputs: orc_ntt_fwd / orc_ntt_inv, orc_modup, orc_moddown,
orc_rescale, orc_ks_inner and orc_tensor must give the same residues, bit for bit.  The reference checks its Mult, Square and Rescale bit-exact
against OpenFHE (test/OpenFheInterfaceTests.cu), so these ops of the oracle — and through the GPU parity tests the
engine's — are pinned to the reference's arithmetic, not only to this repository's restatement of it.
"""
import json
import os

import numpy as np
import pytest

import oracle as O
from tests.golden.make_ref_kernel_pins import (LOGN, N, PARAM_SETS, digest, inner_inputs, pin_key, splitmix_residues,
                                               tensor_inputs)

PINS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_kernel_pins.json")


@pytest.fixture(scope="module")
def pins():
    if not os.path.exists(PINS):
        pytest.skip("no reference-kernel fixtures")
    return json.load(open(PINS))


@pytest.mark.parametrize("name", list(PARAM_SETS))
def test_oracle_matches_reference_kernels(pins, name):
    spec = PARAM_SETS[name]
    got = pins["sets"][name]
    assert pins["logN"] == LOGN
    mods, roots = got["moduli"], got["roots"]
    L, K = len(spec["q"]), len(spec["p"])
    assert mods == O.make_moduli(LOGN, spec["q"], spec["p"])
    assert roots == [O.root_of_unity(m, 2 * N) for m in mods]  # the roots the engine and the oracle generate
    orc = O.Ctx(N, L, K, spec["dnum"], mods, psis=roots, threads=8)
    tabs = [O.ntt_tables(N, m, r) for m, r in zip(mods, roots)]

    x = splitmix_residues(1, mods)
    assert digest(np.stack([O.ntt_fwd(x[j], mods[j], tabs[j][0]) for j in range(L + K)])) == got["ntt"]
    y = splitmix_residues(2, mods)
    assert digest(np.stack([O.ntt_inv(y[j], mods[j], tabs[j][1]) for j in range(L + K)])) == got["intt"]
    for t in spec["levels"]:
        a = splitmix_residues(100 + t, mods[:t])
        assert digest(orc.modup(a, t)) == got[f"modup/{t}"], f"ModUp at {t} towers"
        xq = splitmix_residues(200 + t, mods[:t])
        xp = splitmix_residues(300 + t, mods[L:])
        assert digest(orc.moddown(np.concatenate([xq, xp]), t)) == got[f"moddown/{t}"], f"ModDown at {t} towers"
        if t >= 2:
            ct = splitmix_residues(400 + t, mods[:t] * 2).reshape(2, t, N)
            assert digest(orc.rescale(ct)) == got[f"rescale/{t}"], f"rescale at {t} towers"
        if f"ksinner/{t}" in got:
            key = pin_key(mods, L, K, spec["dnum"])
            _, D = inner_inputs(t, mods, L, K, orc.alpha)
            assert digest(orc.ks_inner(D, t, key)) == got[f"ksinner/{t}"], f"key inner product at {t} towers"
            x, y = tensor_inputs(t, mods)
            assert digest(orc.tensor(x, y)) == got[f"tensor/{t}"], f"tensor product at {t} towers"
