"""Raw residue files on the host (no GPU needed): write / read round trip of every field, and refusal of
corrupted, truncated, foreign and out-of-range files with FIDES_EINVAL."""
import os

import numpy as np
import pytest

import fideslib_gb300 as F
import oracle as O


@pytest.fixture(scope="module")
def so():
    return F.lib()


def _ct(mods, rows, n=1 << 10, seed=3):
    rng = np.random.default_rng(seed)
    return np.stack([np.stack([rng.integers(0, mods[j], n, dtype=np.uint64) for j in range(rows)])
                     for _ in range(2)])


def test_round_trip(so, tmp_path):
    mods = O.make_moduli(10, [60, 50, 50], [60])
    roots = [O.root_of_unity(m, 2 << 10) for m in mods]
    ct = _ct(mods, 3)
    p = str(tmp_path / "ct.fgb")
    F.raw_write(p, F.RAW_CIPHERTEXT, ct, mods, roots, noise_deg=2, slots=512, scale=2.0 ** 50 * 1.25)
    info, m, r, d = F.raw_read(p)
    assert (info.kind, info.log_n, info.rows, info.polys, info.noise_deg, info.slots) == \
        (F.RAW_CIPHERTEXT, 10, 3, 2, 2, 512)
    assert info.scale == 2.0 ** 50 * 1.25
    assert list(m) == mods[:3] and list(r) == roots[:3]
    assert np.array_equal(d, ct)
    assert os.path.getsize(p) == 96 + 3 * 8 * 2 + ct.nbytes + 8
    assert not os.path.exists(p + ".tmp")


def test_refusals(so, tmp_path):
    mods = O.make_moduli(10, [60, 50], [60])
    ct = _ct(mods, 2)
    p = str(tmp_path / "a.fgb")
    F.raw_write(p, F.RAW_CIPHERTEXT, ct, mods)
    raw = bytearray(open(p, "rb").read())

    def refused(blob):
        q = str(tmp_path / "b.fgb")
        open(q, "wb").write(bytes(blob))
        with pytest.raises(F.FidesError) as ei:
            F.raw_read(q)
        assert ei.value.code == F.FIDES_EINVAL
        return F.lib().fides_last_error().decode()

    flipped = bytearray(raw)
    flipped[200] ^= 1
    assert "hash" in refused(flipped)
    assert "truncated" in refused(raw[:-9])
    bad_magic = bytearray(raw)
    bad_magic[0] = ord("X")
    assert "magic" in refused(bad_magic)
    big = ct.copy()
    big[1, 1, 5] = mods[1]  # at the modulus: written as given, refused when read
    F.raw_write(p, F.RAW_CIPHERTEXT, big, mods)
    with pytest.raises(F.FidesError):
        F.raw_read(p)
    assert "modulus" in F.lib().fides_last_error().decode()
