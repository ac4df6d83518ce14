"""CPU checks of the C ABI: the library builds, loads, and exports every symbol the header declares."""
import ctypes

import pytest

import fideslib_gb300 as F
from fideslib_gb300 import build as B


@pytest.fixture(scope="module")
def so():
    B.build()
    return ctypes.CDLL(B.lib_path())


def test_header_declares_entry_points():
    names = F.declared_symbols()
    for must in ["fides_ctx_create", "fides_ntt_batch_device", "fides_eval_rotate", "fides_eval_fast_rotation",
                 "fides_eval_mult", "fides_rescale", "fides_load_rotation_key", "fides_ct_load", "fides_ct_store"]:
        assert must in names


def test_library_exports_every_declared_symbol(so):
    missing = [n for n in F.declared_symbols() if not hasattr(so, n)]
    assert not missing, missing


def test_binding_signatures_cover_header():
    assert set(F.declared_symbols()) <= set(F._SIGS), set(F.declared_symbols()) - set(F._SIGS)


def test_errors_without_gpu_are_status_codes(so):
    """No device here: context creation must fail with a status code and a message, never exit."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    F.lib()
    import numpy as np
    m = np.array([1], dtype=np.uint64)
    prm = F.Params(12, 1, 1, 1, m.ctypes.data_as(F.u64p), None, 0, None, None, None, 0.0)
    h = ctypes.c_void_p()
    rc = F.lib().fides_ctx_create(ctypes.byref(prm), ctypes.byref(h))
    assert rc in (F.FIDES_ENODEV, F.FIDES_EINVAL)
    assert F.lib().fides_last_error()


@pytest.mark.parametrize("bits,count,log_n", [(40, 5, 13), (60, 4, 16), (55, 3, 12)])
def test_find_primes_matches_oracle(so, bits, count, log_n):
    """Host-only helper: the `count` largest primes < 2^bits that are 1 mod 2N, as the oracle generates them,
    and the exclusion list skips given primes."""
    import numpy as np
    import oracle as O
    out = np.zeros(count, dtype=np.uint64)
    n = F.lib().fides_find_primes(bits, count, 2 << log_n, None, 0, out.ctypes.data_as(F.u64p))
    assert n == count
    assert [int(x) for x in out] == O.gen_primes(bits, count, 2 << log_n)
    ex = out[:2].copy()
    got = np.zeros(count, dtype=np.uint64)
    n = F.lib().fides_find_primes(bits, count, 2 << log_n, ex.ctypes.data_as(F.u64p), 2, got.ctypes.data_as(F.u64p))
    assert n == count
    assert [int(x) for x in got] == O.gen_primes(bits, count + 2, 2 << log_n)[2:]
