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
    prm = F.Params(12, 1, 1, 1, m.ctypes.data_as(F.u64p), None, 0)
    h = ctypes.c_void_p()
    rc = F.lib().fides_ctx_create(ctypes.byref(prm), ctypes.byref(h))
    assert rc in (F.FIDES_ENODEV, F.FIDES_EINVAL)
    assert F.lib().fides_last_error()
