"""The allocation-free rotation entry point, fides_eval_rotate_noalloc, against the allocating one.

Some callers of this library cannot allocate device memory while they serve a request: their GPU memory is
pre-reserved by their own allocator, or they cannot pay for cudaMalloc's implicit synchronisation.  For them
the library offers a rotation whose workspace is a fixed 32 MiB array inside the library.  This file checks,
through the C ABI, that it returns the same residues as fides_eval_automorphism (and the oracle) on two calls in
a row — the shared workspace still holds the first call's data when the second runs — and that a rotation too
large for the fixed workspace is refused with a clear error.  It is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _noalloc(F, ctx, dev_in, towers, galois, dev_out, stream=None):
    return F.lib().fides_eval_rotate_noalloc(ctx._h, ctypes.c_void_p(dev_in.data_ptr()), towers, galois,
                                             ctypes.c_void_p(dev_out.data_ptr()),
                                             None if stream is None else ctypes.c_void_p(stream))


def test_noalloc_rotation_matches_allocating_entry_point(engine_lib):
    import torch

    import fideslib_gb300 as F
    logN = 13
    N = 1 << logN
    mods = O.make_moduli(logN, [60] + [40] * 5, [60] * 3)
    ctx = F.CryptoContext(logN, mods, 3, 2)
    orc = O.Ctx(N, 6, 3, 2, mods, threads=4)
    s = orc.secret(11)
    rng = np.random.default_rng(5)
    for call, (t, index) in enumerate([(6, 1), (4, -3)]):
        z = rng.uniform(-1, 1, N // 2) + 1j * rng.uniform(-1, 1, N // 2)
        ct = np.ascontiguousarray(orc.encrypt(40 + call, s, orc.encode(z, 2.0 ** 40, 6))[:, :t])
        g = orc.galois(index)
        key = orc.rot_key(70 + call, s, g)
        ctx.load_rotation_key(g, key)
        h = ctx.load_ciphertext(ct, 2.0 ** 40)
        expected = ctx.store_ciphertext(ctx.eval_automorphism(h, g))  # the allocating entry point
        dev_in = torch.from_numpy(ct.view(np.int64)).cuda()
        dev_out = torch.zeros_like(dev_in)
        torch.cuda.synchronize()
        # The property the entry point exists for: the call allocates no device memory, neither from the
        # context's pool (counted by fides_ctx_mem_in_use) nor through the caller's allocator.
        pool_before, torch_before = ctx.mem_in_use(), torch.cuda.memory_allocated()
        rc = _noalloc(F, ctx, dev_in, t, g, dev_out)
        assert rc == F.FIDES_OK, F.lib().fides_last_error()
        assert ctx.mem_in_use() == pool_before and torch.cuda.memory_allocated() == torch_before
        ctx.synchronize()
        got = dev_out.cpu().numpy().view(np.uint64)
        assert np.array_equal(got, expected), f"call {call}"
        assert np.array_equal(got, orc.rotate(ct, g, key)), f"call {call}"
        # The same call ordered on a caller's stream instead of the context's.
        side = torch.cuda.Stream()
        dev_out2 = torch.zeros_like(dev_in)
        torch.cuda.synchronize()
        rc = _noalloc(F, ctx, dev_in, t, g, dev_out2, stream=side.cuda_stream)
        assert rc == F.FIDES_OK, F.lib().fides_last_error()
        side.synchronize()
        assert ctx.mem_in_use() == pool_before
        assert np.array_equal(dev_out2.cpu().numpy().view(np.uint64), expected), f"call {call} on a side stream"
    ctx.close()


def test_noalloc_rejects_requests_beyond_its_workspace(engine_lib):
    import torch

    import fideslib_gb300 as F
    logN = 16
    mods = O.make_moduli(logN, [60] + [50] * 9, [60] * 2)
    ctx = F.CryptoContext(logN, mods, 2, 2)  # t = 10: 78 limbs of 512 KiB > 32 MiB
    dev_in = torch.zeros((2, 10, 1 << logN), dtype=torch.int64, device="cuda")
    dev_out = torch.zeros_like(dev_in)
    rc = _noalloc(F, ctx, dev_in, 10, 5, dev_out)
    assert rc == F.FIDES_EINVAL
    assert "32 MiB" in F.lib().fides_last_error().decode()
    ctx.close()
