"""Failure handling without a GPU fault: device-memory exhaustion is injected through the context's memory
budget (fides_ctx_set_mem_limit), never by exhausting the GPU.  Every failure must come back as a status code,
leave nothing allocated, and leave the context (and a request server over it) usable."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

LOGN = 12
N = 1 << LOGN


@pytest.fixture(scope="module")
def env(engine_lib):
    import fideslib_gb300 as F
    mods = O.make_moduli(LOGN, [60] + [45] * 5, [60] * 2)
    gpu = F.CryptoContext(LOGN, mods, 2, 3)
    orc = O.Ctx(N, 6, 2, 3, mods, threads=8)
    s = orc.secret(11)
    g = orc.galois(3)
    key = orc.rot_key(12, s, g)
    gpu.load_rotation_key(g, key)
    rlk = orc.relin_key(13, s)
    gpu.load_eval_mult_key(rlk)
    rng = np.random.default_rng(3)
    ct = orc.encrypt(14, s, orc.encode(rng.uniform(-1, 1, N // 2), 2.0 ** 40, 6))
    return dict(F=F, gpu=gpu, orc=orc, g=g, key=key, rlk=rlk, ct=ct)


def test_out_of_memory_is_a_status_and_recoverable(env):
    F, gpu, orc = env["F"], env["gpu"], env["orc"]
    h = gpu.load_ciphertext(env["ct"], 2.0 ** 40)
    base = gpu.mem_in_use()
    gpu.set_mem_limit(base + 8 * N * 4)  # room for 4 limbs: an output ciphertext fits, the key-switch workspace not
    for call in (lambda: gpu.eval_rotate(h, 3), lambda: gpu.eval_mult(h, h),
                 lambda: gpu.eval_batch([(F.OP_ROTATE, h, 0, 3), (F.OP_SQUARE, h, 0, 0)])):
        with pytest.raises(F.FidesError) as ei:
            call()
        assert ei.value.code == F.FIDES_ENOMEM
        assert gpu.mem_in_use() == base  # nothing leaked by the failed op
    gpu.set_mem_limit(0)
    got = gpu.store_ciphertext(gpu.eval_rotate(h, 3))
    assert np.array_equal(got, orc.rotate(env["ct"], env["g"], env["key"]))


def test_server_reports_per_request_status(env):
    """Under a budget that admits rescales but not key switches, a mixed stream completes: the rescales succeed
    with the right residues, the rotations come back with FIDES_ENOMEM, and the server keeps serving."""
    F, gpu, orc = env["F"], env["gpu"], env["orc"]
    h = gpu.load_ciphertext(env["ct"], 2.0 ** 40)
    base = gpu.mem_in_use()
    # a rescale at 6 towers takes 10 output + 12 workspace limbs, a rotation 12 + 50: with up to three rescale
    # results held, 56 limbs admit every rescale and no rotation
    gpu.set_mem_limit(base + 8 * N * 56)
    srv = F.Server(gpu, max_batch=4, max_inflight=1, mem_budget=1 << 30)
    tickets = [srv.submit(F.OP_RESCALE if i % 2 == 0 else F.OP_ROTATE, h, 0, 0 if i % 2 == 0 else 3)
               for i in range(6)]
    results = []
    for i, t in enumerate(tickets):
        try:
            results.append(("ok", srv.wait(t)[0]))
        except F.FidesError as e:
            results.append(("err", e.code))
    srv.close()
    gpu.set_mem_limit(0)
    expect = orc.rescale(env["ct"])
    for i, (kind, v) in enumerate(results):
        if i % 2 == 0:
            assert kind == "ok"
            assert np.array_equal(gpu.store_ciphertext(v), expect)
            gpu.free(v)
        else:
            assert (kind, v) == ("err", F.FIDES_ENOMEM)


def test_input_check_refuses_out_of_range_residues(env):
    """With the opt-in input check on, a residue at or above its prime is refused at load time (FIDES_EINVAL) and
    nothing is registered; in-range objects still load and evaluate to the oracle's result."""
    F, gpu, orc = env["F"], env["gpu"], env["orc"]
    gpu.set_input_check(True)
    try:
        base = gpu.mem_in_use()
        bad = env["ct"].copy()
        bad[1, 4, 17] = gpu.moduli[4]  # == q_4: out of range for tower 4 of c1
        with pytest.raises(F.FidesError) as ei:
            gpu.load_ciphertext(bad, 2.0 ** 40)
        assert ei.value.code == F.FIDES_EINVAL
        assert gpu.mem_in_use() == base
        pt = np.zeros((6, N), dtype=np.uint64)
        pt[5, 0] = np.uint64(2 ** 64 - 1)
        with pytest.raises(F.FidesError) as ei:
            gpu.load_plaintext(pt, 1.0)
        assert ei.value.code == F.FIDES_EINVAL
        g5 = orc.galois(5)
        badkey = orc.rot_key(21, orc.secret(11), g5)
        badkey[1, 2, 7, 9] = gpu.moduli[7]  # a special tower's prime in the b part of digit 2
        with pytest.raises(F.FidesError) as ei:
            gpu.load_rotation_key(g5, badkey)
        assert ei.value.code == F.FIDES_EINVAL
        h = gpu.load_ciphertext(env["ct"], 2.0 ** 40)
        with pytest.raises(F.FidesError) as ei:  # the refused key was not registered
            gpu.eval_rotate(h, 5)
        assert ei.value.code == F.FIDES_ENOKEY
        got = gpu.store_ciphertext(gpu.eval_rotate(h, 3))
        assert np.array_equal(got, orc.rotate(env["ct"], env["g"], env["key"]))
    finally:
        gpu.set_input_check(False)


def test_raw_files_through_a_context(env, tmp_path):
    """A resident ciphertext saved and reloaded keeps its residues and metadata; a rotation key loaded from a raw
    file rotates like the one loaded from memory; a file of another basis is refused."""
    F, gpu, orc = env["F"], env["gpu"], env["orc"]
    h = gpu.load_ciphertext(env["ct"], 2.0 ** 40, 1, 64)
    p = str(tmp_path / "ct.fgb")
    gpu.save_ciphertext(h, p)
    h2 = gpu.load_ciphertext_file(p)
    assert np.array_equal(gpu.store_ciphertext(h2), env["ct"])
    m = gpu.meta(h2)
    assert (m.towers, m.noise_deg, m.slots, m.scale) == (6, 1, 64, 2.0 ** 40)
    g7 = orc.galois(7)
    key = orc.rot_key(31, orc.secret(11), g7)
    kp = str(tmp_path / "rot7.fgb")
    F.raw_write(kp, F.RAW_ROTATION_KEY, key.reshape(-1, 8, N), gpu.moduli, gpu.roots, ident=g7)
    gpu.load_key_file(kp)
    got = gpu.store_ciphertext(gpu.eval_rotate(h2, 7))
    assert np.array_equal(got, orc.rotate(env["ct"], g7, key))
    other = O.make_moduli(LOGN, [59] + [45] * 5, [60] * 2)
    F.raw_write(p, F.RAW_CIPHERTEXT, env["ct"], other)
    with pytest.raises(F.FidesError) as ei:
        gpu.load_ciphertext_file(p)
    assert ei.value.code == F.FIDES_EINVAL
