"""CPU oracle for the CKKS evaluation hot path — TEST INFRASTRUCTURE ONLY.

ctypes wrapper over oracle/ckks_oracle.c (a plain-C restatement of the arithmetic FIDESlib takes from
OpenFHE 1.5.1 and of FIDESlib's own kernels; every C function cites the reference lines it follows) and
over oracle/_ref/libref_cpuntt.so, the reference's own CPU NTT (test/cpuNTT_nega.cpp) compiled from its
sources by oracle/build_ref.sh.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this package; the engine in
fideslib_gb300/ never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(HERE, "_build", "libckks_oracle.so")
_REF_PATH = os.path.join(HERE, "_ref", "libref_cpuntt.so")
_lib = None
_ref = None

u64p = C.POINTER(C.c_uint64)
i64p = C.POINTER(C.c_int64)
u32p = C.POINTER(C.c_uint32)
i32p = C.POINTER(C.c_int32)


def build() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return _LIB_PATH


def build_ref() -> str | None:
    """Compile the reference CPU NTT when the reference tree is present on this host."""
    r = subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout + r.stderr)
    return _REF_PATH if os.path.exists(_REF_PATH) else None


def _p(a: np.ndarray, t=u64p):
    return a.ctypes.data_as(t)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
                os.path.join(HERE, "ckks_oracle.c")):
            build()
        L = C.CDLL(_LIB_PATH)
        L.orc_mulmod.restype = C.c_uint64
        L.orc_mulmod.argtypes = [C.c_uint64] * 3
        L.orc_powmod.restype = C.c_uint64
        L.orc_powmod.argtypes = [C.c_uint64] * 3
        L.orc_invmod.restype = C.c_uint64
        L.orc_invmod.argtypes = [C.c_uint64] * 2
        L.orc_is_prime.restype = C.c_int
        L.orc_is_prime.argtypes = [C.c_uint64]
        L.orc_gen_primes.restype = C.c_int
        L.orc_gen_primes.argtypes = [C.c_int, C.c_int, C.c_uint64, u64p, C.c_int, u64p]
        L.orc_root_of_unity.restype = C.c_uint64
        L.orc_root_of_unity.argtypes = [C.c_uint64, C.c_uint64]
        L.orc_ntt_tables.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, u64p, u64p]
        L.orc_ntt_fwd.argtypes = [u64p, C.c_uint64, C.c_uint64, u64p]
        L.orc_ntt_inv.argtypes = [u64p, C.c_uint64, C.c_uint64, u64p]
        L.orc_ntt_batch.argtypes = [u64p, C.c_int, C.c_uint64, i32p, u64p, u64p, C.c_int, C.c_int]
        L.orc_ctx_new.restype = C.c_void_p
        L.orc_ctx_new.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_int, u64p, u64p]
        L.orc_ctx_free.argtypes = [C.c_void_p]
        L.orc_ctx_set_threads.argtypes = [C.c_void_p, C.c_int]
        L.orc_ctx_alpha.restype = C.c_int
        L.orc_ctx_alpha.argtypes = [C.c_void_p]
        L.orc_to_coeff.argtypes = [C.c_void_p, u64p, C.c_int, i32p]
        L.orc_to_eval.argtypes = [C.c_void_p, u64p, C.c_int, i32p]
        L.orc_modup.argtypes = [C.c_void_p, u64p, C.c_int, u64p]
        L.orc_ks_inner.argtypes = [C.c_void_p, u64p, C.c_int, u64p, u64p]
        L.orc_moddown.argtypes = [C.c_void_p, u64p, C.c_int, u64p]
        L.orc_keyswitch.argtypes = [C.c_void_p, u64p, C.c_int, u64p, u64p]
        L.orc_automorph.argtypes = [C.c_void_p, u64p, C.c_int, C.c_uint32, u64p]
        L.orc_galois_for_index.restype = C.c_uint32
        L.orc_galois_for_index.argtypes = [C.c_uint64, C.c_int32]
        L.orc_rotate.argtypes = [C.c_void_p, u64p, C.c_int, C.c_uint32, u64p, u64p]
        L.orc_rotate_hoisted.argtypes = [C.c_void_p, u64p, C.c_int, C.c_int, u32p, C.POINTER(u64p),
                                         C.POINTER(u64p)]
        L.orc_tensor.argtypes = [C.c_void_p, u64p, u64p, C.c_int, u64p]
        L.orc_mult.argtypes = [C.c_void_p, u64p, u64p, C.c_int, u64p, u64p]
        L.orc_square.argtypes = [C.c_void_p, u64p, C.c_int, u64p, u64p]
        L.orc_rescale.argtypes = [C.c_void_p, u64p, C.c_int, u64p]
        L.orc_add.argtypes = [C.c_void_p, u64p, u64p, C.c_int, C.c_int, u64p]
        L.orc_sub.argtypes = [C.c_void_p, u64p, u64p, C.c_int, C.c_int, u64p]
        L.orc_plain_op.argtypes = [C.c_void_p, u64p, u64p, C.c_int, C.c_int, u64p]
        L.orc_scalar_op.argtypes = [C.c_void_p, u64p, C.c_int, u64p, u64p, u64p]
        L.orc_mod_raise.argtypes = [C.c_void_p, u64p, C.c_int, C.c_int, u64p]
        L.orc_mult_monomial.argtypes = [C.c_void_p, u64p, C.c_int, C.c_uint32, u64p]
        L.orc_rng_fill_uniform.argtypes = [C.c_void_p, C.c_uint64, u64p, C.c_int, i32p]
        L.orc_keygen_secret.argtypes = [C.c_void_p, C.c_uint64, C.c_int, i64p]
        L.orc_secret_eval.argtypes = [C.c_void_p, i64p, u64p]
        L.orc_ksk_gen.argtypes = [C.c_void_p, C.c_uint64, i64p, i64p, u64p]
        L.orc_relin_keygen.argtypes = [C.c_void_p, C.c_uint64, i64p, u64p]
        L.orc_rot_keygen.argtypes = [C.c_void_p, C.c_uint64, i64p, C.c_uint32, u64p]
        L.orc_encode.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int, C.c_double,
                                 C.c_int, u64p]
        L.orc_encode_ids.argtypes = [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int,
                                     C.c_double, C.c_int, i32p, u64p]
        L.orc_ew_ids.argtypes = [C.c_void_p, u64p, u64p, C.c_int, C.c_int, C.c_int, i32p, C.c_int, u64p]
        L.orc_decode.argtypes = [C.c_void_p, u64p, C.c_int, C.c_double, C.c_int, C.POINTER(C.c_double),
                                 C.POINTER(C.c_double)]
        L.orc_encrypt_sk.argtypes = [C.c_void_p, C.c_uint64, i64p, u64p, C.c_int, u64p]
        L.orc_decrypt.argtypes = [C.c_void_p, i64p, u64p, C.c_int, u64p]
        _lib = L
    return _lib


def ref_lib():
    """The reference's own CPU NTT, or None when it was not built (no reference tree on this host)."""
    global _ref
    if _ref is None and os.path.exists(_REF_PATH):
        R = C.CDLL(_REF_PATH)
        for name in ("ref_nega_fft", "ref_nega_fft2"):
            f = getattr(R, name)
            f.argtypes = [u64p, C.c_int, C.c_int, u64p, u64p, C.c_uint64]
            f.restype = None
        _ref = R
    return _ref


# ---------------------------------------------------------------------------------------------------------
# scalar helpers
# ---------------------------------------------------------------------------------------------------------

def gen_primes(bits: int, count: int, two_n: int, exclude=()) -> list[int]:
    ex = np.array(list(exclude) or [0], dtype=np.uint64)
    out = np.zeros(count, dtype=np.uint64)
    n = lib().orc_gen_primes(bits, count, two_n, _p(ex), len(exclude), _p(out))
    if n != count:
        raise ValueError(f"only {n} primes of {bits} bits found")
    return [int(x) for x in out]


def root_of_unity(p: int, order: int) -> int:
    return int(lib().orc_root_of_unity(p, order))


def ntt_tables(N: int, p: int, psi: int):
    tab = np.zeros(N, dtype=np.uint64)
    itab = np.zeros(N, dtype=np.uint64)
    lib().orc_ntt_tables(N, p, psi, _p(tab), _p(itab))
    return tab, itab


def ntt_fwd(a: np.ndarray, p: int, tab: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.uint64).copy()
    lib().orc_ntt_fwd(_p(a), a.size, p, _p(tab))
    return a


def ntt_inv(a: np.ndarray, p: int, itab: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.uint64).copy()
    lib().orc_ntt_inv(_p(a), a.size, p, _p(itab))
    return a


def ntt_batch(data: np.ndarray, prime_of: np.ndarray, moduli: np.ndarray, tabs: np.ndarray, inverse: bool,
              nthreads: int = 1) -> None:
    """In place over data[nlimbs][N]; tabs[nprimes][N] (forward or inverse tables)."""
    assert data.flags.c_contiguous and data.dtype == np.uint64
    po = np.ascontiguousarray(prime_of, dtype=np.int32)
    lib().orc_ntt_batch(_p(data), data.shape[0], data.shape[1], _p(po, i32p), _p(moduli), _p(tabs),
                        1 if inverse else 0, nthreads)


# ---------------------------------------------------------------------------------------------------------
# context
# ---------------------------------------------------------------------------------------------------------

class Ctx:
    """Oracle context over moduli q_0..q_{nq-1}, p_0..p_{np-1} with the given 2N-th roots."""

    def __init__(self, N: int, nq: int, np_: int, dnum: int, moduli, psis=None, threads: int = 1):
        self.N, self.nq, self.np, self.dnum = N, nq, np_, dnum
        self.moduli = np.array(moduli, dtype=np.uint64)
        self.psis = None if psis is None else np.array(psis, dtype=np.uint64)
        self._h = lib().orc_ctx_new(N, nq, np_, dnum, _p(self.moduli),
                                    None if self.psis is None else _p(self.psis))
        if not self._h:
            raise ValueError("bad oracle parameters")
        lib().orc_ctx_set_threads(self._h, threads)
        self.alpha = lib().orc_ctx_alpha(self._h)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.orc_ctx_free(h)
            self._h = None

    def beta(self, t: int) -> int:
        return (t + self.alpha - 1) // self.alpha

    def zeros(self, *shape) -> np.ndarray:
        return np.zeros(shape + (self.N,), dtype=np.uint64)

    def key_shape(self):
        return (2, self.dnum, self.nq + self.np, self.N)

    # --- ops ---
    def to_coeff(self, x: np.ndarray, tower_ids=None) -> np.ndarray:
        y = np.ascontiguousarray(x, dtype=np.uint64).copy()
        ids = None if tower_ids is None else np.ascontiguousarray(tower_ids, dtype=np.int32)
        lib().orc_to_coeff(self._h, _p(y), y.size // self.N, None if ids is None else _p(ids, i32p))
        return y

    def to_eval(self, x: np.ndarray, tower_ids=None) -> np.ndarray:
        y = np.ascontiguousarray(x, dtype=np.uint64).copy()
        ids = None if tower_ids is None else np.ascontiguousarray(tower_ids, dtype=np.int32)
        lib().orc_to_eval(self._h, _p(y), y.size // self.N, None if ids is None else _p(ids, i32p))
        return y

    def modup(self, a: np.ndarray, t: int) -> np.ndarray:
        out = self.zeros(self.beta(t), t + self.np)
        lib().orc_modup(self._h, _p(np.ascontiguousarray(a)), t, _p(out))
        return out

    def ks_inner(self, digits: np.ndarray, t: int, key: np.ndarray) -> np.ndarray:
        out = self.zeros(2, t + self.np)
        lib().orc_ks_inner(self._h, _p(np.ascontiguousarray(digits)), t, _p(key), _p(out))
        return out

    def moddown(self, x: np.ndarray, t: int) -> np.ndarray:
        out = self.zeros(t)
        lib().orc_moddown(self._h, _p(np.ascontiguousarray(x)), t, _p(out))
        return out

    def keyswitch(self, a: np.ndarray, t: int, key: np.ndarray) -> np.ndarray:
        out = self.zeros(2, t)
        lib().orc_keyswitch(self._h, _p(np.ascontiguousarray(a)), t, _p(key), _p(out))
        return out

    def automorph(self, x: np.ndarray, galois: int) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.uint64)
        out = np.zeros_like(x)
        lib().orc_automorph(self._h, _p(x), x.size // self.N, galois, _p(out))
        return out

    def galois(self, index: int) -> int:
        return int(lib().orc_galois_for_index(self.N, index))

    def rotate(self, ct: np.ndarray, galois: int, key: np.ndarray) -> np.ndarray:
        t = ct.shape[1]
        out = self.zeros(2, t)
        lib().orc_rotate(self._h, _p(np.ascontiguousarray(ct)), t, galois, _p(key), _p(out))
        return out

    def rotate_hoisted(self, ct: np.ndarray, galois: list[int], keys: list[np.ndarray]) -> list[np.ndarray]:
        t = ct.shape[1]
        n = len(galois)
        outs = [self.zeros(2, t) for _ in range(n)]
        g = np.array(galois, dtype=np.uint32)
        kp = (u64p * n)(*[_p(k) for k in keys])
        op = (u64p * n)(*[_p(o) for o in outs])
        lib().orc_rotate_hoisted(self._h, _p(np.ascontiguousarray(ct)), t, n, _p(g, u32p), kp, op)
        return outs

    def tensor(self, x: np.ndarray, y: np.ndarray) -> np.ndarray:
        t = x.shape[1]
        out = self.zeros(3, t)
        lib().orc_tensor(self._h, _p(np.ascontiguousarray(x)), _p(np.ascontiguousarray(y)), t, _p(out))
        return out

    def mult(self, x: np.ndarray, y: np.ndarray, rlk: np.ndarray) -> np.ndarray:
        t = x.shape[1]
        out = self.zeros(2, t)
        lib().orc_mult(self._h, _p(np.ascontiguousarray(x)), _p(np.ascontiguousarray(y)), t, _p(rlk), _p(out))
        return out

    def rescale(self, ct: np.ndarray) -> np.ndarray:
        t = ct.shape[1]
        out = self.zeros(2, t - 1)
        lib().orc_rescale(self._h, _p(np.ascontiguousarray(ct)), t, _p(out))
        return out

    def add(self, x: np.ndarray, y: np.ndarray) -> np.ndarray:
        out = np.zeros_like(x)
        lib().orc_add(self._h, _p(np.ascontiguousarray(x)), _p(np.ascontiguousarray(y)), x.shape[-2],
                      x.size // (x.shape[-2] * self.N), _p(out))
        return out

    def sub(self, x: np.ndarray, y: np.ndarray) -> np.ndarray:
        out = np.zeros_like(x)
        lib().orc_sub(self._h, _p(np.ascontiguousarray(x)), _p(np.ascontiguousarray(y)), x.shape[-2],
                      x.size // (x.shape[-2] * self.N), _p(out))
        return out

    def plain_op(self, ct: np.ndarray, pt: np.ndarray, mode: int) -> np.ndarray:
        t = ct.shape[1]
        out = self.zeros(2, t)
        lib().orc_plain_op(self._h, _p(np.ascontiguousarray(ct)), _p(np.ascontiguousarray(pt)), t, mode, _p(out))
        return out

    def scalar_op(self, ct: np.ndarray, mul, add) -> np.ndarray:
        t = ct.shape[1]
        out = self.zeros(2, t)
        m = np.ascontiguousarray(np.array(mul, dtype=np.uint64))
        a = np.ascontiguousarray(np.array(add, dtype=np.uint64))
        lib().orc_scalar_op(self._h, _p(np.ascontiguousarray(ct)), t, _p(m), _p(a), _p(out))
        return out

    def mod_raise(self, ct: np.ndarray, T: int) -> np.ndarray:
        out = self.zeros(2, T)
        lib().orc_mod_raise(self._h, _p(np.ascontiguousarray(ct)), ct.shape[1], T, _p(out))
        return out

    def mult_monomial(self, ct: np.ndarray, k: int) -> np.ndarray:
        out = self.zeros(2, ct.shape[1])
        lib().orc_mult_monomial(self._h, _p(np.ascontiguousarray(ct)), ct.shape[1], k, _p(out))
        return out

    def key_switch(self, ct: np.ndarray, key: np.ndarray) -> np.ndarray:
        """(c0, c1) -> (c0 + KS(c1)_0, KS(c1)_1): a rotation with the identity automorphism."""
        return self.rotate(ct, 1, key)

    # --- synthetic inputs ---
    def uniform(self, seed: int, ntowers: int, tower_ids=None) -> np.ndarray:
        out = self.zeros(ntowers)
        ids = None if tower_ids is None else np.ascontiguousarray(tower_ids, dtype=np.int32)
        lib().orc_rng_fill_uniform(self._h, seed, _p(out), ntowers, None if ids is None else _p(ids, i32p))
        return out

    def secret(self, seed: int, hamming_weight: int = 0) -> np.ndarray:
        s = np.zeros(self.N, dtype=np.int64)
        lib().orc_keygen_secret(self._h, seed, hamming_weight, _p(s, i64p))
        return s

    def relin_key(self, seed: int, s: np.ndarray) -> np.ndarray:
        k = np.zeros(self.key_shape(), dtype=np.uint64)
        lib().orc_relin_keygen(self._h, seed, _p(s, i64p), _p(k))
        return k

    def switch_key(self, seed: int, s_from: np.ndarray, s_to: np.ndarray) -> np.ndarray:
        """Key switching ciphertexts under s_from to s_to."""
        k = np.zeros(self.key_shape(), dtype=np.uint64)
        lib().orc_ksk_gen(self._h, seed, _p(np.ascontiguousarray(s_from), i64p),
                          _p(np.ascontiguousarray(s_to), i64p), _p(k))
        return k

    def rot_key(self, seed: int, s: np.ndarray, galois: int) -> np.ndarray:
        k = np.zeros(self.key_shape(), dtype=np.uint64)
        lib().orc_rot_keygen(self._h, seed, _p(s, i64p), galois, _p(k))
        return k

    def encode(self, z: np.ndarray, scale: float, t: int, tower_ids=None) -> np.ndarray:
        """Encoding into t rows (Q towers 0..t-1, or the rows tower_ids)."""
        z = np.asarray(z, dtype=np.complex128)
        re = np.ascontiguousarray(z.real)
        im = np.ascontiguousarray(z.imag)
        out = self.zeros(t)
        dp = C.POINTER(C.c_double)
        if tower_ids is None:
            lib().orc_encode(self._h, _p(re, dp), _p(im, dp), len(z), scale, t, _p(out))
        else:
            ids = np.ascontiguousarray(tower_ids, dtype=np.int32)
            lib().orc_encode_ids(self._h, _p(re, dp), _p(im, dp), len(z), scale, t, _p(ids, i32p), _p(out))
        return out

    def ext_ids(self, t: int) -> list[int]:
        """Tower ids of the extended basis Q_t ∪ P (rows of an extended ciphertext)."""
        return list(range(t)) + list(range(self.nq, self.nq + self.np))

    def ew(self, x: np.ndarray, y: np.ndarray, tower_ids, op: int) -> np.ndarray:
        """x * y (op 0) or x + y (op 1) limb-wise modulo tower_ids; x [polys][nl][N], y [nl][N] or like x."""
        x = np.ascontiguousarray(x, dtype=np.uint64)
        y = np.ascontiguousarray(y, dtype=np.uint64)
        nl = len(tower_ids)
        out = np.zeros_like(x)
        ids = np.ascontiguousarray(tower_ids, dtype=np.int32)
        lib().orc_ew_ids(self._h, _p(x), _p(y), nl, x.size // (nl * self.N), y.size // (nl * self.N), _p(ids, i32p),
                         op, _p(out))
        return out

    def decode(self, pt: np.ndarray, scale: float, slots: int) -> np.ndarray:
        t = pt.shape[0]
        re = np.zeros(slots)
        im = np.zeros(slots)
        lib().orc_decode(self._h, _p(np.ascontiguousarray(pt)), t, scale, slots, _p(re, C.POINTER(C.c_double)),
                         _p(im, C.POINTER(C.c_double)))
        return re + 1j * im

    def encrypt(self, seed: int, s: np.ndarray, pt: np.ndarray) -> np.ndarray:
        t = pt.shape[0]
        out = self.zeros(2, t)
        lib().orc_encrypt_sk(self._h, seed, _p(s, i64p), _p(np.ascontiguousarray(pt)), t, _p(out))
        return out

    def decrypt(self, s: np.ndarray, ct: np.ndarray) -> np.ndarray:
        t = ct.shape[1]
        out = self.zeros(t)
        lib().orc_decrypt(self._h, _p(s, i64p), _p(np.ascontiguousarray(ct)), t, _p(out))
        return out


def make_moduli(logN: int, q_bits: list[int], p_bits: list[int]) -> list[int]:
    """Primes == 1 mod 2N by descending search below 2^bits, distinct across the whole basis."""
    two_n = 1 << (logN + 1)
    chosen: list[int] = []
    for bits in list(q_bits) + list(p_bits):
        chosen += gen_primes(bits, 1, two_n, exclude=chosen)
    return chosen
