"""fideslib_gb300 — GB300-native CKKS evaluation engine (Python binding over the C ABI).

The engine itself is CUDA/C++ (fideslib_gb300/csrc) behind the C ABI declared in include/fideslib_gb300.h;
this module is a thin ctypes binding used by the tests and the benchmark.  It never falls back to a CPU
path: if the compiled library is missing, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libfideslib_gb300.so")
HEADER = os.path.join(HERE, "..", "include", "fideslib_gb300.h")

FIDES_OK, FIDES_EINVAL, FIDES_ENOKEY, FIDES_ENOMEM, FIDES_ECUDA, FIDES_ENODEV = 0, -1, -2, -3, -4, -5
FIXEDMANUAL, FIXEDAUTO, FLEXIBLEAUTO, FLEXIBLEAUTOEXT = 0, 1, 2, 3

u64p = C.POINTER(C.c_uint64)
u32p = C.POINTER(C.c_uint32)
i32p = C.POINTER(C.c_int32)


class FidesError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class RawInfo(C.Structure):
    _fields_ = [("kind", C.c_uint32), ("log_n", C.c_uint32), ("rows", C.c_uint32), ("polys", C.c_uint32),
                ("noise_deg", C.c_uint32), ("slots", C.c_uint32), ("id", C.c_uint32), ("reserved", C.c_uint32),
                ("scale", C.c_double)]


RAW_CIPHERTEXT, RAW_PLAINTEXT, RAW_RELIN_KEY, RAW_ROTATION_KEY, RAW_SWITCH_KEY = 1, 2, 3, 4, 5


class ProbeResult(C.Structure):
    _fields_ = [("sms", C.c_uint32), ("clock_mhz", C.c_double), ("imad32_per_clk_sm", C.c_double),
                ("imad_wide_per_clk_sm", C.c_double), ("butterflies_per_clk_sm", C.c_double),
                ("int8_mma_tops", C.c_double), ("launch_spacing_us", C.c_double)]


def probe_pipes() -> dict:
    """fides_probe_pipes: integer-pipe, butterfly, INT8 MMA and launch-spacing throughput of the current GPU."""
    r = ProbeResult()
    _check(lib().fides_probe_pipes(C.byref(r)))
    return {k: (round(getattr(r, k), 3) if isinstance(getattr(r, k), float) else getattr(r, k))
            for k, _ in ProbeResult._fields_}


class Params(C.Structure):
    _fields_ = [("log_n", C.c_uint32), ("nq", C.c_uint32), ("np", C.c_uint32), ("dnum", C.c_uint32),
                ("moduli", u64p), ("roots", u64p), ("scaling_technique", C.c_int32),
                ("scaling_factor_real", C.POINTER(C.c_double)), ("scaling_factor_real_big", C.POINTER(C.c_double)),
                ("mod_reduce_factor", C.POINTER(C.c_double)), ("default_scale", C.c_double)]


class CtMeta(C.Structure):
    _fields_ = [("towers", C.c_uint32), ("noise_deg", C.c_uint32), ("slots", C.c_uint32),
                ("reserved", C.c_uint32), ("scale", C.c_double)]


_lib = None

_SIGS = {
    "fides_last_error": (C.c_char_p, []),
    "fides_version": (C.c_char_p, []),
    "fides_find_primes": (C.c_int, [C.c_uint32, C.c_uint32, C.c_uint64, u64p, C.c_uint32, u64p]),
    "fides_ctx_create": (C.c_int, [C.POINTER(Params), C.POINTER(C.c_void_p)]),
    "fides_ctx_destroy": (C.c_int, [C.c_void_p]),
    "fides_ctx_moduli": (C.c_int, [C.c_void_p, u64p, u64p]),
    "fides_ctx_scaling": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_double),
                                    C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "fides_galois_element": (C.c_uint32, [C.c_void_p, C.c_int32]),
    "fides_synchronize": (C.c_int, [C.c_void_p]),
    "fides_ctx_stream": (C.c_void_p, [C.c_void_p]),
    "fides_ctx_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fides_kernel_launches": (C.c_uint64, []),
    "fides_ntt_batch_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int,
                                         C.c_void_p]),
    "fides_ntt_batch_host": (C.c_int, [C.c_void_p, u64p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int]),
    "fides_load_eval_mult_key": (C.c_int, [C.c_void_p, u64p]),
    "fides_load_eval_mult_key_device": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fides_load_rotation_key": (C.c_int, [C.c_void_p, C.c_uint32, u64p]),
    "fides_load_rotation_key_device": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p]),
    "fides_ct_load": (C.c_int, [C.c_void_p, u64p, C.POINTER(CtMeta), u32p]),
    "fides_ct_load_device": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(CtMeta), u32p]),
    "fides_ct_store": (C.c_int, [C.c_void_p, C.c_uint32, u64p, C.POINTER(CtMeta)]),
    "fides_ct_meta_get": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(CtMeta)]),
    "fides_ct_free": (C.c_int, [C.c_void_p, C.c_uint32]),
    "fides_eval_add": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, u32p]),
    "fides_eval_sub": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, u32p]),
    "fides_eval_mult": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, u32p]),
    "fides_eval_square": (C.c_int, [C.c_void_p, C.c_uint32, u32p]),
    "fides_rescale": (C.c_int, [C.c_void_p, C.c_uint32, u32p]),
    "fides_eval_rotate": (C.c_int, [C.c_void_p, C.c_uint32, C.c_int32, u32p]),
    "fides_eval_automorphism": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, u32p]),
    "fides_eval_fast_rotation": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, i32p, u32p]),
    "fides_fast_rotation_precompute": (C.c_int, [C.c_void_p, C.c_uint32, u32p]),
    "fides_eval_fast_rotation_precomputed": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_int32, u32p]),
    "fides_precompute_free": (C.c_int, [C.c_void_p, C.c_uint32]),
    "fides_eval_batch_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32]),
    "fides_eval_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32]),
    "fides_ctx_get_shape": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fides_pt_load": (C.c_int, [C.c_void_p, u64p, C.c_uint32, C.c_double, u32p]),
    "fides_pt_free": (C.c_int, [C.c_void_p, C.c_uint32]),
    "fides_eval_mult_plain": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, u32p]),
    "fides_eval_add_plain": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, u32p]),
    "fides_eval_sub_plain": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, u32p]),
    "fides_eval_mult_int": (C.c_int, [C.c_void_p, C.c_uint32, C.c_int64, u32p]),
    "fides_eval_mult_scalar": (C.c_int, [C.c_void_p, C.c_uint32, C.c_double, C.c_double, u32p]),
    "fides_eval_add_scalar": (C.c_int, [C.c_void_p, C.c_uint32, C.c_double, u32p]),
    "fides_eval_fast_rotation_ext": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.POINTER(C.c_int32),
                                               C.c_int32, u32p]),
    "fides_ext_add": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, u32p]),
    "fides_pt_load_ext": (C.c_int, [C.c_void_p, u64p, C.c_uint32, C.c_double, u32p]),
    "fides_ext_mult_plain": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, u32p]),
    "fides_key_switch_down": (C.c_int, [C.c_void_p, C.c_uint32, u32p]),
    "fides_ext_store": (C.c_int, [C.c_void_p, C.c_uint32, u64p, C.c_void_p]),
    "fides_eval_many_to_one": (C.c_int, [C.c_void_p, C.c_int32, C.c_uint32, C.c_uint32, u32p, u32p,
                                         C.POINTER(C.c_double), C.POINTER(C.c_double), u32p]),
    "fides_eval_linear_wsum": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, u32p, C.POINTER(C.c_double),
                                         C.POINTER(C.c_double), u32p]),
    "fides_level_reduce": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, u32p]),
    "fides_mod_raise": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, u32p]),
    "fides_lt_create": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, u64p, C.POINTER(C.c_uint8),
                                  C.c_double, u32p]),
    "fides_lt_create_strided": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_int32, C.c_int32, C.c_uint32,
                                          u64p, C.POINTER(C.c_uint8), C.c_double, u32p]),
    "fides_lt_create_strided_ext": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_int32, C.c_int32,
                                              C.c_uint32, u64p, C.POINTER(C.c_uint8), C.c_double, u32p]),
    "fides_lt_free": (C.c_int, [C.c_void_p, C.c_uint32]),
    "fides_ctx_ntt_tuning": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "fides_ctx_ntt_tuning_set": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "fides_ctx_ks_tuning": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_float)]),
    "fides_ctx_ks_tuning_set": (C.c_int, [C.c_void_p, C.c_int32]),
    "fides_ctx_set_mem_limit": (C.c_int, [C.c_void_p, C.c_uint64]),
    "fides_ctx_mem_in_use": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "fides_ctx_set_input_check": (C.c_int, [C.c_void_p, C.c_int]),
    "fides_probe_pipes": (C.c_int, [C.c_void_p]),
    "fides_raw_write": (C.c_int, [C.c_char_p, C.c_void_p, u64p, u64p, u64p]),
    "fides_raw_read_info": (C.c_int, [C.c_char_p, C.c_void_p]),
    "fides_raw_read": (C.c_int, [C.c_char_p, C.c_void_p, u64p, u64p, u64p]),
    "fides_ct_save": (C.c_int, [C.c_void_p, C.c_uint32, C.c_char_p]),
    "fides_ct_load_file": (C.c_int, [C.c_void_p, C.c_char_p, u32p]),
    "fides_key_load_file": (C.c_int, [C.c_void_p, C.c_char_p]),
    "fides_pt_encode": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_uint32, C.c_double,
                                  C.c_uint32, u32p]),
    "fides_pt_decode": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "fides_pt_store": (C.c_int, [C.c_void_p, C.c_uint32, u64p]),
    "fides_lt_create_slots": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_int32, C.c_int32, C.c_uint32,
                                        C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_uint8),
                                        C.c_uint32, C.c_double, u32p]),
    "fides_lt_create_slots_ext": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, C.c_int32, C.c_int32, C.c_uint32,
                                            C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_uint8),
                                            C.c_uint32, C.c_double, u32p]),
    "fides_load_switch_key": (C.c_int, [C.c_void_p, C.c_uint32, u64p]),
    "fides_load_switch_key_device": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p]),
    "fides_eval_key_switch": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, u32p]),
    "fides_eval_mult_monomial": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, u32p]),
    "fides_eval_linear_transform": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, u32p]),
    "fides_eval_linear_transform_batch": (C.c_int, [C.c_void_p, C.c_uint32, u32p, C.c_uint32, u32p]),
    "fides_eval_chebyshev": (C.c_int, [C.c_void_p, C.c_uint32, C.POINTER(C.c_double), C.c_uint32, C.c_double,
                                       C.c_double, C.c_double, u32p]),
    "fides_eval_double_angle": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32, u32p]),
    "fides_eval_bootstrap": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, u32p]),
    "fides_eval_bootstrap_batch": (C.c_int, [C.c_void_p, C.c_uint32, u32p, C.c_void_p, u32p]),
    "fides_eval_chebyshev_batch": (C.c_int, [C.c_void_p, C.c_uint32, u32p, C.POINTER(C.c_double), C.c_uint32,
                                             C.c_double, C.c_double, C.c_double, u32p]),
    "fides_eval_double_angle_batch": (C.c_int, [C.c_void_p, C.c_uint32, u32p, C.c_uint32, u32p]),
    "fides_server_create": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
    "fides_server_submit": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_uint64)]),
    "fides_server_submit_to": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.POINTER(C.c_uint64)]),
    "fides_server_create_multi": (C.c_int, [C.c_void_p, C.c_uint32, C.c_void_p, C.POINTER(C.c_void_p)]),
    "fides_server_set_bootstrap_plan": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fides_server_wait": (C.c_int, [C.c_void_p, C.c_uint64, u32p, C.POINTER(C.c_double)]),
    "fides_server_release": (C.c_int, [C.c_void_p, C.c_uint64]),
    "fides_server_stats_get": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fides_server_reset_stats": (C.c_int, [C.c_void_p]),
    "fides_server_destroy": (C.c_int, [C.c_void_p]),
    "fides_eval_rotate_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p,
                                            C.c_void_p]),
}

OP_ADD, OP_SUB, OP_MULT, OP_SQUARE, OP_RESCALE, OP_ROTATE, OP_AUTOMORPHISM, OP_KEY_SWITCH, OP_BOOTSTRAP = range(1, 10)
OP_MULT_PLAIN, OP_ADD_PLAIN, OP_SUB_PLAIN, OP_MULT_SCALAR, OP_ADD_SCALAR, OP_MULT_INT = range(10, 16)


class HostOp(C.Structure):
    _fields_ = [("op", C.c_int32), ("a", C.c_void_p), ("b", C.c_void_p), ("meta", CtMeta), ("index", C.c_int32),
                ("out", C.c_void_p), ("out_meta", CtMeta)]


class Op(C.Structure):
    _fields_ = [("op", C.c_int32), ("a", C.c_uint32), ("b", C.c_uint32), ("index", C.c_int32), ("out", C.c_uint32)]


def lib():
    """Loads the compiled engine; raises if it has not been built (there is no fallback)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"fideslib_gb300 CUDA library missing ({LIB_PATH}); "
                               "build it with `python -m fideslib_gb300.build`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name, None)
            if f is None:
                continue
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def raw_write(path: str, kind: int, data: np.ndarray, moduli, roots=None, noise_deg: int = 1, slots: int = 0,
              ident: int = 0, scale: float = 0.0):
    """data: u64[polys][rows][N] (host) to a raw residue file (fides_raw_write)."""
    data = np.ascontiguousarray(data, dtype=np.uint64)
    polys, rows, n = data.shape
    info = RawInfo(kind, n.bit_length() - 1, rows, polys, noise_deg, slots, ident, 0, scale)
    m = np.ascontiguousarray(np.array(moduli[:rows], dtype=np.uint64))
    r = None if roots is None else np.ascontiguousarray(np.array(roots[:rows], dtype=np.uint64))
    _check(lib().fides_raw_write(path.encode(), C.byref(info), _p(m), None if r is None else _p(r), _p(data)))


def raw_read(path: str):
    """(info, moduli, roots, data[polys][rows][N]) of a raw residue file (fides_raw_read)."""
    info = RawInfo()
    _check(lib().fides_raw_read_info(path.encode(), C.byref(info)))
    m = np.zeros(info.rows, dtype=np.uint64)
    r = np.zeros(info.rows, dtype=np.uint64)
    d = np.zeros((info.polys, info.rows, 1 << info.log_n), dtype=np.uint64)
    _check(lib().fides_raw_read(path.encode(), C.byref(info), _p(m), _p(r), _p(d)))
    return info, m, r, d


def declared_symbols() -> list[str]:
    """Function names declared in include/fideslib_gb300.h."""
    import re
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(fides_\w+)\s*\(", src, re.M)))


def _check(rc: int):
    if rc != FIDES_OK:
        raise FidesError(rc, lib().fides_last_error().decode())


def _p(a: np.ndarray, t=u64p):
    return a.ctypes.data_as(t)


class CryptoContext:
    """Device context: moduli, roots and all derived tables resident on the GPU (LoadContext)."""

    def __init__(self, log_n: int, moduli, np_: int, dnum: int, roots=None, scaling_technique: int = FIXEDMANUAL,
                 scaling_tables=None, default_scale: float = 0.0):
        """scaling_tables: optional (scaling_factor_real, scaling_factor_real_big, mod_reduce_factor), nq doubles
        each indexed by towers - 1 (RawParams' tables); None computes them for the technique."""
        moduli = np.ascontiguousarray(np.array(moduli, dtype=np.uint64))
        self.N = 1 << log_n
        self.log_n = log_n
        self.np = np_
        self.nq = len(moduli) - np_
        self.dnum = dnum
        self.alpha = (self.nq + dnum - 1) // dnum
        r = None if roots is None else np.ascontiguousarray(np.array(roots, dtype=np.uint64))
        dp = C.POINTER(C.c_double)
        tabs = [None, None, None]
        if scaling_tables is not None:
            tabs = [np.ascontiguousarray(np.array(x, dtype=np.float64)) for x in scaling_tables]
        prm = Params(log_n, self.nq, np_, dnum, _p(moduli), None if r is None else _p(r), scaling_technique,
                     *[None if x is None else x.ctypes.data_as(dp) for x in tabs], default_scale)
        h = C.c_void_p()
        _check(lib().fides_ctx_create(C.byref(prm), C.byref(h)))
        self._h = h
        m = np.zeros(self.nq + np_, dtype=np.uint64)
        rr = np.zeros(self.nq + np_, dtype=np.uint64)
        _check(lib().fides_ctx_moduli(self._h, _p(m), _p(rr)))
        self.moduli = [int(x) for x in m]
        self.roots = [int(x) for x in rr]

    def close(self):
        if getattr(self, "_h", None):
            lib().fides_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def scaling(self):
        """(technique, scaling_factor_real, scaling_factor_real_big, mod_reduce_factor) in use."""
        t = C.c_int32()
        sf, big, mrf = (np.zeros(self.nq) for _ in range(3))
        dp = C.POINTER(C.c_double)
        _check(lib().fides_ctx_scaling(self._h, C.byref(t), sf.ctypes.data_as(dp), big.ctypes.data_as(dp),
                                       mrf.ctypes.data_as(dp)))
        return t.value, sf, big, mrf

    # --- primitives ---
    def galois(self, index: int) -> int:
        return int(lib().fides_galois_element(self._h, index))

    def synchronize(self):
        _check(lib().fides_synchronize(self._h))

    @property
    def stream(self) -> int:
        return int(lib().fides_ctx_stream(self._h) or 0)

    def set_stream(self, stream: int | None):
        _check(lib().fides_ctx_set_stream(self._h, None if not stream else C.c_void_p(stream)))


    def save_ciphertext(self, h: int, path: str):
        _check(lib().fides_ct_save(self._h, h, path.encode()))

    def load_ciphertext_file(self, path: str) -> int:
        h = C.c_uint32()
        _check(lib().fides_ct_load_file(self._h, path.encode(), C.byref(h)))
        return h.value

    def load_key_file(self, path: str):
        _check(lib().fides_key_load_file(self._h, path.encode()))

    def set_input_check(self, enable: bool = True):
        """Opt-in check that loaded residues are below their primes (loads refuse others with FIDES_EINVAL)."""
        _check(lib().fides_ctx_set_input_check(self._h, 1 if enable else 0))

    def ntt_host(self, data: np.ndarray, first_prime: int = 0, inverse: bool = False) -> np.ndarray:
        """data: u64[npolys][limbs][N] (host), transformed in place and returned."""
        assert data.dtype == np.uint64 and data.flags.c_contiguous and data.ndim == 3
        _check(lib().fides_ntt_batch_host(self._h, _p(data), data.shape[0], data.shape[1], first_prime,
                                          1 if inverse else 0))
        return data

    def ntt_device(self, ptr: int, npolys: int, limbs: int, first_prime: int = 0, inverse: bool = False,
                   stream: int | None = None):
        _check(lib().fides_ntt_batch_device(self._h, C.c_void_p(ptr), npolys, limbs, first_prime,
                                            1 if inverse else 0, None if stream is None else C.c_void_p(stream)))

    # --- keys ---
    def load_eval_mult_key(self, key: np.ndarray):
        key = np.ascontiguousarray(key, dtype=np.uint64)
        _check(lib().fides_load_eval_mult_key(self._h, _p(key)))

    def load_eval_mult_key_device(self, ptr: int):
        _check(lib().fides_load_eval_mult_key_device(self._h, C.c_void_p(ptr)))

    def load_rotation_key(self, galois: int, key: np.ndarray):
        key = np.ascontiguousarray(key, dtype=np.uint64)
        _check(lib().fides_load_rotation_key(self._h, galois, _p(key)))

    def load_switch_key(self, key_id: int, key: np.ndarray):
        key = np.ascontiguousarray(key, dtype=np.uint64)
        _check(lib().fides_load_switch_key(self._h, key_id, _p(key)))

    def load_switch_key_device(self, key_id: int, ptr: int):
        _check(lib().fides_load_switch_key_device(self._h, key_id, C.c_void_p(ptr)))

    def eval_key_switch(self, a: int, key_id: int) -> int:
        return self._un(lib().fides_eval_key_switch, a, key_id)

    def load_rotation_key_device(self, galois: int, ptr: int):
        _check(lib().fides_load_rotation_key_device(self._h, galois, C.c_void_p(ptr)))

    # --- ciphertexts ---
    def load_ciphertext(self, ct: np.ndarray, scale: float = 1.0, noise_deg: int = 1, slots: int = 0) -> int:
        ct = np.ascontiguousarray(ct, dtype=np.uint64)
        assert ct.ndim == 3 and ct.shape[0] == 2 and ct.shape[2] == self.N
        meta = CtMeta(ct.shape[1], noise_deg, slots, 0, scale)
        h = C.c_uint32()
        _check(lib().fides_ct_load(self._h, _p(ct), C.byref(meta), C.byref(h)))
        return h.value

    def load_ciphertext_device(self, ptr: int, towers: int, scale: float = 1.0, noise_deg: int = 1,
                               slots: int = 0) -> int:
        meta = CtMeta(towers, noise_deg, slots, 0, scale)
        h = C.c_uint32()
        _check(lib().fides_ct_load_device(self._h, C.c_void_p(ptr), C.byref(meta), C.byref(h)))
        return h.value

    def meta(self, h: int) -> CtMeta:
        m = CtMeta()
        _check(lib().fides_ct_meta_get(self._h, h, C.byref(m)))
        return m

    def store_ciphertext(self, h: int, out: np.ndarray | None = None) -> np.ndarray:
        m = self.meta(h)
        if out is None:
            out = np.empty((2, m.towers, self.N), dtype=np.uint64)
        _check(lib().fides_ct_store(self._h, h, _p(out), None))
        return out

    def free(self, h: int):
        _check(lib().fides_ct_free(self._h, h))

    # --- evaluation ---
    def _bin(self, fn, a, b) -> int:
        o = C.c_uint32()
        _check(fn(self._h, a, b, C.byref(o)))
        return o.value

    def eval_add(self, a: int, b: int) -> int:
        return self._bin(lib().fides_eval_add, a, b)

    def eval_sub(self, a: int, b: int) -> int:
        return self._bin(lib().fides_eval_sub, a, b)

    def eval_mult(self, a: int, b: int) -> int:
        return self._bin(lib().fides_eval_mult, a, b)

    def eval_square(self, a: int) -> int:
        o = C.c_uint32()
        _check(lib().fides_eval_square(self._h, a, C.byref(o)))
        return o.value

    def rescale(self, a: int) -> int:
        o = C.c_uint32()
        _check(lib().fides_rescale(self._h, a, C.byref(o)))
        return o.value

    def eval_rotate(self, a: int, index: int) -> int:
        return self._bin(lib().fides_eval_rotate, a, index)

    def eval_automorphism(self, a: int, galois: int) -> int:
        return self._bin(lib().fides_eval_automorphism, a, galois)

    # --- plaintexts, scalars, levels, bootstrap building blocks ---
    def load_plaintext(self, pt: np.ndarray, scale: float = 1.0) -> int:
        pt = np.ascontiguousarray(pt, dtype=np.uint64)
        h = C.c_uint32()
        _check(lib().fides_pt_load(self._h, _p(pt), pt.shape[0], scale, C.byref(h)))
        return h.value

    def free_plaintext(self, h: int):
        _check(lib().fides_pt_free(self._h, h))

    def _un(self, fn, *args) -> int:
        o = C.c_uint32()
        _check(fn(self._h, *args, C.byref(o)))
        return o.value

    def eval_mult_plain(self, a: int, pt: int) -> int:
        return self._un(lib().fides_eval_mult_plain, a, pt)

    def eval_add_plain(self, a: int, pt: int) -> int:
        return self._un(lib().fides_eval_add_plain, a, pt)

    def eval_sub_plain(self, a: int, pt: int) -> int:
        return self._un(lib().fides_eval_sub_plain, a, pt)

    def eval_mult_int(self, a: int, k: int) -> int:
        return self._un(lib().fides_eval_mult_int, a, k)

    def eval_mult_scalar(self, a: int, v: float, scale: float) -> int:
        return self._un(lib().fides_eval_mult_scalar, a, v, scale)

    def eval_add_scalar(self, a: int, v: float) -> int:
        return self._un(lib().fides_eval_add_scalar, a, v)

    def eval_many_to_one(self, op: int, a, b=None, values=None, scales=None, stride: int = 1,
                         in_place: bool = False):
        """Many-to-one batch (fides_eval_many_to_one): a[i*stride + j] combined with operand i (b[i], or
        values[i] / scales[i] for the scalar ops).  Returns the result handles, or None when in place."""
        a_arr = np.ascontiguousarray(np.array(a, dtype=np.uint32))
        nb = len(a_arr) // stride
        assert nb * stride == len(a_arr)
        u32 = C.POINTER(C.c_uint32)
        f64 = C.POINTER(C.c_double)
        b_arr = None if b is None else np.ascontiguousarray(np.array(b, dtype=np.uint32))
        v_arr = None if values is None else np.ascontiguousarray(np.array(values, dtype=np.float64))
        s_arr = None if scales is None else np.ascontiguousarray(np.array(scales, dtype=np.float64))
        outs = None if in_place else np.zeros(len(a_arr), dtype=np.uint32)

        def ptr(x, t):
            return None if x is None else x.ctypes.data_as(t)

        _check(lib().fides_eval_many_to_one(self._h, op, nb, stride, ptr(a_arr, u32), ptr(b_arr, u32),
                                            ptr(v_arr, f64), ptr(s_arr, f64), ptr(outs, u32)))
        return None if in_place else [int(x) for x in outs]

    def eval_linear_wsum(self, terms, weights, scales) -> list[int]:
        """Weighted sums in lock step (fides_eval_linear_wsum): terms[k][i] is term k of sum i, weights[k] its
        weight, scales[k][i] the scale its weight is encoded at; returns one handle per sum."""
        t = np.ascontiguousarray(np.array(terms, dtype=np.uint32))
        n, m = t.shape
        w = np.ascontiguousarray(np.array(weights, dtype=np.float64))
        sc = np.ascontiguousarray(np.array(scales, dtype=np.float64).reshape(n, m))
        outs = np.zeros(m, dtype=np.uint32)
        f64 = C.POINTER(C.c_double)
        _check(lib().fides_eval_linear_wsum(self._h, m, n, _p(t, u32p), w.ctypes.data_as(f64), sc.ctypes.data_as(f64),
                                            _p(outs, u32p)))
        return [int(x) for x in outs]

    # --- extended-basis ciphertexts (EvalFastRotationExt / KeySwitchDown) ---
    def eval_fast_rotation_ext(self, a: int, indices, add_first: bool = True, pre: int = 0) -> list[int]:
        idx = np.ascontiguousarray(np.array(indices, dtype=np.int32))
        outs = np.zeros(len(idx), dtype=np.uint32)
        _check(lib().fides_eval_fast_rotation_ext(self._h, a, pre, len(idx), idx.ctypes.data_as(C.POINTER(C.c_int32)),
                                                  1 if add_first else 0, _p(outs, u32p)))
        return [int(x) for x in outs]

    def ext_add(self, a: int, b: int) -> int:
        return self._un(lib().fides_ext_add, a, b)

    def load_plaintext_ext(self, pt: np.ndarray, towers: int, scale: float = 1.0) -> int:
        """pt: u64[towers + np][N] (Q rows, then the special rows)."""
        pt = np.ascontiguousarray(pt, dtype=np.uint64)
        assert pt.shape[0] == towers + self.np
        h = C.c_uint32()
        _check(lib().fides_pt_load_ext(self._h, _p(pt), towers, scale, C.byref(h)))
        return h.value

    def ext_mult_plain(self, a: int, pt: int) -> int:
        return self._un(lib().fides_ext_mult_plain, a, pt)

    def key_switch_down(self, a: int) -> int:
        return self._un(lib().fides_key_switch_down, a)

    def store_ext(self, h: int, towers: int) -> np.ndarray:
        out = np.zeros((2, towers + self.np, self.N), dtype=np.uint64)
        _check(lib().fides_ext_store(self._h, h, _p(out), None))
        return out

    def level_reduce(self, a: int, towers: int) -> int:
        return self._un(lib().fides_level_reduce, a, towers)

    def mod_raise(self, a: int, towers: int) -> int:
        return self._un(lib().fides_mod_raise, a, towers)

    def lt_create(self, bs: int, gs: int, diags: np.ndarray, present, scale: float = 1.0, stride: int = 1,
                  base: int = 0, ext: bool = False) -> int:
        """diags: u64[gs*bs][towers][N], diagonal k = g*bs+b (slot offset base + k*stride) pre-rotated by
        -(base + g*bs*stride); present: bool[gs*bs].  ext: every diagonal carries towers + np rows (the special
        primes last) and the transform is evaluated double-hoisted."""
        diags = np.ascontiguousarray(diags, dtype=np.uint64)
        pres = np.ascontiguousarray(np.array(present, dtype=np.uint8))
        h = C.c_uint32()
        fn = lib().fides_lt_create_strided_ext if ext else lib().fides_lt_create_strided
        towers = diags.shape[1] - (self.np if ext else 0)
        _check(fn(self._h, bs, gs, stride, base, towers, _p(diags), pres.ctypes.data_as(C.POINTER(C.c_uint8)),
                  scale, C.byref(h)))
        return h.value

    def eval_linear_transform_batch(self, cts, lt: int) -> list[int]:
        a = np.ascontiguousarray(np.array(cts, dtype=np.uint32))
        out = np.zeros(len(a), dtype=np.uint32)
        _check(lib().fides_eval_linear_transform_batch(self._h, len(a), _p(a, u32p), lt, _p(out, u32p)))
        return [int(x) for x in out]

    def lt_create_device(self, bs: int, gs: int, ptr: int, towers: int, present, scale: float = 1.0,
                         stride: int = 1, base: int = 0) -> int:
        """Diagonals already in device memory (u64[gs*bs][towers][N] at ptr)."""
        pres = np.ascontiguousarray(np.array(present, dtype=np.uint8))
        h = C.c_uint32()
        _check(lib().fides_lt_create_strided(self._h, bs, gs, stride, base, towers, C.cast(C.c_void_p(ptr), u64p),
                                             pres.ctypes.data_as(C.POINTER(C.c_uint8)), scale, C.byref(h)))
        return h.value

    def ntt_tuning(self) -> dict:
        """The forward-NTT variants the autotuner chose at creation (small / large launches) and the timings."""
        v = (C.c_int32 * 6)()
        ms = (C.c_float * 18)()
        _check(lib().fides_ctx_ntt_tuning(self._h, v, ms))
        r = lambda a, b: [round(ms[i], 4) for i in range(a, b)]  # noqa: E731
        return {"fwd_variant_tiny": v[0], "fwd_variant_small": v[1], "fwd_variant_large": v[2],
                "inv_variant_tiny": v[3], "inv_variant_small": v[4], "inv_variant_large": v[5],
                "fwd_ms_tiny": r(0, 3), "fwd_ms_small": r(3, 6), "fwd_ms_large": r(6, 9),
                "inv_ms_tiny": r(9, 12), "inv_ms_small": r(12, 15), "inv_ms_large": r(15, 18)}

    def set_mem_limit(self, nbytes: int):
        _check(lib().fides_ctx_set_mem_limit(self._h, nbytes))

    def mem_in_use(self) -> int:
        v = C.c_uint64()
        _check(lib().fides_ctx_mem_in_use(self._h, C.byref(v)))
        return v.value

    def set_ntt_variant(self, fwd_variant: int, inv_variant: int = 0):
        _check(lib().fides_ctx_ntt_tuning_set(self._h, fwd_variant, inv_variant))

    def ks_tuning(self) -> dict:
        """The key inner product's tile the autotuner chose (coefficient pairs per thread) and its timings."""
        it = C.c_int32()
        ms = (C.c_float * 5)()
        _check(lib().fides_ctx_ks_tuning(self._h, C.byref(it), ms))
        return {"pairs_per_thread": it.value, "ms_1_2_4_8_16": [round(ms[i], 4) for i in range(5)]}

    def set_ks_tile(self, pairs_per_thread: int):
        _check(lib().fides_ctx_ks_tuning_set(self._h, pairs_per_thread))

    def encode(self, z, scale: float, towers: int) -> int:
        """Plaintext handle: the slot vector z (complex, length a power of two <= N/2) encoded on the GPU."""
        z = np.asarray(z, dtype=np.complex128)
        re, im = np.ascontiguousarray(z.real), np.ascontiguousarray(z.imag)
        h = C.c_uint32()
        dp = C.POINTER(C.c_double)
        _check(lib().fides_pt_encode(self._h, re.ctypes.data_as(dp), im.ctypes.data_as(dp), len(z), scale, towers,
                                     C.byref(h)))
        return h.value

    def decode(self, pt: int, slots: int) -> np.ndarray:
        re, im = np.zeros(slots), np.zeros(slots)
        dp = C.POINTER(C.c_double)
        _check(lib().fides_pt_decode(self._h, pt, slots, re.ctypes.data_as(dp), im.ctypes.data_as(dp)))
        return re + 1j * im

    def store_plaintext(self, pt: int, towers: int) -> np.ndarray:
        out = np.zeros((towers, self.N), dtype=np.uint64)
        _check(lib().fides_pt_store(self._h, pt, _p(out)))
        return out

    def lt_create_slots(self, bs: int, gs: int, diags, present, scale: float, towers: int, stride: int = 1,
                        base: int = 0, ext: bool = False) -> int:
        """diags: complex [bs*gs][slots] (rows of absent diagonals ignored), encoded on the GPU (also at the
        special primes when ext: a double-hoisted transform)."""
        d = np.asarray(diags, dtype=np.complex128)
        re, im = np.ascontiguousarray(d.real), np.ascontiguousarray(d.imag)
        pres = np.ascontiguousarray(np.array(present, dtype=np.uint8))
        h = C.c_uint32()
        dp = C.POINTER(C.c_double)
        fn = lib().fides_lt_create_slots_ext if ext else lib().fides_lt_create_slots
        _check(fn(self._h, bs, gs, stride, base, towers, re.ctypes.data_as(dp), im.ctypes.data_as(dp),
                  pres.ctypes.data_as(C.POINTER(C.c_uint8)), d.shape[1], scale, C.byref(h)))
        return h.value

    def eval_mult_monomial(self, a: int, k: int) -> int:
        return self._un(lib().fides_eval_mult_monomial, a, k)

    def lt_free(self, h: int):
        _check(lib().fides_lt_free(self._h, h))

    def eval_linear_transform(self, a: int, lt: int) -> int:
        return self._un(lib().fides_eval_linear_transform, a, lt)

    def eval_chebyshev(self, a: int, coeffs, lo: float, hi: float, const_scale: float) -> int:
        c = np.ascontiguousarray(np.array(coeffs, dtype=np.float64))
        return self._un(lib().fides_eval_chebyshev, a, c.ctypes.data_as(C.POINTER(C.c_double)), len(c), lo, hi,
                        const_scale)

    def eval_double_angle(self, a: int, iterations: int) -> int:
        return self._un(lib().fides_eval_double_angle, a, iterations)

    def eval_bootstrap(self, a: int, plan: "BootstrapPlan") -> int:
        return self._un(lib().fides_eval_bootstrap, a, C.byref(plan))

    def _many(self, fn, cts, *args) -> list[int]:
        a = np.ascontiguousarray(np.array(cts, dtype=np.uint32))
        out = np.zeros(len(a), dtype=np.uint32)
        _check(fn(self._h, len(a), _p(a, u32p), *args, _p(out, u32p)))
        return [int(x) for x in out]

    def eval_bootstrap_batch(self, cts, plan: "BootstrapPlan") -> list[int]:
        return self._many(lib().fides_eval_bootstrap_batch, cts, C.byref(plan))

    def eval_chebyshev_batch(self, cts, coeffs, lo: float, hi: float, const_scale: float) -> list[int]:
        c = np.ascontiguousarray(np.array(coeffs, dtype=np.float64))
        return self._many(lib().fides_eval_chebyshev_batch, cts, c.ctypes.data_as(C.POINTER(C.c_double)), len(c),
                          lo, hi, const_scale)

    def eval_double_angle_batch(self, cts, iterations: int) -> list[int]:
        return self._many(lib().fides_eval_double_angle_batch, cts, iterations)

    def eval_batch(self, ops) -> list[int]:
        """ops: iterable of (op_code, a, b, index); returns result handles (one batched pipeline per op family)."""
        ops = list(ops)
        arr = (Op * max(1, len(ops)))()
        for i, (code, a, b, index) in enumerate(ops):
            arr[i] = Op(code, a, b, index, 0)
        _check(lib().fides_eval_batch(self._h, arr, len(ops)))
        return [arr[i].out for i in range(len(ops))]

    def eval_batch_host(self, ops, chunk: int = 0) -> list[CtMeta]:
        """ops: iterable of (op_code, a, b, index, out, scale) with a / b / out host u64[2][t][N] arrays (b None
        for unary ops; out sized for the result).  Results are written into `out`; returns their metadata."""
        ops = list(ops)
        arr = (HostOp * max(1, len(ops)))()
        keep = []
        for i, (code, a, b, index, out, scale) in enumerate(ops):
            for x in (a, b, out):
                if x is not None:
                    assert x.dtype == np.uint64 and x.flags["C_CONTIGUOUS"] and x.shape[-1] == self.N
                    keep.append(x)
            arr[i] = HostOp(code, a.ctypes.data, b.ctypes.data if b is not None else None,
                            CtMeta(a.shape[1], 1, 0, 0, scale), index, out.ctypes.data, CtMeta())
        _check(lib().fides_eval_batch_host(self._h, arr, len(ops), chunk))
        return [arr[i].out_meta for i in range(len(ops))]

    def fast_rotation_precompute(self, a: int) -> int:
        h = C.c_uint32()
        _check(lib().fides_fast_rotation_precompute(self._h, a, C.byref(h)))
        return h.value

    def eval_fast_rotation_precomputed(self, a: int, pre: int, index: int) -> int:
        return self._un(lib().fides_eval_fast_rotation_precomputed, a, pre, index)

    def precompute_free(self, pre: int):
        _check(lib().fides_precompute_free(self._h, pre))

    def eval_fast_rotation(self, a: int, indices) -> list[int]:
        idx = np.ascontiguousarray(np.array(indices, dtype=np.int32))
        outs = np.zeros(len(idx), dtype=np.uint32)
        _check(lib().fides_eval_fast_rotation(self._h, a, len(idx), _p(idx, i32p), _p(outs, u32p)))
        return [int(x) for x in outs]


def kernel_launches() -> int:
    """Engine kernels launched by this process so far."""
    return int(lib().fides_kernel_launches())


class BootstrapPlan(C.Structure):
    _fields_ = [("slots", C.c_uint32), ("raise_towers", C.c_uint32), ("cts_count", C.c_uint32),
                ("lt_cts", C.c_uint32 * 4), ("stc_count", C.c_uint32), ("lt_stc", C.c_uint32 * 4),
                ("sse", C.c_uint32), ("sse_to_sparse", C.c_uint32), ("sse_to_dense", C.c_uint32),
                ("cheb_coeffs", C.POINTER(C.c_double)), ("cheb_n", C.c_uint32), ("double_angle", C.c_uint32),
                ("cheb_lo", C.c_double), ("cheb_hi", C.c_double), ("const_scale", C.c_double),
                ("prescale", C.c_double)]

    @classmethod
    def make(cls, slots: int, raise_towers: int, lt_cts, lt_stc, coeffs: np.ndarray, double_angle: int,
             lo: float, hi: float, const_scale: float, sse_keys=None, prescale: float = 0.0) -> "BootstrapPlan":
        """lt_cts / lt_stc: factor handles in application order; sse_keys: (to_sparse_id, to_dense_id) or None;
        prescale: 0 for a prescaled input, else the factor of the input's adjustment multiply-and-rescale.
        Keeps a reference to the coefficient buffer for the plan's lifetime."""
        c = np.ascontiguousarray(np.array(coeffs, dtype=np.float64))
        p = cls()
        p.slots, p.raise_towers = slots, raise_towers
        p.cts_count, p.stc_count = len(lt_cts), len(lt_stc)
        for i, h in enumerate(lt_cts):
            p.lt_cts[i] = h
        for i, h in enumerate(lt_stc):
            p.lt_stc[i] = h
        if sse_keys is not None:
            p.sse, p.sse_to_sparse, p.sse_to_dense = 1, sse_keys[0], sse_keys[1]
        p.cheb_coeffs = c.ctypes.data_as(C.POINTER(C.c_double))
        p.cheb_n, p.double_angle = len(c), double_angle
        p.cheb_lo, p.cheb_hi, p.const_scale = lo, hi, const_scale
        p.prescale = prescale
        p._coeffs = c
        return p


class ServerConfig(C.Structure):
    _fields_ = [("max_batch", C.c_uint32), ("max_inflight_batches", C.c_uint32), ("mem_budget_bytes", C.c_uint64)]


class ServerStats(C.Structure):
    _fields_ = [("completed", C.c_uint64), ("batches", C.c_uint64), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("mean_ms", C.c_double), ("max_ms", C.c_double), ("ops_per_s", C.c_double),
                ("mean_batch", C.c_double)]


class Server:
    """Continuous-batching request server over one context, or over several (rings) with one admission queue and
    one memory budget (the C server's worker thread owns the contexts)."""

    def __init__(self, ctx, max_batch: int = 64, max_inflight: int = 2, mem_budget: int = 16 << 30):
        ctxs = list(ctx) if isinstance(ctx, (list, tuple)) else [ctx]
        self.ctx = ctxs[0]
        self.ctxs = ctxs
        cfg = ServerConfig(max_batch, max_inflight, mem_budget)
        h = C.c_void_p()
        arr = (C.c_void_p * len(ctxs))(*[c._h for c in ctxs])
        _check(lib().fides_server_create_multi(arr, len(ctxs), C.byref(cfg), C.byref(h)))
        self._h = h

    def set_bootstrap_plan(self, plan: "BootstrapPlan"):
        _check(lib().fides_server_set_bootstrap_plan(self._h, C.byref(plan)))

    def submit(self, code: int, a: int, b: int = 0, index: int = 0, ring: int = 0) -> int:
        op = Op(code, a, b, index, 0)
        t = C.c_uint64()
        _check(lib().fides_server_submit_to(self._h, ring, C.byref(op), C.byref(t)))
        return t.value

    def wait(self, ticket: int):
        out = C.c_uint32()
        lat = C.c_double()
        _check(lib().fides_server_wait(self._h, ticket, C.byref(out), C.byref(lat)))
        return out.value, lat.value

    def release(self, ticket: int):
        _check(lib().fides_server_release(self._h, ticket))

    def stats(self) -> dict:
        st = ServerStats()
        _check(lib().fides_server_stats_get(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def reset_stats(self):
        _check(lib().fides_server_reset_stats(self._h))

    def close(self):
        if getattr(self, "_h", None):
            lib().fides_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
