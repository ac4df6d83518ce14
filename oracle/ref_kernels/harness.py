"""Runs the reference's own GPU kernels — TEST INFRASTRUCTURE ONLY.

Loads oracle/_ref/ref_kernels.cubin (the reference's src/CKKS/Conv.cu and src/NTT.cu compiled from its sources by
oracle/build_ref.sh) through the CUDA driver API and launches, with the reference's launch shapes:
  * NTT_ / INTT_ (two passes each, src/NTT.cu:236-327, 697-769), shapes of LimbPartition::ApplyNTT / ApplyINTT
    (src/CKKS/LimbPartition.cu:318-421), in plain, NTT_RESCALE (the rescale of LimbPartition::rescale,
    :575-652) and NTT_MODDOWN (the ModDown epilogue of LimbPartition::moddown, :1913-1985) modes;
  * DecompAndModUpConv (src/CKKS/Conv.cu:258-407), launched as LimbPartition::modup does (:766-772);
  * ModDown2 (src/CKKS/Conv.cu:26-133), launched as LimbPartition::moddown does (:1948-1954);
  * fusedDotKSK_2_ (src/CKKS/ElemenwiseBatchKernels.cu:202-275), the key inner product, with the digit / key table
    LimbPartition::dotKSKfusedMGPU builds (src/CKKS/LimbPartitionMGPU.cu:404-446);
  * binomialMult_ (src/CKKS/ElemenwiseBatchKernels.cu:1363-1395), the tensor product of a multiplication, launched
    as LimbPartition::binomialMult does (src/CKKS/LimbPartition.cu:2600-2604).
The constant block `FIDESlib::constants` and the table block `Global::Globals` are filled the way the
reference's SetupConstants does (src/ConstantsGPU.cu:125-697), from the same primes and roots the engine uses and
with OpenFHE's CRT tables (PartQlHatInvModq, PartQlHatModp, PHatInvModp, PHatModq, PInvModq,
QlQlInvModqlDivqlModq) computed from their definitions; byte offsets come from oracle/_ref/ref_layout.json.

Used by tests/golden/make_ref_kernel_pins.py (fixtures that pin the oracle) and oracle/ref_kernels/compare.py
(same-GPU timing of the reference's kernels beside the engine's).  Never imported by the engine.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import struct

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(os.path.dirname(HERE), "_ref")
CUBIN = os.path.join(REF, "ref_kernels.cubin")
NAMES = os.path.join(REF, "ref_kernels.json")
LAYOUT = os.path.join(REF, "ref_layout.json")

ALGO_SHOUP = 3
NTT_NONE, NTT_RESCALE, NTT_MULTPT, NTT_MODDOWN = 0, 1, 2, 3
M = 4  # residues per thread and pass in the reference's NTT kernels


def available() -> bool:
    return all(os.path.exists(p) for p in (CUBIN, NAMES, LAYOUT))


# ---------------------------------------------------------------------------------------------------------------
# host-side table math (SetupConstants' formulas)

def bit_reverse(x: int, bits: int) -> int:
    return int(format(x, f"0{bits}b")[::-1], 2) if bits else 0


def shoup(v: int, p: int) -> int:
    """shoup_precomp (src/ConstantsGPU.cu:70-73): floor((v << 1) * 2^63 / p), the shift taken modulo 2^64."""
    return (((v << 1) & (2 ** 64 - 1)) * (1 << 63)) // p


def barrett_mu(p: int, bits: int) -> int:
    """mu_new with VERSION == NEIL (src/ConstantsGPU.cu:31-34)."""
    return ((1 << (2 * bits + 1)) // p) & (2 ** 64 - 1)


def _powers(w: int, n: int, p: int) -> list[int]:
    out = [1] * n
    for j in range(1, n):
        out[j] = out[j - 1] * w % p
    return out


_BR = {}


def _brev_table(bits: int) -> list[int]:
    if bits not in _BR:
        _BR[bits] = [bit_reverse(j, bits) for j in range(1 << bits)]
    return _BR[bits]


def psi_tables(p: int, psi: int, logN: int):
    """Per-prime twiddle tables of SetupConstants (src/ConstantsGPU.cu:221-315)."""
    N = 1 << logN
    ipsi = pow(psi, -1, p)
    n_inv = pow(N, -1, p)
    psi_no = _powers(psi, 2 * N, p)
    ipsi_no = _powers(ipsi, 2 * N, p)
    br = _brev_table(logN)
    tab_psi = [psi_no[b] for b in br]
    tab_ipsi = [ipsi_no[b] for b in br]
    aw = (logN + 1) // 2
    W = 1 << aw
    bw = _brev_table(aw)
    mid = [0] * N
    imid = [0] * N
    for j in range(N // W):
        for k in range(W):
            e = j * bw[k]
            mid[j * W + k] = psi_no[e]
            imid[j * W + k] = ipsi_no[e] * n_inv % p
    ipsi_no = [x * n_inv % p for x in ipsi_no]
    return dict(psi=tab_psi, inv_psi=tab_ipsi, psi_no=psi_no, inv_psi_no=ipsi_no, psi_middle_scale=mid,
                inv_psi_middle_scale=imid, psi_shoup=[shoup(x, p) for x in tab_psi],
                inv_psi_shoup=[shoup(x, p) for x in tab_ipsi])


def prod_mod(vals, m):
    r = 1 % m
    for v in vals:
        r = r * (v % m) % m
    return r


# ---------------------------------------------------------------------------------------------------------------
# CUDA driver API (the context is torch's primary context)

class _Driver:
    def __init__(self):
        import torch
        torch.zeros(1, device="cuda")  # creates and makes current the primary context
        self.cu = C.CDLL("libcuda.so.1")
        cu = self.cu
        cu.cuModuleLoad.argtypes = [C.POINTER(C.c_void_p), C.c_char_p]
        cu.cuModuleGetFunction.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_char_p]
        cu.cuModuleGetGlobal_v2.argtypes = [C.POINTER(C.c_uint64), C.POINTER(C.c_size_t), C.c_void_p, C.c_char_p]
        cu.cuMemcpyHtoD_v2.argtypes = [C.c_uint64, C.c_void_p, C.c_size_t]
        cu.cuFuncSetAttribute.argtypes = [C.c_void_p, C.c_int, C.c_int]
        cu.cuLaunchKernel.argtypes = [C.c_void_p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint,
                                      C.c_void_p, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]
        cu.cuGetErrorString.argtypes = [C.c_int, C.POINTER(C.c_char_p)]

    def check(self, rc, what):
        if rc != 0:
            s = C.c_char_p()
            self.cu.cuGetErrorString(rc, C.byref(s))
            raise RuntimeError(f"{what}: CUDA driver error {rc} ({s.value.decode() if s.value else '?'})")


class RefKernels:
    """The reference's kernels over one parameter set: moduli q_0..q_{L-1}, p_0..p_{K-1} (< 2^60), their primitive
    2N-th roots, and dnum digits of alpha = ceil(L / dnum) towers (OpenFHE's partition)."""

    def __init__(self, logN: int, moduli, roots, L: int, K: int, dnum: int):
        import torch
        assert available(), "oracle/_ref/ref_kernels.cubin missing (oracle/build_ref.sh builds it)"
        assert L + K <= 64 and dnum <= 8 and 10 <= logN <= 16
        self.torch = torch
        self.logN, self.N = logN, 1 << logN
        self.L, self.K, self.dnum = L, K, dnum
        self.alpha = (L + dnum - 1) // dnum
        self.mod = [int(x) for x in moduli]
        self.roots = [int(x) for x in roots]
        self.lay = json.load(open(LAYOUT))
        self.names = json.load(open(NAMES))
        self.d = _Driver()
        self.mod_h = C.c_void_p()
        self.d.check(self.d.cu.cuModuleLoad(C.byref(self.mod_h), CUBIN.encode()), "cuModuleLoad")
        self._fn = {}
        self._keep = []  # device buffers referenced from the table block
        # first_prime argument of ntt / intt for the special primes: the index of primeid_special_partition within
        # the flattened prime-id lists (the reference's SPECIAL(id, 0))
        self.special_base = (self.lay["Constants.primeid_special_partition"] -
                             self.lay["Constants.primeid_partition"]) // 4
        self._build_constants()
        self._build_globals()

    # --- constant and table blocks -----------------------------------------------------------------------------
    def _digits(self):
        """DECOMPmeta / DIGITmeta of one GPU: digit d's towers, and its targets (the special primes first, then the
        Q towers outside the digit, as LimbPartition's DIGITlimb lists them)."""
        L, K, a = self.L, self.K, self.alpha
        dec = [list(range(d * a, min((d + 1) * a, L))) for d in range(self.dnum)]
        dig = [list(range(L, L + K)) + [i for i in range(L) if not (d * a <= i < (d + 1) * a)]
               for d in range(self.dnum)]
        return dec, dig

    def _build_constants(self):
        lay, L, K, N = self.lay, self.L, self.K, self.N
        b = bytearray(lay["sizeof.Constants"])
        P = lambda f, fmt, *v: struct.pack_into(fmt, b, lay["Constants." + f], *v)  # noqa: E731

        def arr(f, fmt, vals, stride):
            base = lay["Constants." + f]
            for i, v in enumerate(vals):
                struct.pack_into(fmt, b, base + i * stride, v)

        P("N", "<i", N)
        P("L", "<i", L)
        P("K", "<i", K)
        P("logN", "<i", self.logN)
        P("type", "<Q", (1 << (L + K)) - 1)  # every prime > 30 bits: U64 limbs
        bits = [m.bit_length() for m in self.mod]
        arr("primes", "<Q", self.mod, 8)
        arr("prime_better_barret_mu", "<Q", [barrett_mu(m, bt) for m, bt in zip(self.mod, bits)], 8)
        arr("prime_bits", "<I", bits, 4)
        arr("N_shoup", "<Q", [shoup(N, m) for m in self.mod], 8)
        # SetupConstants writes one_shoup[i] for the special primes at index i (not L + i): kept as it does.
        one = [shoup(1, m) for m in self.mod[:L]] + [0] * K
        for i in range(K):
            one[i] = shoup(1, self.mod[i])
        arr("one_shoup", "<Q", one, 8)
        ninv = [pow(N, -1, m) for m in self.mod]
        arr("N_inv", "<Q", ninv, 8)
        arr("N_inv_shoup", "<Q", [shoup(x, m) for x, m in zip(ninv, self.mod)], 8)
        iroot = [pow(r, -1, m) for r, m in zip(self.roots, self.mod)]
        arr("root", "<Q", self.roots, 8)
        arr("root_shoup", "<Q", [shoup(r, m) for r, m in zip(self.roots, self.mod)], 8)
        arr("inv_root", "<Q", iroot, 8)
        arr("inv_root_shoup", "<Q", [shoup(r, m) for r, m in zip(iroot, self.mod)], 8)
        P("dnum", "<i", self.dnum)
        Pprod = 1
        for p in self.mod[L:]:
            Pprod *= p
        pinv = [pow(Pprod % q, -1, q) for q in self.mod[:L]]  # PInvModq
        arr("P_inv", "<Q", pinv, 8)
        arr("P_inv_shoup", "<Q", [shoup(x, q) for x, q in zip(pinv, self.mod[:L])], 8)
        arr("P", "<Q", [Pprod % q for q in self.mod[:L]], 8)
        arr("P_shoup", "<Q", [shoup(Pprod % q, q) for q in self.mod[:L]], 8)
        dec, dig = self._digits()
        MAXP = lay["MAXP"]
        digit_of = {}
        for d, ids in enumerate(dec):
            for i in ids:
                digit_of[i] = d
        for j in range(L, L + K):
            digit_of[j] = -1  # LimbRecord::digit default for the special limbs
        arr("primeid_digit", "<i", [digit_of.get(i, 0) for i in range(L + K)], 4)
        arr("primeid_partition", "<i", list(range(L)), 4)  # partition of GPU 0: every Q tower
        arr("primeid_special_partition", "<i", list(range(L, L + K)), 4)
        for d in range(self.dnum):
            # the k loop of SetupConstants (:645-672): counts per level; the id lists end as the k = L-1 lists
            for k in range(L):
                nf = sum(1 for i in dec[d] if i <= k)
                nt = sum(1 for i in dig[d] if i <= k or i >= L)
                struct.pack_into("<i", b, lay["Constants.num_primeid_digit_from"] + 4 * (d * MAXP + k), nf)
                struct.pack_into("<i", b, lay["Constants.num_primeid_digit_to"] + 4 * (d * MAXP + k), nt)
            for n_, i in enumerate(dec[d]):
                struct.pack_into("<i", b, lay["Constants.primeid_digit_from"] + 4 * (d * MAXP + n_), i)
                struct.pack_into("<i", b, lay["Constants.pos_in_digit"] + 4 * (d * MAXP + i), n_)
            for n_, i in enumerate(dig[d]):
                struct.pack_into("<i", b, lay["Constants.primeid_digit_to"] + 4 * (d * MAXP + n_), i)
                struct.pack_into("<i", b, lay["Constants.pos_in_digit"] + 4 * (d * MAXP + i), n_)
        self.constants_bytes = bytes(b)
        ptr, size = C.c_uint64(), C.c_size_t()
        self.d.check(self.d.cu.cuModuleGetGlobal_v2(C.byref(ptr), C.byref(size), self.mod_h, b"_ZN8FIDESlib9constantsE"),
                     "constants symbol")
        assert size.value == len(b), (size.value, len(b))
        host = (C.c_char * len(b)).from_buffer_copy(b)
        self.d.check(self.d.cu.cuMemcpyHtoD_v2(ptr.value, C.cast(host, C.c_void_p), len(b)), "constants upload")

    def _dev(self, vals):
        t = self.torch.tensor(np.array(vals, dtype=np.uint64).view(np.int64), device="cuda")
        self._keep.append(t)
        return t.data_ptr()

    def _build_globals(self):
        lay, L, K, N = self.lay, self.L, self.K, self.N
        MAXP = lay["MAXP"]
        g = np.zeros(lay["sizeof.Globals"] // 8, dtype=np.uint64)

        def put(f, idx, v):
            g[lay["G." + f] // 8 + idx] = v

        for i, (p, r) in enumerate(zip(self.mod, self.roots)):
            t = psi_tables(p, r, self.logN)
            for f in ("psi", "inv_psi", "psi_middle_scale", "inv_psi_middle_scale", "psi_no", "inv_psi_no",
                      "psi_shoup", "inv_psi_shoup"):
                put(f, i, self._dev(t[f]))
        for i in range(L + K):
            for j in range(L + K):
                if i != j:
                    put("q_inv", MAXP * i + j, pow(self.mod[i] % self.mod[j], -1, self.mod[j]))
        # QlQlInvModqlDivqlModq[l][i], i < l: (Q_{l-1} [Q_{l-1}^-1]_{q_l} - 1) / q_l mod q_i = -q_l^-1 mod q_i
        for lv in range(1, L):
            for i in range(lv):
                put("QlQlInvModqlDivqlModq", MAXP * lv + i, (-pow(self.mod[lv], -1, self.mod[i])) % self.mod[i])
        sp = self.mod[L:]
        for k in range(K):
            phat_k = [x for kk, x in enumerate(sp) if kk != k]
            w = pow(prod_mod(phat_k, sp[k]), -1, sp[k])  # PHatInvModp
            put("ModDown_pre_scale", L + k, w)
            put("ModDown_pre_scale_shoup", L + k, shoup(w, sp[k]))
            for j in range(L):
                v = prod_mod(phat_k, self.mod[j])  # PHatModq
                put("ModDown_matrix", MAXP * k + j, v)
                put("ModDown_matrix_shoup", MAXP * k + j, shoup(v, self.mod[j]))
        dec, dig = self._digits()
        for d in range(self.dnum):
            for s in range(1, len(dec[d]) + 1):  # partial digit of s towers (the digit at lower levels)
                part = dec[d][:s]
                for i in part:
                    others = [self.mod[x] for x in part if x != i]
                    w = pow(prod_mod(others, self.mod[i]), -1, self.mod[i])  # PartQlHatInvModq
                    put("DecompAndModUp_pre_scale", MAXP * MAXP * d + MAXP * (s - 1) + i, w)
                    put("DecompAndModUp_pre_scale_shoup", MAXP * MAXP * d + MAXP * (s - 1) + i, shoup(w, self.mod[i]))
        for n in range(1, L + 1):  # ciphertexts of n towers: PartQlHatModp[n-1] (the digit cut at n towers)
            for d in range(self.dnum):
                part = [i for i in dec[d] if i < n]
                for i in part:
                    others = [self.mod[x] for x in part if x != i]
                    for j in dig[d]:
                        if j < n or j >= L:
                            v = prod_mod(others, self.mod[j])
                            put("DecompAndModUp_matrix", MAXP * MAXP * (n - 1) + MAXP * i + j, v)
                            put("DecompAndModUp_matrix_shoup", MAXP * MAXP * (n - 1) + MAXP * i + j,
                                shoup(v, self.mod[j]))
        t = self.torch.tensor(g.view(np.int64), device="cuda")
        self._keep.append(t)
        self.globals_ptr = t.data_ptr()

    # --- launches --------------------------------------------------------------------------------------------------
    def fn(self, demangled: str):
        if demangled not in self._fn:
            h = C.c_void_p()
            self.d.check(self.d.cu.cuModuleGetFunction(C.byref(h), self.mod_h, self.names[demangled].encode()),
                         demangled)
            self._fn[demangled] = h
        return self._fn[demangled]

    def ptrs(self, tensors):
        """Device array of the data pointers of `tensors` (the reference's void** limb lists)."""
        t = self.torch.tensor([x.data_ptr() for x in tensors], dtype=self.torch.int64, device="cuda")
        return t

    def launch(self, f, grid, block, smem, args, stream=0):
        cargs = []
        for kind, v in args:
            cargs.append(C.c_int(v) if kind == "i" else C.c_void_p(v))
        arr = (C.c_void_p * len(cargs))(*[C.cast(C.pointer(a), C.c_void_p) for a in cargs])
        if smem > 48 * 1024:
            self.d.check(self.d.cu.cuFuncSetAttribute(f, 8, smem), "max dynamic shared memory")
        self.d.check(self.d.cu.cuLaunchKernel(f, grid[0], grid[1], 1, block[0], block[1], 1, smem, C.c_void_p(stream),
                                              arr, None), "cuLaunchKernel")

    @staticmethod
    def _ntt_name(second, mode):
        return (f"void FIDESlib::NTT_<{'true' if second else 'false'}, (FIDESlib::ALGO)3, (FIDESlib::NTT_MODE){mode}>"
                "(FIDESlib::Global::Globals const*, void**, int, void**, void**, int, void**, void**)")

    @staticmethod
    def _intt_name(second):
        return (f"void FIDESlib::INTT_<{'true' if second else 'false'}, (FIDESlib::ALGO)3, (FIDESlib::INTT_MODE)0>"
                "(FIDESlib::Global::Globals const*, void**, int, void**, void**, void**, void**, void**, void**, "
                "void**, void**)")

    def ntt(self, limbs, first_prime: int, aux, stream=0, mode=NTT_NONE, src=None, rescale_prime=0, dst=None):
        """Forward NTT of len(limbs) device limbs (uint64 [N] each, natural coefficient order) whose primes are
        first_prime + k, in place, through aux (same count): LimbPartition::ApplyNTT's two launches.  mode
        NTT_RESCALE: limbs are the kept towers, src[0] the top tower in coefficient form (rescale_prime its
        prime); NTT_MODDOWN: src[k] is the converted tower, limbs[k] the tower it is subtracted from."""
        lp, ap = self.ptrs(limbs), self.ptrs(aux)
        first_in = self.ptrs(src) if mode in (NTT_RESCALE, NTT_MODDOWN) else lp
        out = self.ptrs(dst) if dst is not None else lp
        self.ntt_launch(first_in, ap, out, len(limbs), first_prime, mode, rescale_prime, stream)
        return (lp, ap, first_in, out)  # keep the pointer arrays alive until the launches have run

    def ntt_launch(self, first_in, aux, out, n: int, first_prime: int, mode=NTT_NONE, rescale_prime=0, stream=0):
        """The two NTT_ launches over prebuilt device pointer arrays (each of n limbs)."""
        logN = self.logN
        if mode == NTT_RESCALE:  # LimbPartition::rescale's shapes (:597-633)
            b1, b2 = 1 << (logN // 2 - 1), 1 << ((logN + 1) // 2 - 1)
        else:
            b1, b2 = 1 << ((logN + 1) // 2 - 1), 1 << (logN // 2 - 1)
        s1, s2 = 8 * b1 * (2 * M + 2), 8 * b2 * (2 * M + 2)
        self.launch(self.fn(self._ntt_name(False, mode)), (self.N // (b1 * M * 2), n), (b1, 1), s1,
                    [("p", self.globals_ptr), ("p", first_in.data_ptr()), ("i", first_prime), ("p", aux.data_ptr()),
                     ("p", 0), ("i", rescale_prime), ("p", 0), ("p", 0)], stream)
        self.launch(self.fn(self._ntt_name(True, mode)), (self.N // (b2 * M * 2), n), (b2, 1), s2,
                    [("p", self.globals_ptr), ("p", aux.data_ptr()), ("i", first_prime), ("p", out.data_ptr()),
                     ("p", 0), ("i", rescale_prime), ("p", 0), ("p", 0)], stream)

    def intt(self, limbs, first_prime: int, aux, stream=0, dst=None):
        """Inverse NTT (evaluation -> coefficient form, N^-1 included) of device limbs, LimbPartition::ApplyINTT."""
        lp, ap = self.ptrs(limbs), self.ptrs(aux)
        out = self.ptrs(dst) if dst is not None else lp
        self.intt_launch(lp, ap, out, len(limbs), first_prime, stream)
        return (lp, ap, out)

    def intt_launch(self, src, aux, out, n: int, first_prime: int, stream=0):
        """The two INTT_ launches over prebuilt device pointer arrays (each of n limbs)."""
        logN = self.logN
        b1, b2 = 1 << (logN // 2 - 1), 1 << ((logN + 1) // 2 - 1)
        s1, s2 = 8 * b1 * (2 * M + 2), 8 * b2 * (2 * M + 2)
        z = [("p", 0)] * 7
        self.launch(self.fn(self._intt_name(False)), (self.N // (b1 * M * 2), n), (b1, 1), s1,
                    [("p", self.globals_ptr), ("p", src.data_ptr()), ("i", first_prime), ("p", aux.data_ptr())] + z,
                    stream)
        self.launch(self.fn(self._intt_name(True)), (self.N // (b2 * M * 2), n), (b2, 1), s2,
                    [("p", self.globals_ptr), ("p", aux.data_ptr()), ("i", first_prime), ("p", out.data_ptr())] + z,
                    stream)

    def modup_conv(self, digit_in, t: int, d: int, out, stream=0):
        """DecompAndModUpConv for digit d of a ciphertext with t towers: digit_in = the digit's towers below t
        (coefficient form), out = one limb per target of the digit at t towers (the special primes, then the Q
        towers outside the digit below t), in that order."""
        assert len(digit_in) == sum(1 for i in self._digits()[0][d] if i < t)
        assert len(out) == len(self.targets(t, d))
        ip, op = self.ptrs(digit_in), self.ptrs(out)
        self.modup_conv_launch(ip, op, len(digit_in), t, d, stream)
        return (ip, op)

    def modup_conv_launch(self, ip, op, n_in: int, t: int, d: int, stream=0):
        self.launch(self.fn("void FIDESlib::CKKS::DecompAndModUpConv<(FIDESlib::ALGO)3>(void**, int, void**, int, "
                            "FIDESlib::Global::Globals const*)"), (self.N // 64, 1), (64, 2), 8 * n_in * 64,
                    [("p", ip.data_ptr()), ("i", t), ("p", op.data_ptr()), ("i", d), ("p", self.globals_ptr)], stream)

    def digit_base(self, d: int) -> int:
        """first_prime of ntt / intt for the target list of digit d (the reference's DIGIT(d, 0))."""
        return (self.lay["Constants.primeid_digit_to"] - self.lay["Constants.primeid_partition"]) // 4 + \
            d * self.lay["MAXP"]

    def targets(self, t: int, d: int):
        return [j for j in self._digits()[1][d] if j < t or j >= self.L]

    def moddown_conv(self, special_in, out, stream=0):
        """ModDown2: special_in = the K special towers (coefficient form), out = len(out) Q towers 0.. (coefficient
        form) receiving the converted values."""
        assert len(special_in) == self.K
        ip, op = self.ptrs(special_in), self.ptrs(out)
        self.moddown_conv_launch(ip, op, len(out), stream)
        return (ip, op)

    def moddown_conv_launch(self, ip, op, n_out: int, stream=0):
        self.launch(self.fn("void FIDESlib::CKKS::ModDown2<(FIDESlib::ALGO)3>(void**, int, void**, int, "
                            "FIDESlib::Global::Globals const*)"), (self.N // 64, 1), (64, 2), 8 * self.K * 64,
                    [("p", op.data_ptr()), ("i", n_out), ("p", ip.data_ptr()), ("i", 0), ("p", self.globals_ptr)],
                    stream)

    # --- key inner product and tensor product ------------------------------------------------------------------
    def digit_list(self, d: int):
        """Digit d's full target list (the special primes, then the Q towers outside the digit): DIGITlimb order."""
        return self._digits()[1][d]

    def ks_dot(self, c1, digit_limbs, key_a, key_b, t: int, out1, sout1, out2, sout2, stream=0):
        """fusedDotKSK_2_ for a ciphertext with t towers.  c1: its t limbs (the own-digit towers are read from here);
        digit_limbs[d]: digit d's ModUp output limbs in digit_list(d) order; key_a / key_b[d][j]: tower j of digit d
        of the key halves (all nq + np towers).  out1 / out2 (t Q rows) and sout1 / sout2 (np special rows) receive
        sum_d D_d a_d and sum_d D_d b_d."""
        dec, _ = self._digits()
        beta = (t + self.alpha - 1) // self.alpha
        own = {j: d for d, ids in enumerate(dec) for j in ids}
        tables = [None] * (6 * self.dnum)
        for d in range(beta):
            lst = self.digit_list(d)
            tables[d] = self.ptrs(digit_limbs[d])
            tables[self.dnum + d] = self.ptrs([key_a[d][j] for j in lst])
            tables[2 * self.dnum + d] = self.ptrs([key_b[d][j] for j in lst])
            tables[3 * self.dnum + d] = self.ptrs(c1)
            tables[4 * self.dnum + d] = self.ptrs([key_a[own[j]][j] for j in range(self.L)])
            tables[5 * self.dnum + d] = self.ptrs([key_b[own[j]][j] for j in range(self.L)])
        dummy = tables[0]
        tables = [x if x is not None else dummy for x in tables]
        top = self.torch.tensor([x.data_ptr() for x in tables], dtype=self.torch.int64, device="cuda")
        o1, s1, o2, s2 = self.ptrs(out1), self.ptrs(sout1), self.ptrs(out2), self.ptrs(sout2)
        self.launch(self.fn("FIDESlib::CKKS::fusedDotKSK_2_(void**, void**, void**, void**, void***, int, int, int, int)"),
                    (self.N // 128, self.K + t), (128, 1), 0,
                    [("p", o1.data_ptr()), ("p", s1.data_ptr()), ("p", o2.data_ptr()), ("p", s2.data_ptr()),
                     ("p", top.data_ptr()), ("i", beta), ("i", 0), ("i", self.K), ("i", 0)], stream)
        return (tables, top, o1, s1, o2, s2)

    def tensor(self, c0, c1, c2, d0, d1, stream=0):
        """binomialMult_ over len(c0) Q towers from tower 0, in place: c0 <- c0 d0, c1 <- c0 d1 + c1 d0, c2 <- c1 d1."""
        lists = [self.ptrs(x) for x in (c0, c1, c2, d0, d1)]
        self.launch(self.fn("FIDESlib::CKKS::binomialMult_(int, void**, void**, void**, void**, void**)"), (self.N // 128, len(c0)),
                    (128, 1), 0, [("i", 0)] + [("p", x.data_ptr()) for x in lists], stream)
        return lists
