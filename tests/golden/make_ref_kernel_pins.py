"""Writes tests/golden/ref_kernel_pins.json: outputs of the reference's own GPU kernels on seeded inputs.

Runs on a GPU host (python tests/golden/make_ref_kernel_pins.py [out.json]) with oracle/_ref/ref_kernels.cubin,
which oracle/build_ref.sh compiles from the reference's src/CKKS/Conv.cu and src/NTT.cu; the kernels are launched
by oracle/ref_kernels/harness.py exactly as the reference's LimbPartition launches them.  For two parameter sets at
N = 2^12 (the 60 + 5x40-bit basis with 3 special primes and dnum 2; the 60 + 29x50-bit basis with 10 special primes
and dnum 3) it records, per case, a SHA-256 of the output residues and a few leading residues:
  ntt / intt      the reference's NTT_ / INTT_ pair on one limb of every prime;
  modup/t         INTT_ of each digit, DecompAndModUpConv, NTT_ of every converted tower (LimbPartition::modup),
                  laid out [digit][t + K][N] with the digit's own towers copied (the oracle's orc_modup layout);
  moddown/t       INTT_ of the K special rows, ModDown2, NTT_ in NTT_MODDOWN mode (LimbPartition::moddown);
  rescale/t       INTT_ of the top tower, NTT_ in NTT_RESCALE mode (LimbPartition::rescale), on both polys;
  ksinner/t       fusedDotKSK_2_ on seeded digits and a seeded key, laid out [b half, a half][t + K][N] (the oracle's
                  orc_ks_inner order: sum_d D_d b_d, then sum_d D_d a_d);
  tensor/t        binomialMult_ on two seeded t-tower ciphertexts: (c0 d0, c0 d1 + c1 d0, c1 d1).
tests/test_ref_kernel_pins.py recomputes every case with the oracle on the same inputs and compares.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

LOGN = 12
N = 1 << LOGN
PARAM_SETS = {
    "q6_p3_d2": dict(q=[60] + [40] * 5, p=[60] * 3, dnum=2, levels=[1, 2, 3, 4, 5, 6]),
    "q30_p10_d3": dict(q=[60] + [50] * 29, p=[60] * 10, dnum=3, levels=[1, 2, 9, 10, 11, 17, 20, 21, 29, 30]),
}


def splitmix_residues(seed: int, moduli, n: int = N) -> np.ndarray:
    """Deterministic residues [len(moduli)][n]: SplitMix64 stream reduced mod each prime (the same on every host)."""
    out = np.empty((len(moduli), n), dtype=np.uint64)
    with np.errstate(over="ignore"):
        for r, q in enumerate(moduli):
            x = (np.arange(n, dtype=np.uint64) + np.uint64((seed * 1000003 + r) * n)) * np.uint64(0x9E3779B97F4A7C15)
            x = x + np.uint64(0x9E3779B97F4A7C15)
            x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
            x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
            x = x ^ (x >> np.uint64(31))
            out[r] = x % np.uint64(q)
    return out


def digest(a: np.ndarray) -> dict:
    a = np.ascontiguousarray(a, dtype=np.uint64).reshape(-1, N)
    return {"sha256": hashlib.sha256(a.astype("<u8").tobytes()).hexdigest(),
            "head": [[int(v) for v in a[r, :4]] for r in (0, len(a) - 1)]}


def moduli_and_roots(spec):
    import oracle as O
    mods = O.make_moduli(LOGN, spec["q"], spec["p"])
    return mods, [O.root_of_unity(m, 2 * N) for m in mods]


def run_reference(name: str, spec) -> dict:
    import torch

    from oracle.ref_kernels.harness import NTT_MODDOWN, NTT_RESCALE, RefKernels
    mods, roots = moduli_and_roots(spec)
    L, K = len(spec["q"]), len(spec["p"])
    R = RefKernels(LOGN, mods, roots, L, K, spec["dnum"])
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).cuda()  # noqa: E731
    host = lambda t: t.cpu().numpy().view(np.uint64)  # noqa: E731
    keep = []

    def ntt_rows(rows, ids, inverse):
        """rows: list of device limbs, ids: their prime ids (< L: Q tower, >= L: special)."""
        for r, j in zip(rows, ids):
            aux = [torch.empty_like(r)]
            first = j if j < L else R.special_base + (j - L)
            keep.append((R.intt if inverse else R.ntt)([r], first, aux))
            keep.append(aux)

    res = {"moduli": [int(m) for m in mods], "roots": [int(r) for r in roots]}
    # NTT and INTT of one limb per prime
    x = splitmix_residues(1, mods)
    limbs = [dev(x[j]) for j in range(L + K)]
    ntt_rows(limbs, range(L + K), False)
    torch.cuda.synchronize()
    res["ntt"] = digest(np.stack([host(t) for t in limbs]))
    y = splitmix_residues(2, mods)
    limbs = [dev(y[j]) for j in range(L + K)]
    ntt_rows(limbs, range(L + K), True)
    torch.cuda.synchronize()
    res["intt"] = digest(np.stack([host(t) for t in limbs]))

    alpha = (L + spec["dnum"] - 1) // spec["dnum"]
    key = pin_key(mods, L, K, spec["dnum"])
    for t in spec["levels"]:
        # ModUp of a t-tower polynomial (evaluation form)
        a = splitmix_residues(100 + t, mods[:t])
        beta = (t + alpha - 1) // alpha
        D = np.zeros((beta, t + K, N), dtype=np.uint64)
        for d in range(beta):
            own = list(range(d * alpha, min((d + 1) * alpha, t)))
            coeff = [torch.empty(N, dtype=torch.int64, device="cuda") for _ in own]
            src = [dev(a[i]) for i in own]
            aux = [torch.empty_like(c) for c in coeff]
            keep.append(R.intt(src, own[0], aux, dst=coeff))
            keep += [src, aux]
            tg = R.targets(t, d)
            out = [torch.empty(N, dtype=torch.int64, device="cuda") for _ in tg]
            keep.append(R.modup_conv(coeff, t, d, out))
            keep += [coeff]
            ntt_rows(out, tg, False)
            torch.cuda.synchronize()
            for i in own:
                D[d, i] = a[i]
            for j, o in zip(tg, out):
                D[d, j if j < L else t + (j - L)] = host(o)
        res[f"modup/{t}"] = digest(D)

        # ModDown of one extended polynomial [t + K] (evaluation form)
        xq = splitmix_residues(200 + t, mods[:t])
        xp = splitmix_residues(300 + t, mods[L:])
        sp = [dev(xp[k]) for k in range(K)]
        ntt_rows(sp, range(L, L + K), True)  # special rows to coefficient form
        conv = [torch.empty(N, dtype=torch.int64, device="cuda") for _ in range(t)]
        keep.append(R.moddown_conv(sp, conv))
        qrows = [dev(xq[j]) for j in range(t)]
        aux = [torch.empty_like(c) for c in conv]
        keep.append(R.ntt(qrows, 0, aux, mode=NTT_MODDOWN, src=conv))
        keep += [sp, conv, aux]
        torch.cuda.synchronize()
        res[f"moddown/{t}"] = digest(np.stack([host(r) for r in qrows]))

        # Rescale of a two-poly ciphertext with t >= 2 towers
        if t >= 2:
            ct = splitmix_residues(400 + t, mods[:t] * 2).reshape(2, t, N)
            outp = []
            for poly in range(2):
                rows = [dev(ct[poly, j]) for j in range(t)]
                top = rows[t - 1]
                taux = [torch.empty_like(top)]
                keep.append(R.intt([top], t - 1, taux))
                aux = [torch.empty_like(r) for r in rows[:t - 1]]
                keep.append(R.ntt(rows[:t - 1], 0, aux, mode=NTT_RESCALE, src=[top], rescale_prime=t - 1))
                keep += [rows, taux, aux]
                torch.cuda.synchronize()
                outp.append(np.stack([host(r) for r in rows[:t - 1]]))
            res[f"rescale/{t}"] = digest(np.stack(outp))

        # key inner product: digits in the oracle's layout, handed to the kernel as the reference's lists
        c1, D = inner_inputs(t, mods, L, K, alpha)
        dec_lists = R._digits()[0]
        c1_dev = [dev(c1[j]) for j in range(t)]
        key_a = [[dev(key[0, d, j]) for j in range(L + K)] for d in range(spec["dnum"])]
        key_b = [[dev(key[1, d, j]) for j in range(L + K)] for d in range(spec["dnum"])]
        zero = torch.zeros(N, dtype=torch.int64, device="cuda")
        digit_limbs = []
        for d in range(beta):
            row = lambda j: j if j < L else t + (j - L)  # noqa: E731
            digit_limbs.append([dev(D[d, row(j)]) if (j < t or j >= L) and j not in dec_lists[d] else zero
                                for j in R.digit_list(d)])
        outs = [[torch.empty(N, dtype=torch.int64, device="cuda") for _ in range(n)] for n in (t, K, t, K)]
        keep.append(R.ks_dot(c1_dev, digit_limbs, key_a, key_b, t, *outs))
        keep += [c1_dev, key_a, key_b, digit_limbs, outs]
        torch.cuda.synchronize()
        a_half = np.stack([host(x) for x in outs[0] + outs[1]])
        b_half = np.stack([host(x) for x in outs[2] + outs[3]])
        res[f"ksinner/{t}"] = digest(np.stack([b_half, a_half]))

        # tensor product of two t-tower ciphertexts
        x, y = tensor_inputs(t, mods)
        c0, c1t, d0, d1 = ([dev(v[j]) for j in range(t)] for v in (x[0], x[1], y[0], y[1]))
        c2 = [torch.empty(N, dtype=torch.int64, device="cuda") for _ in range(t)]
        keep.append(R.tensor(c0, c1t, c2, d0, d1))
        keep += [c0, c1t, c2, d0, d1]
        torch.cuda.synchronize()
        res[f"tensor/{t}"] = digest(np.stack([np.stack([host(r) for r in v]) for v in (c0, c1t, c2)]))
    torch.cuda.synchronize()
    return res


def pin_key(mods, L, K, dnum):
    """A seeded key of the real shape [2][dnum][L + K][N]."""
    return splitmix_residues(500, list(mods) * (2 * dnum)).reshape(2, dnum, L + K, N)


def inner_inputs(t, mods, L, K, alpha):
    """c1 (t towers) and digits in the oracle's layout [beta][t + K][N] whose own-tower rows are c1's."""
    beta = (t + alpha - 1) // alpha
    c1 = splitmix_residues(600 + t, mods[:t])
    D = np.stack([splitmix_residues(700 + 10 * t + d, list(mods[:t]) + list(mods[L:])) for d in range(beta)])
    for d in range(beta):
        for j in range(d * alpha, min((d + 1) * alpha, t)):
            D[d, j] = c1[j]
    return c1, D


def tensor_inputs(t, mods):
    x = splitmix_residues(800 + t, list(mods[:t]) * 2).reshape(2, t, N)
    y = splitmix_residues(900 + t, list(mods[:t]) * 2).reshape(2, t, N)
    return x, y


def main():
    out = sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                              "ref_kernel_pins.json")
    data = {"logN": LOGN, "sets": {}}
    for name, spec in PARAM_SETS.items():
        data["sets"][name] = run_reference(name, spec)
        print(f"{name}: {len(data['sets'][name]) - 2} cases", flush=True)
    json.dump(data, open(out, "w"), indent=1)
    print(out)


if __name__ == "__main__":
    main()
