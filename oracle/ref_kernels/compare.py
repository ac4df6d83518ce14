"""Same-GPU timing of the reference's own kernels beside the engine's — TEST INFRASTRUCTURE ONLY.

python oracle/ref_kernels/compare.py [out.json] on a GPU host (needs oracle/_ref/ref_kernels.cubin from
oracle/build_ref.sh and the engine library).  CUDA events on the default stream, 3 warm-up and 10 timed rounds, the
mean reported; inputs are seeded residues.  Stages, each run by both sides on identical data shapes:
  ntt / intt       config 2: 16 polynomials x 40 primes of 60 bits at N = 2^16 (640 limbs).  Reference: its two-pass
                   NTT_ / INTT_ with LimbPartition::ApplyNTT's shapes, one launch pair per polynomial (a launch
                   covers one polynomial's limbs, as in the reference).  Engine: fides_ntt_batch_device.
  modup            config 3 (N = 2^16, 60 + 29x50-bit Q, 10 special primes of 60 bits, dnum 3), 8 polynomials at
                   30 towers.  Reference: per digit INTT_ of its towers, DecompAndModUpConv, NTT_ of the 30
                   converted towers (LimbPartition::modup).  Engine: fides_fast_rotation_precompute (the same ModUp
                   plus a copy of c1), one call per ciphertext.
  moddown          config 3, 8 extended ciphertexts (2 polys each, 30 + 10 towers).  Reference: per poly INTT_ of the
                   special rows, ModDown2, NTT_ in NTT_MODDOWN mode (LimbPartition::moddown).  Engine:
                   fides_key_switch_down, one call per ciphertext.
The reference kernels here are the compiled reference sources as they are; only the launch loop is this script's.
"""
from __future__ import annotations

import json
import os
import statistics
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

LOGN = 16
N = 1 << LOGN


def timed(fn, stream, warm=3, reps=10):
    """Mean ms per call of fn, with CUDA events on `stream` (every launch of both sides goes to that stream)."""
    import torch
    torch.cuda.synchronize()  # inputs were made on the default stream
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(reps + 1)]
    ev[0].record(stream)
    for r in range(reps):
        fn()
        ev[r + 1].record(stream)
    torch.cuda.synchronize()
    return statistics.mean(ev[r].elapsed_time(ev[r + 1]) for r in range(reps))


def residues(mods, rows, seed):
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    m = torch.tensor([int(x) for x in mods], dtype=torch.int64, device="cuda")
    return torch.randint(0, 1 << 62, (rows, len(mods), N), dtype=torch.int64, device="cuda", generator=g) % \
        m.view(1, -1, 1)


def ntt_stage(out, st):
    import torch

    import fideslib_gb300 as F
    from bench import gen_primes_host
    from oracle.ref_kernels.harness import RefKernels
    mods = gen_primes_host(60, 41, 2 * N)
    ctx = F.CryptoContext(LOGN, mods, 1, 1)
    ctx.set_stream(st.cuda_stream)
    R = RefKernels(LOGN, mods, ctx.roots, 40, 1, 1)
    sp = st.cuda_stream
    data = residues(mods[:40], 16, 0x5EED0002)
    aux = torch.empty_like(data)
    lp = [R.ptrs([data[p, j] for j in range(40)]) for p in range(16)]
    ap = [R.ptrs([aux[p, j] for j in range(40)]) for p in range(16)]
    ptr = data.data_ptr()
    out["ntt_640_limbs_ms"] = {
        "reference_NTT_": timed(lambda: [R.ntt_launch(lp[p], ap[p], lp[p], 40, 0, stream=sp) for p in range(16)], st),
        "engine": timed(lambda: ctx.ntt_device(ptr, 16, 40, 0, False), st),
    }
    out["intt_640_limbs_ms"] = {
        "reference_INTT_": timed(lambda: [R.intt_launch(lp[p], ap[p], lp[p], 40, 0, stream=sp) for p in range(16)],
                                 st),
        "engine": timed(lambda: ctx.ntt_device(ptr, 16, 40, 0, True), st),
    }
    # the two sides agree on what they compute: engine forward NTT == reference forward NTT on the same limbs
    x = residues(mods[:40], 1, 7)
    y = x.clone()
    torch.cuda.synchronize()
    ctx.ntt_device(x.data_ptr(), 1, 40, 0, False)
    py, pa = R.ptrs([y[0, j] for j in range(40)]), R.ptrs([aux[0, j] for j in range(40)])
    R.ntt_launch(py, pa, py, 40, 0, stream=sp)
    torch.cuda.synchronize()
    out["ntt_outputs_identical"] = bool(torch.equal(x, y))
    ctx.close()


def keyswitch_stages(out, st):
    import torch

    import fideslib_gb300 as F
    from bench import moduli_cfg3
    from oracle.ref_kernels.harness import NTT_MODDOWN, RefKernels
    mods = moduli_cfg3()
    L, K, dnum, t, n = 30, 10, 3, 30, 8
    ctx = F.CryptoContext(LOGN, mods, K, dnum)
    ctx.set_stream(st.cuda_stream)
    R = RefKernels(LOGN, mods, ctx.roots, L, K, dnum)
    alpha = R.alpha
    sp = st.cuda_stream
    cts = residues(mods[:L], 2 * n, 0x5EED0003).view(n, 2, L, N)
    # --- ModUp of c1 ---
    coeff = torch.empty((n, L, N), dtype=torch.int64, device="cuda")
    conv = torch.empty((n, dnum, t, N), dtype=torch.int64, device="cuda")  # 30 targets per digit at t = 30
    aux = torch.empty((n, dnum, t, N), dtype=torch.int64, device="cuda")
    plans = []
    for c in range(n):
        for d in range(dnum):
            own = list(range(d * alpha, min((d + 1) * alpha, t)))
            src = R.ptrs([cts[c, 1, i] for i in own])
            cf = R.ptrs([coeff[c, i] for i in own])
            ax1 = R.ptrs([aux[c, d, k] for k in range(len(own))])
            tg = R.targets(t, d)
            cv = R.ptrs([conv[c, d, k] for k in range(len(tg))])
            ax2 = R.ptrs([aux[c, d, k] for k in range(len(tg))])
            plans.append((src, cf, ax1, cv, ax2, len(own), d, len(tg), own[0]))

    def ref_modup():
        for src, cf, ax1, cv, ax2, no, d, nt, f0 in plans:
            R.intt_launch(src, ax1, cf, no, f0, stream=sp)
            R.modup_conv_launch(cf, cv, no, t, d, stream=sp)
            R.ntt_launch(cv, ax2, cv, nt, R.digit_base(d), stream=sp)

    hs = [ctx.load_ciphertext_device(cts[c].data_ptr(), t) for c in range(n)]
    pres = []

    def eng_modup():
        for p in pres:
            ctx.precompute_free(p)
        pres.clear()
        for h in hs:
            pres.append(ctx.fast_rotation_precompute(h))

    out["modup_8x30_towers_ms"] = {"reference": timed(ref_modup, st), "engine": timed(eng_modup, st)}
    # --- ModDown of extended ciphertexts (2 polys x (30 + 10) towers) ---
    ext = torch.cat([cts, residues(mods[L:], 2 * n, 99).view(n, 2, K, N)], dim=2).contiguous()  # [n][2][40][N]
    sp_coeff = torch.empty((n, 2, K, N), dtype=torch.int64, device="cuda")
    mdc = torch.empty((n, 2, t, N), dtype=torch.int64, device="cuda")
    aux2 = torch.empty((n, 2, t, N), dtype=torch.int64, device="cuda")
    work = ext.clone()
    mplans = []
    for c in range(n):
        for p in range(2):
            spk = R.ptrs([ext[c, p, L + k] for k in range(K)])
            spc = R.ptrs([sp_coeff[c, p, k] for k in range(K)])
            axk = R.ptrs([aux2[c, p, k] for k in range(K)])
            md = R.ptrs([mdc[c, p, j] for j in range(t)])
            q = R.ptrs([work[c, p, j] for j in range(t)])
            axt = R.ptrs([aux2[c, p, j] for j in range(t)])
            mplans.append((spk, spc, axk, md, q, axt))

    def ref_moddown():
        for spk, spc, axk, md, q, axt in mplans:
            R.intt_launch(spk, axk, spc, K, R.special_base, stream=sp)
            R.moddown_conv_launch(spc, md, t, stream=sp)
            R.ntt_launch(md, axt, q, t, 0, mode=NTT_MODDOWN, stream=sp)

    # engine: extended ciphertexts from index-0 fast rotations (P*c0, P*c1), then KeySwitchDown
    xs = [ctx.eval_fast_rotation_ext(h, [0], True)[0] for h in hs]
    downs = []

    def eng_moddown():
        for d_ in downs:
            ctx.free(d_)
        downs.clear()
        for x in xs:
            downs.append(ctx.key_switch_down(x))

    out["moddown_8x2x(30+10)_towers_ms"] = {"reference": timed(ref_moddown, st), "engine": timed(eng_moddown, st)}
    ctx.close()


def main():
    out_path = sys.argv[1] if len(sys.argv) > 1 else "ref_kernel_compare.json"
    import torch
    res = {"gpu": torch.cuda.get_device_name(0)}
    st = torch.cuda.Stream()
    ntt_stage(res, st)
    keyswitch_stages(res, st)
    for k, v in res.items():
        if isinstance(v, dict) and "engine" in v:
            ref = [x for kk, x in v.items() if kk != "engine"][0]
            v["reference_over_engine"] = round(ref / v["engine"], 3)
    json.dump(res, open(out_path, "w"), indent=1)
    print(json.dumps(res, indent=1))


if __name__ == "__main__":
    main()
