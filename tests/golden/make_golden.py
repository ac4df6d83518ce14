"""Generates tests/golden/ntt_reference.npz from the reference's own CPU NTT.

The reference functions FIDESlib::Testing::nega_fft / nega_fft2 (test/cpuNTT_nega.cpp:24-170) are compiled
from the reference sources by oracle/build_ref.sh; this script calls them on seeded inputs and stores inputs,
tables and outputs.  Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle as O  # noqa: E402


def main():
    O.build_ref()
    R = O.ref_lib()
    if R is None:
        raise SystemExit("reference tree not available; cannot regenerate golden vectors")
    out = {}
    cases = [(3, 17), (4, 97), (10, None), (12, None), (13, None)]
    rng = np.random.default_rng(0x5EED0002)
    for idx, (logn, p) in enumerate(cases):
        N = 1 << logn
        if p is None:
            p = O.gen_primes(60 - idx, 1, 2 * N)[0]
        psi = O.root_of_unity(p, 2 * N)
        tab, itab = O.ntt_tables(N, p, psi)
        if N == 8 and p == 17:
            a = np.array([1, 2, 3, 7, 5, 4, 1, 2], dtype=np.uint64)  # test/NegacyclicNTTtests.cu:44-68
        else:
            a = rng.integers(0, p, N, dtype=np.uint64)
        f1 = a.copy()
        R.ref_nega_fft(O._p(f1), N, 0, O._p(tab), O._p(itab), p)
        f2 = a.copy()
        R.ref_nega_fft2(O._p(f2), N, 0, O._p(tab), O._p(itab), p)
        i2 = f2.copy()
        R.ref_nega_fft2(O._p(i2), N, 1, O._p(tab), O._p(itab), p)
        key = f"n{N}_p{p}"
        out[key + "_in"] = a
        out[key + "_psi"] = np.array([psi], dtype=np.uint64)
        out[key + "_nega_fft"] = f1
        out[key + "_nega_fft2"] = f2
        out[key + "_nega_fft2_inv"] = i2
    np.savez_compressed(os.path.join(os.path.dirname(os.path.abspath(__file__)), "ntt_reference.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
