// Device-side 64-bit modular arithmetic for residues modulo primes p < 2^60.
//
// Role in the reference: src/ModMult.cuh (Shoup / "better Barrett" / native u128 %) and src/AddSub.cuh.
// Formulation here (derived from the definitions, not from the reference):
//   * shoup_lazy(y, w, w') with w' = floor(w * 2^64 / p): q = hi64(w' * y), r = w*y - q*p, r in [0, 2p) for any
//     y < 2^64 (Shoup 1990s / Harvey 2014).  Used for every multiply by a precomputed constant (twiddles, CRT
//     factors, N^-1, P^-1).
//   * reduce128(hi, lo): any 128-bit z = hi*2^64 + lo is congruent to hi*[2^64 mod p] + lo, both terms are
//     reduced with shoup_lazy (constants [2^64 mod p] and 1), then summed and corrected: result in [0, p).
//     Used for data x data products and for the 128-bit accumulators of the basis conversions.
#pragma once
#include <cstdint>

namespace fgb {

typedef unsigned long long u64;

// Process-wide count of engine kernel launches (reported through fides_kernel_launches()).
void count_launch(unsigned n = 1);
unsigned long long launch_count();

// Per-prime constants, one entry per tower of the Q ∪ P basis, resident in device global memory.
struct PrimeConst {
  u64 p;        // modulus
  u64 p2;       // 2p
  u64 r64;      // 2^64 mod p
  u64 r64_sh;   // floor(r64 * 2^64 / p)
  u64 one_sh;   // floor(2^64 / p)
  u64 ninv;     // N^-1 mod p
  u64 ninv_sh;
  u64 negp;     // 2^64 - p
  u64 w1ninv;   // psi^-brev(1) * N^-1 mod p: the inverse transform's last-stage twiddle with N^-1 folded in
  u64 w1ninv_sh;
};

__device__ __forceinline__ u64 mulhi(u64 a, u64 b) { return __umul64hi(a, b); }

// y*w mod p in [0, 2p) for y < 2^64, w < p, wsh = floor(w*2^64/p).
__device__ __forceinline__ u64 shoup_lazy(u64 y, u64 w, u64 wsh, u64 p) {
  u64 q = mulhi(wsh, y);
  return y * w - q * p;
}

__device__ __forceinline__ u64 csub(u64 x, u64 m) { return x >= m ? x - m : x; }

// y*w mod p in [0, 4p) for any y < 2^64: the quotient hi64(wsh*y) is estimated from the three high 32x32
// partial products (dropping w0'*y0 and the low halves of the cross terms under-estimates it by at most 2),
// and r = w*y + q*(2^64 - p) is formed exactly modulo 2^64 (r < 4p).  Every 64-bit partial sum is built from 32-bit
// multiply-adds with a carry chain (mad.lo.cc / madc.hi) instead of 32x32->64 wide multiply-adds: on GB300 the wide
// form issues at about a third of the 32-bit multiply-add rate, and this form ran the NTT butterfly 6.5% faster
// (3.61 against 3.39 butterflies per clock per SM, identical results).
__device__ __forceinline__ u64 shoup_lazy4(u64 y, u64 w, u64 wsh, u64 negp) {
  u64 r;
  asm("{\n\t.reg .u32 y0,y1,s0,s1,w0,w1,n0,n1,t1,t2,q0,q1,r0,r1,c0,c1;\n\t"
      "mov.b64 {y0,y1}, %1;\n\tmov.b64 {w0,w1}, %2;\n\tmov.b64 {s0,s1}, %3;\n\tmov.b64 {n0,n1}, %4;\n\t"
      "mul.hi.u32 t1, s1, y0;\n\tmul.hi.u32 t2, s0, y1;\n\t"
      "add.cc.u32 c0, t1, t2;\n\taddc.u32 c1, 0, 0;\n\t"
      "mad.lo.cc.u32 q0, s1, y1, c0;\n\tmadc.hi.u32 q1, s1, y1, c1;\n\t"
      "mul.lo.u32 r0, w0, y0;\n\tmul.hi.u32 r1, w0, y0;\n\t"
      "mad.lo.cc.u32 r0, q0, n0, r0;\n\tmadc.hi.u32 r1, q0, n0, r1;\n\t"
      "mad.lo.u32 r1, w0, y1, r1;\n\tmad.lo.u32 r1, w1, y0, r1;\n\tmad.lo.u32 r1, q0, n1, r1;\n\t"
      "mad.lo.u32 r1, q1, n0, r1;\n\tmov.b64 %0, {r0,r1};\n\t}"
      : "=l"(r)
      : "l"(y), "l"(w), "l"(wsh), "l"(negp));
  return r;
}

__device__ __forceinline__ u64 shoup(u64 y, u64 w, u64 wsh, u64 p) { return csub(shoup_lazy(y, w, wsh, p), p); }

__device__ __forceinline__ u64 add_mod(u64 a, u64 b, u64 p) { return csub(a + b, p); }
__device__ __forceinline__ u64 sub_mod(u64 a, u64 b, u64 p) { return a >= b ? a - b : a + p - b; }

// z = hi*2^64 + lo reduced to [0, p).
__device__ __forceinline__ u64 reduce128(u64 hi, u64 lo, const PrimeConst& c) {
  u64 a = shoup_lazy(hi, c.r64, c.r64_sh, c.p);  // [0, 2p)
  u64 b = shoup_lazy(lo, 1ull, c.one_sh, c.p);   // [0, 2p)
  u64 s = a + b;                                 // [0, 4p) < 2^62
  s = csub(s, c.p2);
  return csub(s, c.p);
}

// y mod p in [0, 4p) for any y < 2^64: the w = 1 case of shoup_lazy4 (quotient hi64(floor(2^64/p) * y) from the
// three high partial products, remainder y + q * (2^64 - p)).
__device__ __forceinline__ u64 reduce64_lazy4(u64 y, u64 one_sh, u64 negp) {
  u64 r;
  asm("{\n\t.reg .u32 y0,y1,s0,s1,n0,n1,t1,t2,q0,q1,r0,r1,c0,c1;\n\t"
      "mov.b64 {y0,y1}, %1;\n\tmov.b64 {s0,s1}, %2;\n\tmov.b64 {n0,n1}, %3;\n\t"
      "mul.hi.u32 t1, s1, y0;\n\tmul.hi.u32 t2, s0, y1;\n\t"
      "add.cc.u32 c0, t1, t2;\n\taddc.u32 c1, 0, 0;\n\t"
      "mad.lo.cc.u32 q0, s1, y1, c0;\n\tmadc.hi.u32 q1, s1, y1, c1;\n\t"
      "mad.lo.cc.u32 r0, q0, n0, y0;\n\tmadc.hi.u32 r1, q0, n0, y1;\n\t"
      "mad.lo.u32 r1, q0, n1, r1;\n\tmad.lo.u32 r1, q1, n0, r1;\n\tmov.b64 %0, {r0,r1};\n\t}"
      : "=l"(r)
      : "l"(y), "l"(one_sh), "l"(negp));
  return r;
}

// z = hi*2^64 + lo reduced to [0, p): hi*[2^64 mod p] and lo each in [0, 4p), sum in [0, 8p), three corrections.
__device__ __forceinline__ u64 reduce128_fast(u64 hi, u64 lo, const PrimeConst& c) {
  const u64 a = shoup_lazy4(hi, c.r64, c.r64_sh, c.negp);
  const u64 b = reduce64_lazy4(lo, c.one_sh, c.negp);
  u64 s = a + b;
  s = csub(s, c.p2 << 1);
  s = csub(s, c.p2);
  return csub(s, c.p);
}

// The same without the final corrections: a value congruent to z in [0, 8p), for consumers that accept lazy
// inputs (the forward NTT takes [0, 8p)).
__device__ __forceinline__ u64 reduce128_lazy8(u64 hi, u64 lo, const PrimeConst& c) {
  return shoup_lazy4(hi, c.r64, c.r64_sh, c.negp) + reduce64_lazy4(lo, c.one_sh, c.negp);
}

__device__ __forceinline__ u64 mul_mod(u64 a, u64 b, const PrimeConst& c) {
  return reduce128_fast(mulhi(a, b), a * b, c);
}

// 128-bit accumulator helpers.
struct U128 {
  u64 lo, hi;
};
__device__ __forceinline__ void mac(U128& acc, u64 a, u64 b) {
  u64 lo = a * b;
  u64 hi = mulhi(a, b);
  acc.lo += lo;
  acc.hi += hi + (acc.lo < lo ? 1ull : 0ull);
}

}  // namespace fgb
