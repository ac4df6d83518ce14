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
  u64 pad;
};

__device__ __forceinline__ u64 mulhi(u64 a, u64 b) { return __umul64hi(a, b); }

// y*w mod p in [0, 2p) for y < 2^64, w < p, wsh = floor(w*2^64/p).
__device__ __forceinline__ u64 shoup_lazy(u64 y, u64 w, u64 wsh, u64 p) {
  u64 q = mulhi(wsh, y);
  return y * w - q * p;
}

__device__ __forceinline__ u64 csub(u64 x, u64 m) { return x >= m ? x - m : x; }

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

__device__ __forceinline__ u64 mul_mod(u64 a, u64 b, const PrimeConst& c) {
  return reduce128(mulhi(a, b), a * b, c);
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
