// Polynomial evaluation on ciphertexts: EvalChebyshevSeries and the double-angle iterations of EvalMod.
//
// Reference counterparts: CryptoContextImpl::EvalChebyshevSeries (api/CryptoContext.hpp:154-156),
// FIDESlib's Chebyshev Paterson–Stockmeyer evaluation and double-angle loop (src/CKKS/ApproxModEval.cu:
// 138-370, 724-739).  Here the series is evaluated from the Chebyshev polynomials T_1..T_d built by the
// doubling identities (depth ceil(log2 d) + 2), a recipe chosen so that every step is one engine op and the
// whole sequence can be replayed op-for-op by an independent checker:
//   y   = x                                  when [lo, hi] = [-1, 1]
//       = Rescale(x * (2/(hi-lo))) - (hi+lo)/(hi-lo)   otherwise (constant encoded at const_scale)
//   T_1 = y
//   T_k = Rescale(T_{k/2}^2) * 2 - 1                               k even
//   T_k = Rescale(T_a * T_b) * 2 - T_1,  a = (k-1)/2, b = (k+1)/2    k odd   (operands level-aligned by
//         dropping towers of the higher one; T_1 dropped to the product's towers)
//   p   = Rescale( sum_{k>=1, c_k != 0} T_k * c_k ) + c_0   (each T_k dropped to the smallest tower count,
//         c_k encoded at const_scale; terms summed in increasing k)
// Scales follow the ciphertext metadata (rescale divides by the dropped prime); sums of terms whose scales
// differ by the primes' distance from the nominal scale carry that relative error, as in OpenFHE's fixed
// scaling modes.  The *_batch forms run m ciphertexts through the recipe in lock step, one batched launch
// per step; each result is the same as the single-ciphertext call's.
#include <algorithm>
#include <cmath>
#include <vector>

#include "vecops.hpp"

namespace {

using fgb::vec::Scope;
using fgb::vec::V;

// 2*Rescale(prod) + c where c = -1 (t1 empty: even step) or -T1 (odd step).
int double_and_shift(Scope& sc, const V& prod, const V* t1, V& out) {
  V r, m2;
  FGB_TRY(fgb::vec::rescale(sc, prod, r));
  FGB_TRY(fgb::vec::mult_int(sc, r, 2, m2));
  if (!t1) return fgb::vec::add_scalar(sc, m2, -1.0, out);
  V t1d;
  FGB_TRY(fgb::vec::drop_to(sc, *t1, fgb::vec::towers(sc.ctx, m2), t1d));
  return fgb::vec::sub(sc, m2, t1d, out);
}

int chebyshev(fides_ctx* ctx, const V& a, const double* coeffs, uint32_t n, double lo, double hi, double const_scale,
              V& out) {
  if (!ctx || !coeffs || n < 2) return fgb::set_last_error(FIDES_EINVAL, "need a context, >= 2 coefficients");
  if (!(hi > lo)) return fgb::set_last_error(FIDES_EINVAL, "need lo < hi");
  Scope sc(ctx);
  const int d = (int)n - 1;
  std::vector<V> T(d + 1);
  if (lo == -1.0 && hi == 1.0) {
    T[1] = a;
  } else {
    V u, r;
    FGB_TRY(fgb::vec::mult_scalar(sc, a, 2.0 / (hi - lo), const_scale, u));
    FGB_TRY(fgb::vec::rescale(sc, u, r));
    FGB_TRY(fgb::vec::add_scalar(sc, r, -(hi + lo) / (hi - lo), T[1]));
  }
  for (int k = 2; k <= d; k++) {
    V prod;
    if (k % 2 == 0) {
      FGB_TRY(fgb::vec::square(sc, T[k / 2], prod));
      FGB_TRY(double_and_shift(sc, prod, nullptr, T[k]));
    } else {
      const V& A = T[(k - 1) / 2];
      const V& B = T[(k + 1) / 2];
      std::vector<uint32_t> t = fgb::vec::towers(ctx, A), tb = fgb::vec::towers(ctx, B);
      for (size_t i = 0; i < t.size(); i++) t[i] = std::min(t[i], tb[i]);
      V Ad, Bd;
      FGB_TRY(fgb::vec::drop_to(sc, A, t, Ad));
      FGB_TRY(fgb::vec::drop_to(sc, B, t, Bd));
      FGB_TRY(fgb::vec::mult(sc, Ad, Bd, prod));
      FGB_TRY(double_and_shift(sc, prod, &T[1], T[k]));
    }
  }
  std::vector<uint32_t> tmin(a.size(), ~0u);
  bool any = false;
  for (int k = 1; k <= d; k++) {
    if (coeffs[k] == 0.0) continue;
    any = true;
    const std::vector<uint32_t> tk = fgb::vec::towers(ctx, T[k]);
    for (size_t i = 0; i < a.size(); i++) tmin[i] = std::min(tmin[i], tk[i]);
  }
  if (!any) return fgb::set_last_error(FIDES_EINVAL, "all non-constant coefficients are zero");
  V acc;
  for (int k = 1; k <= d; k++) {
    if (coeffs[k] == 0.0) continue;
    V X, term;
    FGB_TRY(fgb::vec::drop_to(sc, T[k], tmin, X));
    FGB_TRY(fgb::vec::mult_scalar(sc, X, coeffs[k], const_scale, term));
    if (acc.empty()) {
      acc = term;
    } else {
      V s2;
      FGB_TRY(fgb::vec::add(sc, acc, term, s2));
      acc = s2;
    }
  }
  V r;
  FGB_TRY(fgb::vec::rescale(sc, acc, r));
  FGB_TRY(fgb::vec::add_scalar(sc, r, coeffs[0], out));
  sc.release(out);
  return FIDES_OK;
}

int double_angle(fides_ctx* ctx, const V& a, uint32_t iterations, V& out) {
  if (!ctx) return fgb::set_last_error(FIDES_EINVAL, "null argument");
  if (iterations == 0) return fgb::set_last_error(FIDES_EINVAL, "iterations must be >= 1");
  Scope sc(ctx);
  V x = a;
  for (uint32_t i = 0; i < iterations; i++) {
    V sq, nx;
    FGB_TRY(fgb::vec::square(sc, x, sq));
    FGB_TRY(double_and_shift(sc, sq, nullptr, nx));
    x = nx;
  }
  out = x;
  sc.release(out);
  return FIDES_OK;
}

}  // namespace

namespace fgb::vec {
// Entry points for the other composite routines (bootstrapping).
int chebyshev_batch(fides_ctx* ctx, const V& a, const double* coeffs, uint32_t n, double lo, double hi,
                    double const_scale, V& out) {
  return chebyshev(ctx, a, coeffs, n, lo, hi, const_scale, out);
}
int double_angle_batch(fides_ctx* ctx, const V& a, uint32_t iterations, V& out) {
  return double_angle(ctx, a, iterations, out);
}
}  // namespace fgb::vec

extern "C" int fides_eval_chebyshev(fides_ctx* ctx, uint32_t a, const double* coeffs, uint32_t n, double lo, double hi,
                                    double const_scale, uint32_t* out) {
  return fides_eval_chebyshev_batch(ctx, 1, &a, coeffs, n, lo, hi, const_scale, out);
}

extern "C" int fides_eval_chebyshev_batch(fides_ctx* ctx, uint32_t m, const uint32_t* cts, const double* coeffs,
                                          uint32_t n, double lo, double hi, double const_scale, uint32_t* outs) {
  if (!cts || !outs) return fgb::set_last_error(FIDES_EINVAL, "null argument");
  V out;
  FGB_TRY(chebyshev(ctx, V(cts, cts + m), coeffs, n, lo, hi, const_scale, out));
  std::copy(out.begin(), out.end(), outs);
  return FIDES_OK;
}

// x <- 2 x^2 - 1, `iterations` times (cos(2t) from cos(t)): ApplyDoubleAngleIterations.
extern "C" int fides_eval_double_angle(fides_ctx* ctx, uint32_t a, uint32_t iterations, uint32_t* out) {
  return fides_eval_double_angle_batch(ctx, 1, &a, iterations, out);
}

extern "C" int fides_eval_double_angle_batch(fides_ctx* ctx, uint32_t m, const uint32_t* cts, uint32_t iterations,
                                             uint32_t* outs) {
  if (!cts || !outs) return fgb::set_last_error(FIDES_EINVAL, "null argument");
  V out;
  FGB_TRY(double_angle(ctx, V(cts, cts + m), iterations, out));
  std::copy(out.begin(), out.end(), outs);
  return FIDES_OK;
}
