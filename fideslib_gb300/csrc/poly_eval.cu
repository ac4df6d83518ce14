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
// scaling modes.
#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/fideslib_gb300.h"

namespace fgb {
int set_last_error(int code, const char* msg);
}

namespace {

struct Scope {
  fides_ctx* ctx;
  std::vector<uint32_t> owned;
  int rc = FIDES_OK;
  explicit Scope(fides_ctx* c) : ctx(c) {}
  ~Scope() {
    for (uint32_t h : owned)
      if (h) fides_ct_free(ctx, h);
  }
  uint32_t keep(uint32_t h) {
    owned.push_back(h);
    return h;
  }
  void release(uint32_t h) {
    for (auto& x : owned)
      if (x == h) x = 0;
  }
};

uint32_t towers_of(fides_ctx* ctx, uint32_t h) {
  fides_ct_meta m{};
  fides_ct_meta_get(ctx, h, &m);
  return m.towers;
}

// a dropped to `t` towers (a itself when it already has t towers); new handles are owned by the scope.
int drop_to(Scope& sc, uint32_t a, uint32_t t, uint32_t* out) {
  if (towers_of(sc.ctx, a) == t) {
    *out = a;
    return FIDES_OK;
  }
  int rc = fides_level_reduce(sc.ctx, a, t, out);
  if (rc == FIDES_OK) sc.keep(*out);
  return rc;
}

#define TRY(x)                   \
  do {                           \
    const int rc_ = (x);         \
    if (rc_ != FIDES_OK) return rc_; \
  } while (0)

// 2*Rescale(v) + c where c = -1 (even step) or -T1 (odd step); v is owned by the scope.
int double_and_shift(Scope& sc, uint32_t prod, uint32_t t1, uint32_t* out) {
  uint32_t r, m2;
  TRY(fides_rescale(sc.ctx, prod, &r));
  sc.keep(r);
  TRY(fides_eval_mult_int(sc.ctx, r, 2, &m2));
  sc.keep(m2);
  if (!t1) {
    TRY(fides_eval_add_scalar(sc.ctx, m2, -1.0, out));
  } else {
    uint32_t t1d;
    TRY(drop_to(sc, t1, towers_of(sc.ctx, m2), &t1d));
    TRY(fides_eval_sub(sc.ctx, m2, t1d, out));
  }
  return FIDES_OK;
}

}  // namespace

extern "C" int fides_eval_chebyshev(fides_ctx* ctx, uint32_t a, const double* coeffs, uint32_t n, double lo, double hi,
                                    double const_scale, uint32_t* out) {
  if (!ctx || !coeffs || !out || n < 2) return fgb::set_last_error(FIDES_EINVAL, "need a context, >= 2 coefficients");
  if (!(hi > lo)) return fgb::set_last_error(FIDES_EINVAL, "need lo < hi");
  Scope sc(ctx);
  const int d = (int)n - 1;
  std::vector<uint32_t> T(d + 1, 0);
  if (lo == -1.0 && hi == 1.0) {
    T[1] = a;
  } else {
    uint32_t u, r;
    TRY(fides_eval_mult_scalar(ctx, a, 2.0 / (hi - lo), const_scale, &u));
    sc.keep(u);
    TRY(fides_rescale(ctx, u, &r));
    sc.keep(r);
    TRY(fides_eval_add_scalar(ctx, r, -(hi + lo) / (hi - lo), &T[1]));
    sc.keep(T[1]);
  }
  for (int k = 2; k <= d; k++) {
    uint32_t prod;
    if (k % 2 == 0) {
      TRY(fides_eval_square(ctx, T[k / 2], &prod));
      sc.keep(prod);
      TRY(double_and_shift(sc, prod, 0, &T[k]));
    } else {
      const uint32_t A = T[(k - 1) / 2], B = T[(k + 1) / 2];
      const uint32_t t = std::min(towers_of(ctx, A), towers_of(ctx, B));
      uint32_t Ad, Bd;
      TRY(drop_to(sc, A, t, &Ad));
      TRY(drop_to(sc, B, t, &Bd));
      TRY(fides_eval_mult(ctx, Ad, Bd, &prod));
      sc.keep(prod);
      TRY(double_and_shift(sc, prod, T[1], &T[k]));
    }
    sc.keep(T[k]);
  }
  uint32_t tmin = ~0u;
  for (int k = 1; k <= d; k++)
    if (coeffs[k] != 0.0) tmin = std::min(tmin, towers_of(ctx, T[k]));
  uint32_t acc = 0;
  for (int k = 1; k <= d; k++) {
    if (coeffs[k] == 0.0) continue;
    uint32_t X, term;
    TRY(drop_to(sc, T[k], tmin, &X));
    TRY(fides_eval_mult_scalar(ctx, X, coeffs[k], const_scale, &term));
    sc.keep(term);
    if (!acc) {
      acc = term;
    } else {
      uint32_t s2;
      TRY(fides_eval_add(ctx, acc, term, &s2));
      sc.keep(s2);
      acc = s2;
    }
  }
  if (!acc) return fgb::set_last_error(FIDES_EINVAL, "all non-constant coefficients are zero");
  uint32_t r;
  TRY(fides_rescale(ctx, acc, &r));
  sc.keep(r);
  TRY(fides_eval_add_scalar(ctx, r, coeffs[0], out));
  if (T[1] == a) sc.release(a);
  return FIDES_OK;
}

// x <- 2 x^2 - 1, `iterations` times (cos(2t) from cos(t)): ApplyDoubleAngleIterations.
extern "C" int fides_eval_double_angle(fides_ctx* ctx, uint32_t a, uint32_t iterations, uint32_t* out) {
  if (!ctx || !out) return fgb::set_last_error(FIDES_EINVAL, "null argument");
  Scope sc(ctx);
  uint32_t x = a;
  for (uint32_t i = 0; i < iterations; i++) {
    uint32_t sq, nx;
    TRY(fides_eval_square(ctx, x, &sq));
    sc.keep(sq);
    TRY(double_and_shift(sc, sq, 0, &nx));
    if (i + 1 < iterations) sc.keep(nx);
    x = nx;
  }
  if (iterations == 0) return fgb::set_last_error(FIDES_EINVAL, "iterations must be >= 1");
  *out = x;
  return FIDES_OK;
}
