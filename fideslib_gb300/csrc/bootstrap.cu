// CKKS bootstrapping composed from the engine's ops (C ABI: fides_eval_bootstrap).
//
// Reference counterpart: FIDESlib::CKKS::Bootstrap (src/CKKS/Bootstrap.cu:169-333): ModRaise, the sparse-slot
// accumulation (AccumulateBroadcast.cu:79-113), EvalCoeffsToSlots (CoeffsToSlots.cu:26-151 over
// LinearTransform.cu:63-256), approxModReduction (ApproxModEval.cu:24-130) and SlotsToCoeffs.  The linear
// transforms' diagonals are supplied by the caller through fides_lt_create, the way FIDESlib receives its
// bootstrap plaintexts from OpenFHE (RawCiphertext.cu AddBootstrapPrecomputation); only the homomorphic
// evaluation runs here.  Steps:
//   1. x  = ModRaise(ct) to raise_towers towers;
//   2. x  = x + rot_{n 2^s}(x) for 2^s < N/(2n)   (trace onto the n-slot subring; needs keys n, 2n, ...);
//   3. re = Rescale(LT_cts_re(x) + conj(LT_cts_re(x))),  im = Rescale(LT_cts_im(x) + conj(LT_cts_im(x)))
//      (the caller's CoeffsToSlots diagonals give w/2 and -i w/2, w = coefficients packed as lo + i hi);
//   4. for v in (re, im): v = Rescale(DoubleAngle^R(Chebyshev(v)) * (K / 2 pi)) with K = q_0 / scale(ct),
//      the Chebyshev series approximating cos(2 pi (v/K - 1/4) / 2^R) on [cheb_lo, cheb_hi] (EvalMod);
//   5. out = Rescale(LT_stc_re(re) + LT_stc_im(im))  (SlotsToCoeffs).
// Every step is an engine op (bit-exact against the oracle); the caller chooses the ring, scales and the
// approximation.
#include <cmath>
#include <vector>

#include "../../include/fideslib_gb300.h"

namespace fgb {
int set_last_error(int code, const char* msg);
}

namespace {

struct Owned {
  fides_ctx* ctx;
  std::vector<uint32_t> h;
  explicit Owned(fides_ctx* c) : ctx(c) {}
  ~Owned() {
    for (uint32_t x : h)
      if (x) fides_ct_free(ctx, x);
  }
  uint32_t operator()(uint32_t x) {
    h.push_back(x);
    return x;
  }
};

#define TRY(x)                       \
  do {                               \
    const int rc_ = (x);             \
    if (rc_ != FIDES_OK) return rc_; \
  } while (0)

int cts_half(fides_ctx* ctx, Owned& own, uint32_t x, uint32_t lt, uint32_t conj_galois, uint32_t* out) {
  uint32_t y, c, s;
  TRY(fides_eval_linear_transform(ctx, x, lt, &y));
  own(y);
  TRY(fides_eval_automorphism(ctx, y, conj_galois, &c));
  own(c);
  TRY(fides_eval_add(ctx, y, c, &s));
  own(s);
  return fides_rescale(ctx, s, out);
}

// K = q_0 / (scale of the bootstrapped input): after CoeffsToSlots a slot holds (m_i + q_0 I_i) / scale_in.
int eval_mod(fides_ctx* ctx, Owned& own, uint32_t v, const fides_bootstrap_plan* p, double K, uint32_t* out) {
  uint32_t c, d, m;
  TRY(fides_eval_chebyshev(ctx, v, p->cheb_coeffs, p->cheb_n, p->cheb_lo, p->cheb_hi, p->const_scale, &c));
  own(c);
  if (p->double_angle) {
    TRY(fides_eval_double_angle(ctx, c, p->double_angle, &d));
    own(d);
  } else {
    d = c;
  }
  TRY(fides_eval_mult_scalar(ctx, d, K / (2.0 * M_PI), p->const_scale, &m));
  own(m);
  return fides_rescale(ctx, m, out);
}

}  // namespace

extern "C" int fides_eval_bootstrap(fides_ctx* ctx, uint32_t ct, const fides_bootstrap_plan* p, uint32_t* out) {
  if (!ctx || !p || !out || !p->cheb_coeffs || p->slots == 0)
    return fgb::set_last_error(FIDES_EINVAL, "null argument");
  fides_ctx_shape shape{};
  TRY(fides_ctx_get_shape(ctx, &shape));
  const uint32_t N = shape.n;
  if ((p->slots & (p->slots - 1)) || p->slots > N / 2)
    return fgb::set_last_error(FIDES_EINVAL, "slots must be a power of two <= N/2");
  uint64_t moduli[64];
  TRY(fides_ctx_moduli(ctx, moduli, nullptr));
  fides_ct_meta min{};
  TRY(fides_ct_meta_get(ctx, ct, &min));
  const double K = (double)moduli[0] / min.scale;
  Owned own(ctx);
  uint32_t x;
  TRY(fides_mod_raise(ctx, ct, p->raise_towers, &x));
  own(x);
  for (uint32_t r = p->slots; r < N / 2; r <<= 1) {  // trace onto the subring of the n-slot encoding
    uint32_t rx, s;
    TRY(fides_eval_rotate(ctx, x, (int32_t)r, &rx));
    own(rx);
    TRY(fides_eval_add(ctx, x, rx, &s));
    x = own(s);
  }
  const uint32_t conj = 2 * N - 1;
  uint32_t re, im;
  TRY(cts_half(ctx, own, x, p->lt_cts_re, conj, &re));
  own(re);
  TRY(cts_half(ctx, own, x, p->lt_cts_im, conj, &im));
  own(im);
  uint32_t mre, mim;
  TRY(eval_mod(ctx, own, re, p, K, &mre));
  own(mre);
  TRY(eval_mod(ctx, own, im, p, K, &mim));
  own(mim);
  uint32_t a, b, s;
  TRY(fides_eval_linear_transform(ctx, mre, p->lt_stc_re, &a));
  own(a);
  TRY(fides_eval_linear_transform(ctx, mim, p->lt_stc_im, &b));
  own(b);
  TRY(fides_eval_add(ctx, a, b, &s));
  own(s);
  return fides_rescale(ctx, s, out);
}
