// CKKS bootstrapping composed from the engine's ops (C ABI: fides_eval_bootstrap, fides_eval_bootstrap_batch).
//
// Reference counterpart: FIDESlib::CKKS::Bootstrap (src/CKKS/Bootstrap.cu:169-333): ModRaise with optional
// sparse-secret encapsulation (Bootstrap.cu:592-600, 254-262), the sparse-slot accumulation
// (AccumulateBroadcast.cu:79-113), EvalCoeffsToSlots over the level-budget factors (CoeffsToSlots.cu:77-151,
// LinearTransform.cu:63-256), the full-slot real/imaginary split by conjugation and multMonomial
// (Bootstrap.cu:256-270), approxModReduction (ApproxModEval.cu:24-130) and SlotsToCoeffs.  The transforms'
// diagonals are supplied by the caller through fides_lt_create_strided, the way FIDESlib receives its
// bootstrap plaintexts from OpenFHE (RawCiphertext.cu AddBootstrapPrecomputation); only the homomorphic
// evaluation runs here.  For n = slots and each input ciphertext:
//   0. (prescale != 0) x = Rescale(x * round(prescale * q_top)), q_top the top prime of x
//   1. (sse)  x = KeySwitch_{dense->sparse}(x dropped to one tower)
//   2.        x = ModRaise(x) to raise_towers towers;  (sse) x = KeySwitch_{sparse->dense}(x)
//   3.        x = x + rot_r(x) for r = n, 2n, ..., N/4        (trace onto the n-slot subring; n < N/2 only)
//   4.        x = Rescale(LT_cts[l](x)) for each CoeffsToSlots factor l
//   5.        re = x + conj(x),  im = (x - conj(x)) * X^(3N/2)      (X^(3N/2) multiplies slots by -i)
//   6.        v = Rescale(DoubleAngle^R(Chebyshev(v)) * (K / 2 pi)) for v in (re, im), K = q_0 / scale(input)
//             (the series approximates cos(2 pi (v/K - 1/4) / 2^R) on [cheb_lo, cheb_hi]: EvalMod)
//   7.        w = re + im * X^(N/2)                                  (X^(N/2) multiplies slots by i)
//   8.        w = Rescale(LT_stc[l](w)) for each SlotsToCoeffs factor l
// The batch form runs m ciphertexts through these steps in lock step: every rotation, key switch, product
// and rescale of a step is one batched launch for all of them (EvalMod on 2m ciphertexts), and each result
// equals the single-ciphertext call's.  Every step is an engine op, so the whole recipe replays op-for-op
// on a CPU restatement.
#include <cmath>
#include <vector>

#include "vecops.hpp"

namespace fgb::vec {
int chebyshev_batch(fides_ctx* ctx, const V& a, const double* coeffs, uint32_t n, double lo, double hi,
                    double const_scale, V& out);
int double_angle_batch(fides_ctx* ctx, const V& a, uint32_t iterations, V& out);
}  // namespace fgb::vec

namespace {

using fgb::vec::Scope;
using fgb::vec::V;

int rescaled_lt(Scope& sc, const V& x, uint32_t lt, V& out) {
  V y;
  FGB_TRY(fgb::vec::linear_transform(sc, x, lt, y));
  return fgb::vec::rescale(sc, y, out);
}

int bootstrap(fides_ctx* ctx, const V& in, const fides_bootstrap_plan* p, V& out) {
  if (!ctx || !p || !p->cheb_coeffs || p->slots == 0) return fgb::set_last_error(FIDES_EINVAL, "null argument");
  if (p->cts_count < 1 || p->cts_count > 4 || p->stc_count < 1 || p->stc_count > 4)
    return fgb::set_last_error(FIDES_EINVAL, "1 to 4 CoeffsToSlots and SlotsToCoeffs factors");
  fides_ctx_shape shape{};
  FGB_TRY(fides_ctx_get_shape(ctx, &shape));
  const uint32_t N = shape.n;
  if ((p->slots & (p->slots - 1)) || p->slots > N / 2)
    return fgb::set_last_error(FIDES_EINVAL, "slots must be a power of two <= N/2");
  uint64_t moduli[64];
  FGB_TRY(fides_ctx_moduli(ctx, moduli, nullptr));
  const size_t m = in.size();
  Scope sc(ctx);
  V x = in;
  if (p->prescale != 0.0) {  // the reference's ModRaise adjustment (its `prescaled` = false)
    std::vector<double> top(m);
    for (size_t i = 0; i < m; i++) {
      const uint32_t t = fgb::vec::towers_of(ctx, x[i]);
      if (t < 2) return fgb::set_last_error(FIDES_EINVAL, "prescaling needs an input of at least two towers");
      top[i] = (double)moduli[t - 1];
    }
    V y, z;
    FGB_TRY(fgb::vec::mult_scalar_at(sc, x, p->prescale, top, y));
    FGB_TRY(fgb::vec::rescale(sc, y, z));
    x = z;
  }
  std::vector<double> k_over_2pi(2 * m);
  for (size_t i = 0; i < m; i++) {
    const double scale_in = fgb::vec::scale_of(ctx, x[i]);
    if (!(scale_in > 0)) return fgb::set_last_error(FIDES_EINVAL, "unknown ciphertext handle");
    k_over_2pi[i] = k_over_2pi[m + i] = (double)moduli[0] / scale_in / (2.0 * M_PI);
  }
  if (p->sse) {
    V low, sw;
    FGB_TRY(fgb::vec::drop_to(sc, x, std::vector<uint32_t>(m, 1), low));
    FGB_TRY(fgb::vec::key_switch(sc, low, p->sse_to_sparse, sw));
    x = sw;
  }
  {
    V r;
    FGB_TRY(fgb::vec::mod_raise(sc, x, p->raise_towers, r));
    x = r;
  }
  if (p->sse) {
    V sw;
    FGB_TRY(fgb::vec::key_switch(sc, x, p->sse_to_dense, sw));
    x = sw;
  }
  for (uint32_t r = p->slots; r < N / 2; r <<= 1) {  // trace onto the subring of the n-slot encoding
    V rx, s;
    FGB_TRY(fgb::vec::rotate(sc, x, (int32_t)r, rx));
    FGB_TRY(fgb::vec::add(sc, x, rx, s));
    x = s;
  }
  for (uint32_t l = 0; l < p->cts_count; l++) {
    V y;
    FGB_TRY(rescaled_lt(sc, x, p->lt_cts[l], y));
    x = y;
  }
  V halves(2 * m);
  {
    V c, re, d, im;
    FGB_TRY(fgb::vec::automorphism(sc, x, 2 * N - 1, c));
    FGB_TRY(fgb::vec::add(sc, x, c, re));
    FGB_TRY(fgb::vec::sub(sc, x, c, d));
    FGB_TRY(fgb::vec::monomial(sc, d, 3 * N / 2, im));
    for (size_t i = 0; i < m; i++) {
      halves[i] = re[i];
      halves[m + i] = im[i];
    }
  }
  V modded;
  {
    V c, d;
    FGB_TRY(fgb::vec::chebyshev_batch(ctx, halves, p->cheb_coeffs, p->cheb_n, p->cheb_lo, p->cheb_hi,
                                      p->const_scale, c));
    sc.keep(c);
    if (p->double_angle) {
      FGB_TRY(fgb::vec::double_angle_batch(ctx, c, p->double_angle, d));
      sc.keep(d);
    } else {
      d = c;
    }
    V sm;
    FGB_TRY(fgb::vec::mult_scalar(sc, d, k_over_2pi, p->const_scale, sm));
    FGB_TRY(fgb::vec::rescale(sc, sm, modded));
  }
  V w;
  {
    const V re(modded.begin(), modded.begin() + m), im(modded.begin() + m, modded.end());
    V iim;
    FGB_TRY(fgb::vec::monomial(sc, im, N / 2, iim));
    FGB_TRY(fgb::vec::add(sc, re, iim, w));
  }
  for (uint32_t l = 0; l < p->stc_count; l++) {
    V y;
    FGB_TRY(rescaled_lt(sc, w, p->lt_stc[l], y));
    w = y;
  }
  out = w;
  sc.release(out);
  return FIDES_OK;
}

}  // namespace

extern "C" int fides_eval_bootstrap(fides_ctx* ctx, uint32_t ct, const fides_bootstrap_plan* p, uint32_t* out) {
  return fides_eval_bootstrap_batch(ctx, 1, &ct, p, out);
}

extern "C" int fides_eval_bootstrap_batch(fides_ctx* ctx, uint32_t m, const uint32_t* cts,
                                          const fides_bootstrap_plan* p, uint32_t* outs) {
  if (!cts || !outs || m == 0) return fgb::set_last_error(FIDES_EINVAL, "null argument");
  V out;
  FGB_TRY(bootstrap(ctx, V(cts, cts + m), p, out));
  std::copy(out.begin(), out.end(), outs);
  return FIDES_OK;
}
