// Scaling techniques at the boundary: per-level scaling tables and the automatic rescaling / level alignment of
// FIXEDAUTO, FLEXIBLEAUTO and FLEXIBLEAUTOEXT that the reference applies before additions and multiplications
// (Ciphertext::adjustForAddOrSub, adjustForMult and adjustScaleAndLevel, src/CKKS/Ciphertext.cpp:1376-1518; the
// constant encoding of ContextData::ElemForEvalMult, src/CKKS/Context.cu:366-458).  Every step is an engine op
// (rescale, scalar product, tower drop) issued on the context stream ahead of the op it prepares.
#include <cmath>
#include <string>

#include "../../include/fideslib_gb300.h"
#include "autoscale.hpp"

namespace fgb {
int set_last_error(int code, const char* msg);

namespace {
typedef __int128 i128;
typedef unsigned __int128 u128;

u64 shoup_const(u64 w, u64 q) { return (u64)(((u128)w << 64) / q); }
u64 mulmod(u64 a, u64 b, u64 q) { return (u64)((u128)a * b % q); }
}  // namespace

int Context::set_scaling(int tech, const double* sf_in, const double* big_in, const double* mrf_in,
                         double default_scale, std::string* err) {
  if (tech < FIDES_FIXEDMANUAL || tech > FIDES_FLEXIBLEAUTOEXT) {
    *err = "unknown scaling technique";
    return FIDES_EINVAL;
  }
  technique = tech;
  sf.assign(nq, 0.0);
  big.assign(nq, 0.0);
  mrf.assign(nq, 0.0);
  // ModReduceFactor: the prime a rescale divides by (OpenFHE GetModReduceFactor(l) = q_l as a double).
  for (int l = 0; l < nq; l++) mrf[l] = mrf_in ? mrf_in[l] : (double)mod[l];
  if (sf_in) {
    for (int l = 0; l < nq; l++) sf[l] = sf_in[l];
  } else if (tech == FIDES_FIXEDMANUAL || tech == FIDES_FIXEDAUTO) {
    // One approximate factor 2^p for every level (OpenFHE's FIXED* techniques).
    const double d = default_scale > 0 ? default_scale : std::ldexp(1.0, (int)std::lround(std::log2((double)mod[nq - 1])));
    for (int l = 0; l < nq; l++) sf[l] = d;
  } else {
    // FLEXIBLEAUTO: the top level's factor is its prime, and each lower level's is the square of the one above
    // divided by the prime the rescale removes, so that mult + rescale lands exactly on the next factor
    // (sf[l - 1] * q_l = sf[l]^2).  FLEXIBLEAUTOEXT starts one prime lower: the top two levels use q_{L-1}.
    const int L = nq - 1;
    if (tech == FIDES_FLEXIBLEAUTO) {
      sf[L] = (double)mod[L];
    } else {
      sf[L] = nq >= 2 ? (double)mod[L - 1] : (double)mod[L];
      if (L >= 1) sf[L - 1] = (double)mod[L - 1];
    }
    for (int l = (tech == FIDES_FLEXIBLEAUTO ? L : L - 1) - 1; l >= 0; l--) sf[l] = sf[l + 1] * sf[l + 1] / (double)mod[l + 1];
  }
  if (big_in) {
    for (int l = 0; l < nq; l++) big[l] = big_in[l];
  } else {
    for (int l = 0; l < nq; l++) big[l] = sf[l] * sf[l];
    if (tech == FIDES_FLEXIBLEAUTOEXT && nq >= 2) big[nq - 1] = sf[nq - 1] * sf[nq - 2];
  }
  for (int l = 0; l < nq; l++)
    if (!(sf[l] > 0) || !(big[l] > 0) || !(mrf[l] > 0)) {
      *err = "scaling tables must be positive";
      return FIDES_EINVAL;
    }
  return FIDES_OK;
}

void Context::eval_mult_constants(int t, double operand, u64* out) const {
  // round(operand * sf[t - 1]) as an exact integer (truncation of x + 0.5 toward zero, the reference's cast), then
  // reduced per tower; values past 2^125 are scaled down by 2^k first and the factor is restored per tower.
  const double scf = sf[t - 1];
  int log_approx = 0;
  const double res = std::fabs(operand * scf);
  if (res > 0) {
    const int log_sf = (int)std::ceil(std::log2(res));
    const int log_valid = log_sf <= 125 ? log_sf : 125;
    log_approx = log_sf - log_valid;
  }
  const double approx = std::pow(2.0, log_approx);
  const i128 large = (i128)(operand / approx * scf + 0.5);
  const i128 large_abs = large < 0 ? -large : large;
  const i128 bound = (i128)1 << 63;
  for (int i = 0; i < t; i++) {
    const u64 q = mod[i];
    u64 f;
    if (large_abs > bound) {
      const i128 r = large % (i128)q;
      f = (u64)(r < 0 ? r + (i128)q : r);
    } else {
      const int64_t r = (int64_t)large % (int64_t)q;
      f = (u64)(r < 0 ? r + (int64_t)q : r);
    }
    if (log_approx > 0) {
      u64 p2 = 1 % q, b = 2 % q;
      for (int k = log_approx; k > 0; k >>= 1) {
        if (k & 1) p2 = mulmod(p2, b, q);
        b = mulmod(b, b, q);
      }
      f = mulmod(f, p2, q);
    }
    out[i] = f % q;
  }
}

// ---------------------------------------------------------------------------------------------------------------
// Operand alignment

AutoScaler::~AutoScaler() {
  for (u64* p : temps_) c_->free_limbs(p, s_);
}

void AutoScaler::replace(DevCt& x, const DevCt& y) {
  // x's previous data is freed only if it is a temporary of this scaler (never a caller's ciphertext); the free is
  // stream-ordered after the op that read it.
  for (size_t i = 0; i < temps_.size(); i++)
    if (temps_[i] == x.data) {
      c_->free_limbs(x.data, s_);
      temps_.erase(temps_.begin() + (long)i);
      break;
    }
  x = y;
}

int AutoScaler::alloc(int t, DevCt* out) {
  out->data = c_->alloc_limbs((size_t)2 * t, s_);
  if (!out->data) return set_last_error(FIDES_ENOMEM, "ciphertext allocation failed (automatic rescaling)");
  out->t = t;
  temps_.push_back(out->data);
  return FIDES_OK;
}

int AutoScaler::rescale(DevCt& x) {
  if (x.t < 2) return set_last_error(FIDES_EINVAL, "automatic rescaling needs a second tower");
  DevCt y = x;
  if (int rc = alloc(x.t - 1, &y)) return rc;
  const Context::RescaleReq r{x.data, x.t, y.data};
  if (cudaError_t e = c_->rescale_batch(&r, 1, s_)) return set_last_error(FIDES_ECUDA, cudaGetErrorString(e));
  y.scale = x.scale / c_->mrf[x.t - 1];
  y.noise_deg = x.noise_deg - 1;
  replace(x, y);
  return FIDES_OK;
}

int AutoScaler::drop(DevCt& x, int t) {
  if (t >= x.t) return FIDES_OK;
  if (t < 1) return set_last_error(FIDES_EINVAL, "cannot drop below one tower");
  DevCt y = x;
  if (int rc = alloc(t, &y)) return rc;
  const size_t NN = (size_t)c_->N, bytes = (size_t)t * NN * sizeof(u64);
  cudaError_t e = cudaMemcpyAsync(y.data, x.data, bytes, cudaMemcpyDeviceToDevice, s_);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(y.data + (size_t)t * NN, x.data + (size_t)x.t * NN, bytes, cudaMemcpyDeviceToDevice, s_);
  if (e != cudaSuccess) return set_last_error(FIDES_ECUDA, cudaGetErrorString(e));
  replace(x, y);
  return FIDES_OK;
}

int AutoScaler::mult_const(DevCt& x, double operand) {
  // multScalarNoPrecheck: product by the constant encoded at sf[level]; the degree and the scale grow.
  DevCt y = x;
  if (int rc = alloc(x.t, &y)) return rc;
  ScalarBatch sb{};
  sb.njobs = 1;
  sb.jobs[0] = ScalarJob{x.data, y.data, x.t, 0};
  u64 k[64];
  c_->eval_mult_constants(x.t, operand, k);
  for (int i = 0; i < x.t; i++) {
    sb.sets[0].mul[i] = k[i];
    sb.sets[0].mul_sh[i] = shoup_const(k[i], c_->mod[i]);
    sb.sets[0].add[i] = 0;
  }
  const Ring ring{c_->N, c_->logN};
  if (cudaError_t e = launch_scalar(sb, ring, c_->d_pc, s_)) return set_last_error(FIDES_ECUDA, cudaGetErrorString(e));
  y.noise_deg = x.noise_deg + 1;
  y.scale = x.scale * c_->sf[x.t - 1];
  replace(x, y);
  return FIDES_OK;
}

int AutoScaler::scale_and_level(DevCt& x, int deg2, int t2, double scale2, bool* ok) {
  // Ciphertext::adjustScaleAndLevel with levels counted as towers - 1.
  const Context& C = *c_;
  const int l1 = x.t - 1, l2 = t2 - 1, d1 = x.noise_deg;
  *ok = true;
  if (l1 > l2) {
    if (d1 == 2) {
      if (deg2 == 2) {
        const double scf1 = x.scale, scf = C.sf[l1], q1 = C.mrf[l2 + 1];
        if (int rc = mult_const(x, scale2 * q1 / scf1 / scf)) return rc;
        if (x.t - 1 > l2 + 1)
          if (int rc = drop(x, l2 + 2)) return rc;
        x.scale = C.big[l2] * C.mrf[l2 + 1];
        if (int rc = rescale(x)) return rc;
        x.scale = scale2;
      } else if (l1 - 1 == l2) {
        if (int rc = rescale(x)) return rc;
      } else {
        const double scf1 = x.scale, scf2 = C.big[l2 + 1], scf = C.sf[l1], q1 = C.mrf[l1];
        if (int rc = mult_const(x, scf2 / scf1 * q1 / scf)) return rc;
        x.scale = C.big[x.t - 2] * C.mrf[l1];
        if (int rc = rescale(x)) return rc;
        if (x.t - 2 > l2)
          if (int rc = drop(x, l2 + 2)) return rc;
        x.scale = C.big[x.t - 1];
        if (int rc = rescale(x)) return rc;
        x.scale = scale2;
      }
    } else {
      if (deg2 == 2) {
        const double scf1 = x.scale, scf = C.sf[l1];
        if (int rc = mult_const(x, scale2 / scf1 / scf)) return rc;
        if (int rc = drop(x, l2 + 1)) return rc;
        x.scale = scale2;
      } else {
        const double scf1 = x.scale, scf2 = C.big[l2 + 1], scf = C.sf[l1];
        if (int rc = mult_const(x, scf2 / scf1 / scf)) return rc;
        if (l1 - 1 > l2)
          if (int rc = drop(x, l2 + 2)) return rc;
        x.scale *= scf2 / scf1 / scf;
        if (int rc = rescale(x)) return rc;
        x.scale = scale2;
      }
    }
    return FIDES_OK;
  }
  if (l1 < l2) {
    *ok = false;
    return FIDES_OK;
  }
  if (d1 < deg2) return mult_const(x, 1.0);
  if (deg2 < d1) *ok = false;
  return FIDES_OK;
}

int AutoScaler::for_add(DevCt& x, const DevCt& y, bool* ok) {
  // Ciphertext::adjustForAddOrSub.
  *ok = true;
  if (c_->technique == FIDES_FLEXIBLEAUTO || c_->technique == FIDES_FLEXIBLEAUTOEXT)
    return scale_and_level(x, y.noise_deg, y.t, y.scale, ok);
  if ((x.t - 1) - x.noise_deg > (y.t - 1) - y.noise_deg) {
    if (y.noise_deg == 1 && x.noise_deg == 2) return rescale(x);
    if (y.noise_deg == 2 && x.noise_deg == 1) return mult_const(x, 1.0);
    return FIDES_OK;
  }
  if (y.noise_deg == 1 && x.noise_deg == 2) return rescale(x);
  if (x.noise_deg == 1 && y.noise_deg == 2) *ok = false;
  return FIDES_OK;
}

int AutoScaler::for_mult(DevCt& x, const DevCt& y, bool* ok) {
  // Ciphertext::adjustForMult.
  bool add_ok = true;
  if (int rc = for_add(x, y, &add_ok)) return rc;
  if (x.noise_deg == 2)
    if (int rc = rescale(x)) return rc;
  *ok = add_ok && y.noise_deg != 2;
  return FIDES_OK;
}

int AutoScaler::align(int op, DevCt& a, DevCt& b) {
  // The reference's add / sub / mult: adjust `a` against `b`; when that reports the roles reversed, adjust a copy
  // of `b` against the (already adjusted) `a` and retry, until both sides agree (at most a few rounds).
  const bool mult = op == FIDES_OP_MULT;
  for (int round = 0; round < 4; round++) {
    bool ok = true;
    if (int rc = mult ? for_mult(a, b, &ok) : for_add(a, b, &ok)) return rc;
    if (ok) break;
    bool ok_b = true;
    if (int rc = mult ? for_mult(b, a, &ok_b) : for_add(b, a, &ok_b)) return rc;
    if (!ok_b) return set_last_error(FIDES_EINVAL, "operands cannot be brought to one level and scale");
  }
  if (c_->technique == FIDES_FLEXIBLEAUTO || c_->technique == FIDES_FLEXIBLEAUTOEXT) {
    if (a.t != b.t) return set_last_error(FIDES_EINVAL, "automatic rescaling left the operands at different levels");
  }
  return FIDES_OK;
}

int AutoScaler::prepare_binary(int op, DevCt& a, DevCt& b) {
  if (c_->technique != FIDES_FIXEDMANUAL)
    if (int rc = align(op, a, b)) return rc;
  // FIXEDMANUAL (and the FIXEDAUTO tail): the operand with more towers is cut down to the other's level.
  if (a.t > b.t) return drop(a, b.t);
  if (b.t > a.t) return drop(b, a.t);
  return FIDES_OK;
}

int AutoScaler::prepare_unary(DevCt& a) {
  // Square, scalar and plaintext products: an automatic technique first rescales a degree-2 ciphertext.
  if (c_->technique != FIDES_FIXEDMANUAL && a.noise_deg >= 2) return rescale(a);
  return FIDES_OK;
}

}  // namespace fgb
