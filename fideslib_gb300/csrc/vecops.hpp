// Lock-step evaluation helpers: each call applies one engine op to a vector of ciphertext handles, as one
// batch (fides_eval_batch / fides_eval_linear_transform_batch) where the op has a batched form and as a loop
// of elementwise launches otherwise.  Used by the composite routines (polynomial evaluation, bootstrapping) so
// that n ciphertexts go through the same recipe together.  Every handle an op creates is owned by the Scope
// and freed when it ends, unless released to the caller.
#pragma once

#include <algorithm>
#include <vector>

#include "../../include/fideslib_gb300.h"

namespace fgb {
int set_last_error(int code, const char* msg);
}

namespace fgb::vec {

using V = std::vector<uint32_t>;

#define FGB_TRY(x)                       \
  do {                                   \
    const int rc_ = (x);                 \
    if (rc_ != FIDES_OK) return rc_;     \
  } while (0)

struct Scope {
  fides_ctx* ctx;
  std::vector<uint32_t> owned;
  explicit Scope(fides_ctx* c) : ctx(c) {}
  Scope(const Scope&) = delete;
  Scope& operator=(const Scope&) = delete;
  ~Scope() {
    for (uint32_t h : owned)
      if (h) fides_ct_free(ctx, h);
  }
  void keep(const V& v) { owned.insert(owned.end(), v.begin(), v.end()); }
  void release(const V& v) {
    for (auto& x : owned)
      if (std::find(v.begin(), v.end(), x) != v.end()) x = 0;
  }
};

inline uint32_t towers_of(fides_ctx* ctx, uint32_t h) {
  fides_ct_meta m{};
  fides_ct_meta_get(ctx, h, &m);
  return m.towers;
}

inline double scale_of(fides_ctx* ctx, uint32_t h) {
  fides_ct_meta m{};
  fides_ct_meta_get(ctx, h, &m);
  return m.scale;
}

}  // namespace fgb::vec
namespace fgb {
// fides_eval_batch without the scaling technique's operand alignment (capi.cu).
int eval_batch_exact(fides_ctx* ctx, fides_op* ops, uint32_t n);
}  // namespace fgb
namespace fgb::vec {

// One batched op over a (and b, element-wise); outputs kept by the scope.  The composites keep their operands at
// matching levels and scales themselves, so the batch skips the scaling technique's alignment.
inline int batch(Scope& sc, int32_t op, const V& a, const V* b, int32_t index, V& out) {
  std::vector<fides_op> ops(a.size());
  for (size_t i = 0; i < a.size(); i++) ops[i] = fides_op{op, a[i], b ? (*b)[i] : 0u, index, 0u};
  FGB_TRY(eval_batch_exact(sc.ctx, ops.data(), (uint32_t)ops.size()));
  out.resize(a.size());
  for (size_t i = 0; i < a.size(); i++) out[i] = ops[i].out;
  sc.keep(out);
  return FIDES_OK;
}

inline int add(Scope& sc, const V& a, const V& b, V& out) { return batch(sc, FIDES_OP_ADD, a, &b, 0, out); }
inline int sub(Scope& sc, const V& a, const V& b, V& out) { return batch(sc, FIDES_OP_SUB, a, &b, 0, out); }
inline int mult(Scope& sc, const V& a, const V& b, V& out) { return batch(sc, FIDES_OP_MULT, a, &b, 0, out); }
inline int square(Scope& sc, const V& a, V& out) { return batch(sc, FIDES_OP_SQUARE, a, nullptr, 0, out); }
inline int rescale(Scope& sc, const V& a, V& out) { return batch(sc, FIDES_OP_RESCALE, a, nullptr, 0, out); }
inline int rotate(Scope& sc, const V& a, int32_t index, V& out) {
  return batch(sc, FIDES_OP_ROTATE, a, nullptr, index, out);
}
inline int automorphism(Scope& sc, const V& a, uint32_t galois, V& out) {
  return batch(sc, FIDES_OP_AUTOMORPHISM, a, nullptr, (int32_t)galois, out);
}
inline int key_switch(Scope& sc, const V& a, uint32_t key_id, V& out) {
  return batch(sc, FIDES_OP_KEY_SWITCH, a, nullptr, (int32_t)key_id, out);
}

// Elementwise ops: one launch per ciphertext.
template <class F>
inline int each(Scope& sc, const V& a, V& out, F f) {
  out.assign(a.size(), 0);
  for (size_t i = 0; i < a.size(); i++) {
    const int rc = f(i, &out[i]);
    if (rc != FIDES_OK) {
      sc.keep(out);
      return rc;
    }
  }
  sc.keep(out);
  return FIDES_OK;
}
// Scalar ops: one many-to-one call (one launch) for the whole vector; element i uses v[i] (and scale[i]).
inline int scalar_batch(Scope& sc, int32_t op, const V& a, const std::vector<double>& v,
                        const std::vector<double>* scale, V& out) {
  out.assign(a.size(), 0);
  if (a.empty()) return FIDES_OK;
  FGB_TRY(fides_eval_many_to_one(sc.ctx, op, (uint32_t)a.size(), 1, a.data(), nullptr, v.data(),
                                 scale ? scale->data() : nullptr, out.data()));
  sc.keep(out);
  return FIDES_OK;
}
inline int mult_scalar(Scope& sc, const V& a, const std::vector<double>& v, double scale, V& out) {
  const std::vector<double> s(a.size(), scale);
  return scalar_batch(sc, FIDES_OP_MULT_SCALAR, a, v, &s, out);
}
inline int mult_scalar(Scope& sc, const V& a, double v, double scale, V& out) {
  return mult_scalar(sc, a, std::vector<double>(a.size(), v), scale, out);
}
// Per-element constant scales: element i gets round(v * scale[i]) and scale *= scale[i].
inline int mult_scalar_at(Scope& sc, const V& a, double v, const std::vector<double>& scale, V& out) {
  return scalar_batch(sc, FIDES_OP_MULT_SCALAR, a, std::vector<double>(a.size(), v), &scale, out);
}
inline int add_scalar(Scope& sc, const V& a, double v, V& out) {
  return scalar_batch(sc, FIDES_OP_ADD_SCALAR, a, std::vector<double>(a.size(), v), nullptr, out);
}
inline int mult_int(Scope& sc, const V& a, int64_t k, V& out) {
  return scalar_batch(sc, FIDES_OP_MULT_INT, a, std::vector<double>(a.size(), (double)k), nullptr, out);
}
inline int monomial(Scope& sc, const V& a, uint32_t k, V& out) {
  return each(sc, a, out, [&](size_t i, uint32_t* o) { return fides_eval_mult_monomial(sc.ctx, a[i], k, o); });
}
inline int mod_raise(Scope& sc, const V& a, uint32_t towers, V& out) {
  return each(sc, a, out, [&](size_t i, uint32_t* o) { return fides_mod_raise(sc.ctx, a[i], towers, o); });
}

// a[i] dropped to t[i] towers; elements already there are passed through (not owned twice).
inline int drop_to(Scope& sc, const V& a, const std::vector<uint32_t>& t, V& out) {
  out.assign(a.size(), 0);
  for (size_t i = 0; i < a.size(); i++) {
    if (towers_of(sc.ctx, a[i]) == t[i]) {
      out[i] = a[i];
      continue;
    }
    FGB_TRY(fides_level_reduce(sc.ctx, a[i], t[i], &out[i]));
    sc.keep(V{out[i]});
  }
  return FIDES_OK;
}

// out[i] = sum_k round(w[k] * scale[k][i]) * terms[k][i] on the smallest tower count of element i's terms, one
// weighted-sum launch per 64 elements (fides_eval_linear_wsum); the result has the scale of terms[0][i] times
// scale[0][i] and noise degree 2.
inline int wsum(Scope& sc, const std::vector<V>& terms, const std::vector<double>& w,
                const std::vector<std::vector<double>>& scale, V& out) {
  const size_t n = terms.size(), m = terms[0].size();
  std::vector<uint32_t> cts(n * m);
  std::vector<double> s(n * m);
  for (size_t k = 0; k < n; k++)
    for (size_t i = 0; i < m; i++) {
      cts[k * m + i] = terms[k][i];
      s[k * m + i] = scale[k][i];
    }
  out.assign(m, 0);
  FGB_TRY(fides_eval_linear_wsum(sc.ctx, (uint32_t)m, (uint32_t)n, cts.data(), w.data(), s.data(), out.data()));
  sc.keep(out);
  return FIDES_OK;
}

inline std::vector<double> scales(fides_ctx* ctx, const V& a) {
  std::vector<double> s(a.size());
  for (size_t i = 0; i < a.size(); i++) s[i] = scale_of(ctx, a[i]);
  return s;
}

inline std::vector<uint32_t> towers(fides_ctx* ctx, const V& a) {
  std::vector<uint32_t> t(a.size());
  for (size_t i = 0; i < a.size(); i++) t[i] = towers_of(ctx, a[i]);
  return t;
}

inline int linear_transform(Scope& sc, const V& a, uint32_t lt, V& out) {
  out.assign(a.size(), 0);
  FGB_TRY(fides_eval_linear_transform_batch(sc.ctx, (uint32_t)a.size(), a.data(), lt, out.data()));
  sc.keep(out);
  return FIDES_OK;
}

}  // namespace fgb::vec
