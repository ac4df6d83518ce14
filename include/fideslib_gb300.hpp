// fideslib_gb300 — C++ host facade over the C ABI (include/fideslib_gb300.h).
//
// Mirrors the method names and argument meaning of the reference's fideslib::CryptoContextImpl<DCRTPoly>
// (api/CryptoContext.hpp:43-203) for the evaluation hot path, on raw residues instead of OpenFHE objects:
// LoadContext (the constructor), LoadCiphertext / LoadPlaintext, EvalAdd / EvalSub / EvalMult / EvalSquare,
// EvalRotate, EvalFastRotationPrecompute / EvalFastRotation / EvalFastRotationExt + KeySwitchDown, the *InPlace
// forms, Rescale, EvalChebyshevSeries, EvalBootstrap, Synchronize.  Like the reference API it reports failures by
// throwing (fideslib_gb300::Error carries the C status code and message); the C ABI
// underneath never throws or exits.  Ciphertext is a shared, reference-counted device handle
// (the reference's Ciphertext<DCRTPoly> is a shared_ptr, api/Ciphertext.hpp:13-58).
#pragma once

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "fideslib_gb300.h"

namespace fideslib_gb300 {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

inline void check(int rc) {
  if (rc != FIDES_OK) throw Error(rc, fides_last_error());
}

struct Params {
  uint32_t log_n = 16;
  std::vector<uint64_t> q;  // Q primes (OpenFHE moduli)
  std::vector<uint64_t> p;  // special primes
  uint32_t dnum = 3;
  std::vector<uint64_t> roots;  // optional primitive 2N-th roots for q then p (OpenFHE root_of_unity)
  int32_t scaling_technique = FIDES_FIXEDMANUAL;
  // RawParams' per-level tables (ScalingFactorReal, ScalingFactorRealBig, ModReduceFactor), indexed by towers - 1;
  // empty = computed for the technique.
  std::vector<double> scaling_factor_real, scaling_factor_real_big, mod_reduce_factor;
  double default_scale = 0;
};

// The `count` largest primes < 2^bits with p == 1 mod 2N (for building synthetic parameter sets).
inline std::vector<uint64_t> FindPrimes(uint32_t bits, uint32_t count, uint32_t log_n,
                                        const std::vector<uint64_t>& exclude = {}) {
  std::vector<uint64_t> out(count);
  const int n = fides_find_primes(bits, count, 2ull << log_n, exclude.data(), (uint32_t)exclude.size(), out.data());
  if (n != (int)count) throw Error(FIDES_EINVAL, "not enough primes of the requested size");
  return out;
}

class CryptoContext;

class Ciphertext {
 public:
  Ciphertext() = default;
  uint32_t handle() const { return h_ ? h_->id : 0; }
  explicit operator bool() const { return (bool)h_; }
  fides_ct_meta Meta() const {
    fides_ct_meta m{};
    check(fides_ct_meta_get(h_->ctx, h_->id, &m));
    return m;
  }
  uint32_t GetTowers() const { return Meta().towers; }
  uint32_t GetNoiseScaleDeg() const { return Meta().noise_deg; }
  double GetScalingFactor() const { return Meta().scale; }

 private:
  friend class CryptoContext;
  struct Handle {
    Handle(fides_ctx* c, uint32_t i) : ctx(c), id(i) {}
    Handle(const Handle&) = delete;
    Handle& operator=(const Handle&) = delete;
    ~Handle() { fides_ct_free(ctx, id); }
    fides_ctx* ctx;
    uint32_t id;
  };
  Ciphertext(fides_ctx* ctx, uint32_t id) : h_(std::make_shared<Handle>(ctx, id)) {}
  std::shared_ptr<Handle> h_;
};

class Plaintext {
 public:
  Plaintext() = default;
  uint32_t handle() const { return h_ ? h_->id : 0; }

 private:
  friend class CryptoContext;
  struct Handle {
    Handle(fides_ctx* c, uint32_t i) : ctx(c), id(i) {}
    Handle(const Handle&) = delete;
    Handle& operator=(const Handle&) = delete;
    ~Handle() { fides_pt_free(ctx, id); }
    fides_ctx* ctx;
    uint32_t id;
  };
  Plaintext(fides_ctx* ctx, uint32_t id) : h_(std::make_shared<Handle>(ctx, id)) {}
  std::shared_ptr<Handle> h_;
};

// A ciphertext in the extended basis Q_t ∪ P (EvalFastRotationExt's result, consumed by KeySwitchDown).
class ExtCiphertext {
 public:
  ExtCiphertext() = default;
  uint32_t handle() const { return h_ ? h_->id : 0; }

 private:
  friend class CryptoContext;
  struct Handle {
    Handle(fides_ctx* c, uint32_t i) : ctx(c), id(i) {}
    Handle(const Handle&) = delete;
    Handle& operator=(const Handle&) = delete;
    ~Handle() { fides_ct_free(ctx, id); }
    fides_ctx* ctx;
    uint32_t id;
  };
  ExtCiphertext(fides_ctx* ctx, uint32_t id) : h_(std::make_shared<Handle>(ctx, id)) {}
  std::shared_ptr<Handle> h_;
};

// EvalFastRotationPrecompute's result (the reference returns a shared_ptr<void>, api/CryptoContext.hpp:169).
class Precomputation {
 public:
  Precomputation() = default;
  uint32_t handle() const { return h_ ? h_->id : 0; }

 private:
  friend class CryptoContext;
  struct Handle {
    Handle(fides_ctx* c, uint32_t i) : ctx(c), id(i) {}
    Handle(const Handle&) = delete;
    Handle& operator=(const Handle&) = delete;
    ~Handle() { fides_precompute_free(ctx, id); }
    fides_ctx* ctx;
    uint32_t id;
  };
  Precomputation(fides_ctx* ctx, uint32_t id) : h_(std::make_shared<Handle>(ctx, id)) {}
  std::shared_ptr<Handle> h_;
};

class CryptoContext {
 public:
  // LoadContext: moduli, roots and all derived tables to the device.
  explicit CryptoContext(const Params& prm) {
    std::vector<uint64_t> mods(prm.q);
    mods.insert(mods.end(), prm.p.begin(), prm.p.end());
    auto opt = [](const std::vector<double>& v) { return v.empty() ? nullptr : v.data(); };
    fides_params p{prm.log_n, (uint32_t)prm.q.size(), (uint32_t)prm.p.size(), prm.dnum, mods.data(),
                   prm.roots.empty() ? nullptr : prm.roots.data(), prm.scaling_technique,
                   opt(prm.scaling_factor_real), opt(prm.scaling_factor_real_big), opt(prm.mod_reduce_factor),
                   prm.default_scale};
    check(fides_ctx_create(&p, &ctx_));
    N_ = 1u << prm.log_n;
  }
  ~CryptoContext() { fides_ctx_destroy(ctx_); }
  CryptoContext(const CryptoContext&) = delete;
  CryptoContext& operator=(const CryptoContext&) = delete;

  fides_ctx* raw() const { return ctx_; }
  uint32_t GetRingDimension() const { return N_; }
  uint32_t GetCyclotomicOrder() const { return 2 * N_; }

  // Keys: u64[2][dnum][nq+np][N] (RawKeySwitchKey::r_key layout).
  void LoadEvalMultKey(const uint64_t* key) { check(fides_load_eval_mult_key(ctx_, key)); }
  void LoadRotationKey(int32_t index, const uint64_t* key) {
    check(fides_load_rotation_key(ctx_, fides_galois_element(ctx_, index), key));
  }
  void LoadConjugationKey(const uint64_t* key) { check(fides_load_rotation_key(ctx_, 2 * N_ - 1, key)); }

  // LoadCiphertext: u64[2][towers][N] evaluation form.
  Ciphertext LoadCiphertext(const uint64_t* data, uint32_t towers, double scale, uint32_t noise_deg = 1,
                            uint32_t slots = 0) {
    fides_ct_meta m{towers, noise_deg, slots, 0, scale};
    uint32_t h;
    check(fides_ct_load(ctx_, data, &m, &h));
    return Ciphertext(ctx_, h);
  }
  std::vector<uint64_t> StoreCiphertext(const Ciphertext& ct) {
    std::vector<uint64_t> out((size_t)2 * ct.GetTowers() * N_);
    check(fides_ct_store(ctx_, ct.handle(), out.data(), nullptr));
    return out;
  }
  Plaintext LoadPlaintext(const uint64_t* data, uint32_t towers, double scale) {
    uint32_t h;
    check(fides_pt_load(ctx_, data, towers, scale, &h));
    return Plaintext(ctx_, h);
  }

  Ciphertext EvalAdd(const Ciphertext& a, const Ciphertext& b) { return bin(fides_eval_add, a, b); }
  Ciphertext EvalSub(const Ciphertext& a, const Ciphertext& b) { return bin(fides_eval_sub, a, b); }
  Ciphertext EvalMult(const Ciphertext& a, const Ciphertext& b) { return bin(fides_eval_mult, a, b); }
  Ciphertext EvalMult(const Ciphertext& a, const Plaintext& p) { return wrap(fides_eval_mult_plain(ctx_, a.handle(), p.handle(), &tmp_)); }
  Ciphertext EvalAdd(const Ciphertext& a, const Plaintext& p) { return wrap(fides_eval_add_plain(ctx_, a.handle(), p.handle(), &tmp_)); }
  Ciphertext EvalMult(const Ciphertext& a, double v, double scale) {
    return wrap(fides_eval_mult_scalar(ctx_, a.handle(), v, scale, &tmp_));
  }
  Ciphertext EvalAdd(const Ciphertext& a, double v) { return wrap(fides_eval_add_scalar(ctx_, a.handle(), v, &tmp_)); }
  Ciphertext EvalSquare(const Ciphertext& a) { return wrap(fides_eval_square(ctx_, a.handle(), &tmp_)); }
  Ciphertext Rescale(const Ciphertext& a) { return wrap(fides_rescale(ctx_, a.handle(), &tmp_)); }
  Ciphertext EvalRotate(const Ciphertext& a, int32_t index) {
    return wrap(fides_eval_rotate(ctx_, a.handle(), index, &tmp_));
  }
  // EvalFastRotation (hoisted): one ModUp shared by every index.
  std::vector<Ciphertext> EvalFastRotation(const Ciphertext& a, const std::vector<int32_t>& indices) {
    std::vector<uint32_t> outs(indices.size());
    check(fides_eval_fast_rotation(ctx_, a.handle(), (uint32_t)indices.size(), indices.data(), outs.data()));
    std::vector<Ciphertext> r;
    for (uint32_t h : outs) r.push_back(Ciphertext(ctx_, h));
    return r;
  }
  Precomputation EvalFastRotationPrecompute(const Ciphertext& a) {
    uint32_t h;
    check(fides_fast_rotation_precompute(ctx_, a.handle(), &h));
    return Precomputation(ctx_, h);
  }
  // EvalFastRotation(ct, index, m, precomp): m (the cyclotomic order) is implied by the context.
  Ciphertext EvalFastRotation(const Ciphertext& a, int32_t index, uint32_t /*m*/, const Precomputation& pre) {
    return wrap(fides_eval_fast_rotation_precomputed(ctx_, a.handle(), pre.handle(), index, &tmp_));
  }
  // EvalFastRotationExt (api/CryptoContext.cpp:1497-1617): the rotations left in the extended basis, with or
  // without P * c0; products with plaintexts loaded by LoadPlaintextExt and sums stay there; KeySwitchDown ends.
  std::vector<ExtCiphertext> EvalFastRotationExt(const Ciphertext& a, const std::vector<int32_t>& indices,
                                                 const Precomputation& pre, bool addFirst) {
    std::vector<uint32_t> h(indices.size());
    check(fides_eval_fast_rotation_ext(ctx_, a.handle(), pre.handle(), (uint32_t)indices.size(), indices.data(),
                                       addFirst ? 1 : 0, h.data()));
    std::vector<ExtCiphertext> out;
    for (uint32_t x : h) out.push_back(ExtCiphertext(ctx_, x));
    return out;
  }
  ExtCiphertext EvalFastRotationExt(const Ciphertext& a, int32_t index, const Precomputation& pre, bool addFirst) {
    return EvalFastRotationExt(a, std::vector<int32_t>{index}, pre, addFirst)[0];
  }
  // data = u64[towers + np][N]: the Q rows, then the special-prime rows.
  Plaintext LoadPlaintextExt(const uint64_t* data, uint32_t towers, double scale) {
    uint32_t h;
    check(fides_pt_load_ext(ctx_, data, towers, scale, &h));
    return Plaintext(ctx_, h);
  }
  ExtCiphertext EvalMult(const ExtCiphertext& a, const Plaintext& pt) {
    check(fides_ext_mult_plain(ctx_, a.handle(), pt.handle(), &tmp_));
    return ExtCiphertext(ctx_, tmp_);
  }
  ExtCiphertext EvalAdd(const ExtCiphertext& a, const ExtCiphertext& b) {
    check(fides_ext_add(ctx_, a.handle(), b.handle(), &tmp_));
    return ExtCiphertext(ctx_, tmp_);
  }
  Ciphertext KeySwitchDown(const ExtCiphertext& a) { return wrap(fides_key_switch_down(ctx_, a.handle(), &tmp_)); }
  // In-place forms (EvalAddInPlace, EvalMultInPlace, EvalSquareInPlace, RescaleInPlace, EvalRotateInPlace): the
  // handle is replaced by the result's.
  void EvalAddInPlace(Ciphertext& a, const Ciphertext& b) { a = EvalAdd(a, b); }
  void EvalSubInPlace(Ciphertext& a, const Ciphertext& b) { a = EvalSub(a, b); }
  void EvalMultInPlace(Ciphertext& a, const Ciphertext& b) { a = EvalMult(a, b); }
  void EvalSquareInPlace(Ciphertext& a) { a = EvalSquare(a); }
  void RescaleInPlace(Ciphertext& a) { a = Rescale(a); }
  void EvalRotateInPlace(Ciphertext& a, int32_t index) { a = EvalRotate(a, index); }
  Ciphertext EvalChebyshevSeries(const Ciphertext& a, const std::vector<double>& coeffs, double lo, double hi,
                                 double const_scale) {
    return wrap(fides_eval_chebyshev(ctx_, a.handle(), coeffs.data(), (uint32_t)coeffs.size(), lo, hi, const_scale,
                                     &tmp_));
  }
  Ciphertext EvalBootstrap(const Ciphertext& a, const fides_bootstrap_plan& plan) {
    return wrap(fides_eval_bootstrap(ctx_, a.handle(), &plan, &tmp_));
  }
  void Synchronize() { check(fides_synchronize(ctx_)); }

 private:
  Ciphertext wrap(int rc) {
    check(rc);
    return Ciphertext(ctx_, tmp_);
  }
  template <class F>
  Ciphertext bin(F f, const Ciphertext& a, const Ciphertext& b) {
    return wrap(f(ctx_, a.handle(), b.handle(), &tmp_));
  }
  fides_ctx* ctx_ = nullptr;
  uint32_t N_ = 0;
  uint32_t tmp_ = 0;
};

}  // namespace fideslib_gb300
