// Polynomial evaluation on ciphertexts: EvalChebyshevSeries and the double-angle iterations of EvalMod.
//
// Reference counterparts: CryptoContextImpl::EvalChebyshevSeries (api/CryptoContext.hpp:154-156),
// FIDESlib's Chebyshev Paterson–Stockmeyer evaluation and double-angle loop (src/CKKS/ApproxModEval.cu:
// 138-370, 724-739).  The series is evaluated in baby-step/giant-step form (Paterson–Stockmeyer over the
// Chebyshev basis), every step one engine op so that the whole sequence replays op-for-op on a CPU
// restatement:
//   y    = x                                  when [lo, hi] = [-1, 1]
//        = Rescale(x * (2/(hi-lo))) - (hi+lo)/(hi-lo)   otherwise (constant encoded at const_scale)
//   T_1  = y; baby steps T_2 .. T_bs, bs = 2^max(1, round(log2(d+1)/2)), by
//          T_k = Rescale(T_{k/2}^2) * 2 - 1 (k even),
//          T_k = Rescale(T_a * T_b) * 2 - T_1' (k odd, a = (k-1)/2, b = (k+1)/2, operands dropped to the
//                smaller tower count; T_1' = Rescale(T_1 * 1), T_1 dropped to one tower above the product and
//                the 1 encoded at the scale that gives T_1' exactly the product's scale);
//   giant steps T_{bs 2^i} = Rescale(T_{bs 2^(i-1)}^2) * 2 - 1 while bs 2^i <= d;
//   p    = the coefficients (zero-padded to bs 2^m) split recursively by Chebyshev division at M = bs 2^(i-1)
//          (node()); each part is evaluated at a target scale chosen so that every addition adds equal scales:
//          a leaf sum_{k<bs} c_k T_k is Rescale(sum T_k * c_k) with c_k encoded at target * q_drop / scale(T_k)
//          (one weighted sum over the terms at their smallest tower count); the top-level target is the scale of
//          T_1, so the result keeps the input's scale; the constant of the series is added last.
// Non-scalar products for degree d: bs - 1 + (m - 1) + (2^m - 1) (16 for d = 47, against 46 for the full
// T_1 .. T_d ladder).  Exact scale matching is what OpenFHE's FLEXIBLEAUTO mode does; without it sums of
// terms whose scales differ by the primes' distance from the nominal scale carry that relative error, which the
// division's larger intermediate terms amplify.  The *_batch forms run m ciphertexts through the recipe in lock
// step, one batched launch per step; each result is the same as the single-ciphertext call's.
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

// x and y dropped to their common (smaller) tower count.
int align(Scope& sc, const V& x, const V& y, V& xd, V& yd) {
  std::vector<uint32_t> t = fgb::vec::towers(sc.ctx, x), ty = fgb::vec::towers(sc.ctx, y);
  for (size_t i = 0; i < t.size(); i++) t[i] = std::min(t[i], ty[i]);
  FGB_TRY(fgb::vec::drop_to(sc, x, t, xd));
  return fgb::vec::drop_to(sc, y, t, yd);
}

// Everything below keeps the scales of added ciphertexts identical (the FLEXIBLEAUTO treatment): wherever two
// ciphertexts meet in an addition, the constant multiplied into one of them is encoded at the scale that makes
// its result's scale equal the other's, so no sum carries a scale mismatch.
struct Poly {
  fides_ctx* ctx;
  Scope& sc;
  std::vector<double> q;  // moduli as doubles
  std::vector<V> T, G;    // baby steps T_1..T_top (T[0] unused), giant steps T_{bs 2^i}
  double cs;
};

using Towers = std::vector<int>;  // per element, -1 = no ciphertext part

// T_k from the lower ones: 2 Rescale(T_{k/2}^2) - 1 (k even);  2 Rescale(T_a T_b) - T_1' (k odd, a = (k-1)/2,
// b = (k+1)/2, operands dropped to the smaller tower count), T_1' = Rescale(T_1 * 1) with the constant 1
// encoded at the scale that gives T_1' the product's scale (T_1 first dropped to one tower above it).
int next_t(Poly& P, int k, V& out) {
  Scope& sc = P.sc;
  const std::vector<V>& T = P.T;
  V prod, r, m2;
  if (k % 2 == 0) {
    FGB_TRY(fgb::vec::square(sc, T[k / 2], prod));
    return double_and_shift(sc, prod, nullptr, out);
  }
  V Ad, Bd;
  FGB_TRY(align(sc, T[(k - 1) / 2], T[(k + 1) / 2], Ad, Bd));
  FGB_TRY(fgb::vec::mult(sc, Ad, Bd, prod));
  FGB_TRY(fgb::vec::rescale(sc, prod, r));
  FGB_TRY(fgb::vec::mult_int(sc, r, 2, m2));
  const std::vector<uint32_t> tm = fgb::vec::towers(P.ctx, m2);
  std::vector<uint32_t> up(tm.size());
  for (size_t i = 0; i < tm.size(); i++) up[i] = tm[i] + 1;
  V t1d, t1s, t1r;
  FGB_TRY(fgb::vec::drop_to(sc, T[1], up, t1d));
  const std::vector<double> sm = fgb::vec::scales(P.ctx, m2), s1 = fgb::vec::scales(P.ctx, t1d);
  std::vector<double> f(tm.size());
  for (size_t i = 0; i < tm.size(); i++) f[i] = sm[i] * P.q[tm[i]] / s1[i];
  FGB_TRY(fgb::vec::mult_scalar_at(sc, t1d, 1.0, f, t1s));
  FGB_TRY(fgb::vec::rescale(sc, t1s, t1r));
  return fgb::vec::sub(sc, m2, t1r, out);
}

// Tower counts a leaf / node result will have (tower counts do not depend on scales).
Towers leaf_towers(const Poly& P, const double* c, int bs) {
  const size_t m = P.T[1].size();
  Towers t(m, -1);
  for (int k = 1; k < bs; k++) {
    if (c[k] == 0.0) continue;
    const std::vector<uint32_t> tk = fgb::vec::towers(P.ctx, P.T[k]);
    for (size_t i = 0; i < m; i++) t[i] = t[i] < 0 ? (int)tk[i] : std::min(t[i], (int)tk[i]);
  }
  for (auto& x : t)
    if (x >= 0) x -= 1;
  return t;
}

void split(const std::vector<double>& c, std::vector<double>& q, std::vector<double>& r) {
  const size_t M = c.size() / 2;
  q.assign(M, 0.0);
  r.assign(c.begin(), c.begin() + M);
  q[0] = c[M];
  for (size_t j = 1; j < M; j++) {
    q[j] = 2.0 * c[M + j];
    r[M - j] -= c[M + j];
  }
}

bool has_terms(const std::vector<double>& c) {
  for (size_t k = 1; k < c.size(); k++)
    if (c[k] != 0.0) return true;
  return false;
}

Towers node_towers(const Poly& P, const std::vector<double>& c, int i) {
  const int bs = (int)(c.size() >> i);
  if (i == 0) return leaf_towers(P, c.data(), bs);
  std::vector<double> q, r;
  split(c, q, r);
  const Towers tq = node_towers(P, q, i - 1), tr = node_towers(P, r, i - 1);
  const std::vector<uint32_t> tg = fgb::vec::towers(P.ctx, P.G[i - 1]);
  Towers t(tq.size());
  for (size_t e = 0; e < t.size(); e++) {
    int tp = -1;
    if (tq[e] >= 0) tp = std::min(tq[e], (int)tg[e]) - 1;
    else if (q[0] != 0.0) tp = (int)tg[e] - 1;
    t[e] = tp < 0 ? tr[e] : (tr[e] < 0 ? tp : std::min(tp, tr[e]));
  }
  return t;
}

// A partial result: ct + c (ct empty: the constant c alone).
struct Part {
  V ct;
  double c = 0.0;
};

// sum_{k<bs} c_k T_k at scale `target`: Rescale(sum T_k * c_k over k >= 1, c_k != 0), term k's constant encoded at
// target * q_drop / scale(T_k) (q_drop = the prime the rescale removes), the terms read at their smallest tower
// count and summed by one weighted-sum launch (the reference evaluates the same leaf with evalLinearWSumMutable,
// src/CKKS/ApproxModEval.cu:213); c_0 kept aside.
int leaf(Poly& P, const double* c, int bs, const std::vector<double>& target, Part& out) {
  const Towers tl = leaf_towers(P, c, bs);
  std::vector<V> terms;
  std::vector<double> w;
  std::vector<std::vector<double>> f;
  for (int k = 1; k < bs; k++) {
    if (c[k] == 0.0) continue;
    const std::vector<double> sk = fgb::vec::scales(P.ctx, P.T[k]);
    std::vector<double> fk(sk.size());
    for (size_t e = 0; e < fk.size(); e++) fk[e] = target[e] * P.q[tl[e]] / sk[e];
    terms.push_back(P.T[k]);
    w.push_back(c[k]);
    f.push_back(std::move(fk));
  }
  out.ct.clear();
  if (!terms.empty()) {
    V acc;
    FGB_TRY(fgb::vec::wsum(P.sc, terms, w, f, acc));
    FGB_TRY(fgb::vec::rescale(P.sc, acc, out.ct));
  }
  out.c = c[0];
  return FIDES_OK;
}

// p = sum_{k < bs 2^i} c_k T_k = q T_M + r with M = bs 2^(i-1) (T_{M+j} = 2 T_M T_j - T_{M-j}):
// q = c_M + sum_{j>=1} 2 c_{M+j} T_j,  r = sum_{k<M} c_k T_k - sum_{j>=1} c_{M+j} T_{M-j}.
// Result (scale `target`) = Rescale(q' * T_M) + r, q' = q with its constant folded in and evaluated at the scale
// that makes the product's scale `target` (q a constant alone: T_M * q_0 with that constant scale), r evaluated
// at `target`; operands level-aligned by dropping towers; the constant of r stays aside.
int node(Poly& P, const std::vector<double>& c, int i, const std::vector<double>& target, Part& out) {
  const int bs = (int)(c.size() >> i);
  if (i == 0) return leaf(P, c.data(), bs, target, out);
  std::vector<double> q, r;
  split(c, q, r);
  const V& Gm = P.G[i - 1];
  const std::vector<uint32_t> tg = fgb::vec::towers(P.ctx, Gm);
  const std::vector<double> sg = fgb::vec::scales(P.ctx, Gm);
  const size_t m = target.size();
  V prod;
  if (has_terms(q)) {
    const Towers tq = node_towers(P, q, i - 1);
    std::vector<double> tgt(m);
    for (size_t e = 0; e < m; e++) tgt[e] = target[e] * P.q[std::min(tq[e], (int)tg[e]) - 1] / sg[e];
    Part Q;
    FGB_TRY(node(P, q, i - 1, tgt, Q));
    V X = Q.ct;
    if (Q.c != 0.0) FGB_TRY(fgb::vec::add_scalar(P.sc, Q.ct, Q.c, X));
    V Xd, Gd, pr;
    FGB_TRY(align(P.sc, X, Gm, Xd, Gd));
    FGB_TRY(fgb::vec::mult(P.sc, Xd, Gd, pr));
    FGB_TRY(fgb::vec::rescale(P.sc, pr, prod));
  } else if (q[0] != 0.0) {
    std::vector<double> f(m);
    for (size_t e = 0; e < m; e++) f[e] = target[e] * P.q[tg[e] - 1] / sg[e];
    V pr;
    FGB_TRY(fgb::vec::mult_scalar_at(P.sc, Gm, q[0], f, pr));
    FGB_TRY(fgb::vec::rescale(P.sc, pr, prod));
  }
  Part R;
  FGB_TRY(node(P, r, i - 1, target, R));
  out.c = R.c;
  if (prod.empty()) {
    out.ct = R.ct;
  } else if (R.ct.empty()) {
    out.ct = prod;
  } else {
    V pd, rd;
    FGB_TRY(align(P.sc, prod, R.ct, pd, rd));
    FGB_TRY(fgb::vec::add(P.sc, pd, rd, out.ct));
  }
  return FIDES_OK;
}

int chebyshev(fides_ctx* ctx, const V& a, const double* coeffs, uint32_t n, double lo, double hi, double const_scale,
              V& out) {
  if (!ctx || !coeffs || n < 2) return fgb::set_last_error(FIDES_EINVAL, "need a context, >= 2 coefficients");
  if (!(hi > lo)) return fgb::set_last_error(FIDES_EINVAL, "need lo < hi");
  Scope sc(ctx);
  fides_ctx_shape shape{};
  FGB_TRY(fides_ctx_get_shape(ctx, &shape));
  std::vector<uint64_t> mods(shape.nq + shape.np);
  FGB_TRY(fides_ctx_moduli(ctx, mods.data(), nullptr));
  Poly P{ctx, sc, std::vector<double>(mods.begin(), mods.end()), {}, {}, const_scale};
  const int d = (int)n - 1;
  V t1;
  if (lo == -1.0 && hi == 1.0) {
    t1 = a;
  } else {
    V u, r;
    FGB_TRY(fgb::vec::mult_scalar(sc, a, 2.0 / (hi - lo), const_scale, u));
    FGB_TRY(fgb::vec::rescale(sc, u, r));
    FGB_TRY(fgb::vec::add_scalar(sc, r, -(hi + lo) / (hi - lo), t1));
  }
  // baby steps T_1 .. T_{bs} (T_{bs} only when there are giant steps), giant steps T_{bs 2^i}
  const int lb = std::max(1, (int)std::lround(std::log2((double)(d + 1)) / 2.0));
  const int bs = 1 << lb;
  int m = 0;
  while ((bs << m) <= d) m++;
  const int top = m > 0 ? bs : bs - 1;
  P.T.resize(top + 1);
  P.T[1] = t1;
  for (int k = 2; k <= top; k++) FGB_TRY(next_t(P, k, P.T[k]));
  P.G.resize(m);
  if (m > 0) P.G[0] = P.T[bs];
  for (int i = 1; i < m; i++) {
    V sq;
    FGB_TRY(fgb::vec::square(sc, P.G[i - 1], sq));
    FGB_TRY(double_and_shift(sc, sq, nullptr, P.G[i]));
  }
  std::vector<double> c(coeffs, coeffs + n);
  c.resize((size_t)bs << m, 0.0);
  if (!has_terms(c)) return fgb::set_last_error(FIDES_EINVAL, "all non-constant coefficients are zero");
  Part R;
  FGB_TRY(node(P, c, m, fgb::vec::scales(ctx, t1), R));
  FGB_TRY(fgb::vec::add_scalar(sc, R.ct, R.c, out));
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
