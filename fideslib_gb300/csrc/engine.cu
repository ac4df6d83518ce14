// Host-side CKKS evaluation engine (see engine.hpp).
#include <algorithm>
#include <cstring>
#include <thread>

#include "engine.hpp"

namespace fgb {
namespace {

typedef unsigned __int128 u128;

u64 hmul(u64 a, u64 b, u64 p) { return (u64)(((u128)a * b) % p); }
u64 hpow(u64 a, u64 e, u64 p) {
  u64 r = 1 % p;
  a %= p;
  while (e) {
    if (e & 1) r = hmul(r, a, p);
    a = hmul(a, a, p);
    e >>= 1;
  }
  return r;
}
u64 hinv(u64 a, u64 p) { return hpow(a % p, p - 2, p); }
u64 shoup_of(u64 w, u64 p) { return (u64)(((u128)w << 64) / p); }

bool is_prime(u64 n) {
  if (n < 2) return false;
  for (u64 q : {2ull, 3ull, 5ull, 7ull, 11ull, 13ull, 17ull, 19ull, 23ull, 29ull, 31ull, 37ull}) {
    if (n == q) return true;
    if (n % q == 0) return false;
  }
  u64 d = n - 1;
  int r = 0;
  while (!(d & 1)) {
    d >>= 1;
    r++;
  }
  for (u64 a : {2ull, 325ull, 9375ull, 28178ull, 450775ull, 9780504ull, 1795265022ull}) {
    a %= n;
    if (!a) continue;
    u64 x = hpow(a, d, n);
    if (x == 1 || x == n - 1) continue;
    bool comp = true;
    for (int k = 1; k < r && comp; k++) {
      x = hmul(x, x, n);
      if (x == n - 1) comp = false;
    }
    if (comp) return false;
  }
  return true;
}

// Primitive 2N-th root g^((p-1)/2N) for the smallest generator g of Z_p^*.
u64 root_2n(u64 p, u64 twoN) {
  std::vector<u64> fac;
  u64 n = p - 1;
  for (u64 f = 2; f * f <= n; f += (f == 2 ? 1 : 2)) {
    if (n % f == 0) {
      fac.push_back(f);
      while (n % f == 0) n /= f;
      if (n > 1 && is_prime(n)) break;
    }
  }
  if (n > 1) fac.push_back(n);
  for (u64 g = 2; g < p; g++) {
    bool ok = true;
    for (u64 f : fac)
      if (hpow(g, (p - 1) / f, p) == 1) {
        ok = false;
        break;
      }
    if (ok) return hpow(g, (p - 1) / twoN, p);
  }
  return 0;
}

uint32_t brev(uint32_t x, int bits) {
  uint32_t r = 0;
  for (int i = 0; i < bits; i++) r |= ((x >> i) & 1u) << (bits - 1 - i);
  return r;
}

template <class F>
void parallel_for(int n, F f) {
  const int nt = std::max(1, std::min<int>(n, (int)std::thread::hardware_concurrency()));
  std::vector<std::thread> th;
  for (int w = 0; w < nt; w++)
    th.emplace_back([&, w] {
      for (int i = w; i < n; i += nt) f(i);
    });
  for (auto& t : th) t.join();
}

#define FGB_TRY(x)                          \
  do {                                      \
    cudaError_t e_ = (x);                   \
    if (e_ != cudaSuccess) return e_;       \
  } while (0)

}  // namespace

void* Context::dmalloc(size_t bytes) {
  void* p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) return nullptr;
  owned_.push_back(p);
  return p;
}

Context::~Context() {
  if (stream) cudaStreamSynchronize(stream);
  stream = own_stream;
  for (auto& kv : cts)
    if (kv.second.data) cudaFree(kv.second.data);
  for (auto& kv : rot_keys) cudaFree(kv.second);
  if (relin_key) cudaFree(relin_key);
  for (void* p : owned_) cudaFree(p);
  if (stream) cudaStreamDestroy(stream);
}

Context* Context::create(int logN, int nq, int np, int dnum, const u64* moduli, const u64* roots, std::string* err) {
  if (logN < 10 || logN > 16) {
    *err = "log_n must be in [10, 16]";
    return nullptr;
  }
  if (nq < 1 || np < 1 || nq + np > 64 || dnum < 1 || dnum > 8 || dnum > nq) {
    *err = "need 1 <= nq, 1 <= np, nq + np <= 64, 1 <= dnum <= min(8, nq)";
    return nullptr;
  }
  Context* c = new Context();
  c->logN = logN;
  c->N = 1 << logN;
  c->nq = nq;
  c->np = np;
  c->dnum = dnum;
  c->alpha = (nq + dnum - 1) / dnum;
  c->ntow = nq + np;
  if (np > 32) {
    *err = "at most 32 special primes";
    delete c;
    return nullptr;
  }
  c->mod.assign(moduli, moduli + nq + np);
  if (!c->build(roots, err)) {
    delete c;
    return nullptr;
  }
  return c;
}

bool Context::build(const u64* roots, std::string* err) {
  const u64 twoN = 2ull * N;
  for (int i = 0; i < ntow; i++) {
    const u64 p = mod[i];
    if (p >= (1ull << 60) || p % twoN != 1 || !is_prime(p)) {
      *err = "modulus " + std::to_string(i) + " is not a prime < 2^60 congruent to 1 mod 2N";
      return false;
    }
    for (int j = 0; j < i; j++)
      if (mod[j] == p) {
        *err = "moduli must be distinct";
        return false;
      }
  }
  psi.resize(ntow);
  parallel_for(ntow, [&](int i) { psi[i] = roots ? roots[i] % mod[i] : root_2n(mod[i], twoN); });
  for (int i = 0; i < ntow; i++)
    if (hpow(psi[i], (u64)N, mod[i]) != mod[i] - 1) {
      *err = "root " + std::to_string(i) + " is not a primitive 2N-th root of unity";
      return false;
    }

  if (cudaStreamCreateWithFlags(&own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    *err = "cudaStreamCreate failed";
    return false;
  }
  stream = own_stream;
  {  // keep freed stream-ordered allocations cached in the pool
    int dev = 0;
    cudaGetDevice(&dev);
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t thr = ~0ull;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
  }

  // per-prime constants
  std::vector<PrimeConst> pc(ntow);
  for (int i = 0; i < ntow; i++) {
    const u64 p = mod[i];
    PrimeConst& c = pc[i];
    c.p = p;
    c.p2 = 2 * p;
    c.r64 = (u64)(((u128)1 << 64) % p);
    c.r64_sh = shoup_of(c.r64, p);
    c.one_sh = shoup_of(1, p);
    c.ninv = hinv((u64)N, p);
    c.ninv_sh = shoup_of(c.ninv, p);
    c.pad = 0;
  }
  d_pc = (PrimeConst*)dmalloc(sizeof(PrimeConst) * ntow);
  if (!d_pc) {
    *err = "device allocation failed";
    return false;
  }
  cudaMemcpy(d_pc, pc.data(), sizeof(PrimeConst) * ntow, cudaMemcpyHostToDevice);

  // twiddles: tw[i] = psi^(+-brev(i)) with Shoup companion (OpenFHE rootOfUnityTable layout,
  // src/ConstantsGPU.cu:222-255)
  std::vector<ulonglong2> fwd((size_t)ntow * N), inv((size_t)ntow * N);
  parallel_for(ntow, [&](int i) {
    const u64 p = mod[i];
    const u64 w = psi[i], wi = hinv(psi[i], p);
    std::vector<u64> pw(N), ipw(N);
    pw[0] = ipw[0] = 1;
    for (int k = 1; k < N; k++) {
      pw[k] = hmul(pw[k - 1], w, p);
      ipw[k] = hmul(ipw[k - 1], wi, p);
    }
    for (int k = 0; k < N; k++) {
      const u64 a = pw[brev(k, logN)], b = ipw[brev(k, logN)];
      fwd[(size_t)i * N + k] = make_ulonglong2(a, shoup_of(a, p));
      inv[(size_t)i * N + k] = make_ulonglong2(b, shoup_of(b, p));
    }
  });
  ulonglong2* d_fwd = (ulonglong2*)dmalloc(sizeof(ulonglong2) * fwd.size());
  ulonglong2* d_inv = (ulonglong2*)dmalloc(sizeof(ulonglong2) * inv.size());
  if (!d_fwd || !d_inv) {
    *err = "device allocation failed";
    return false;
  }
  cudaMemcpy(d_fwd, fwd.data(), sizeof(ulonglong2) * fwd.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(d_inv, inv.data(), sizeof(ulonglong2) * inv.size(), cudaMemcpyHostToDevice);
  tabs.pc = d_pc;
  tabs.tw_fwd = d_fwd;
  tabs.tw_inv = d_inv;
  tabs.logN = logN;

  // CRT tables (OpenFHE PartQlHatInvModq / PartQlHatModp / PHatInvModp / PHatModq / PInvModq /
  // qlInvModq, as pulled by src/CKKS/openfhe-interface/RawCiphertext.cu:395-470)
  const int A = alpha;
  std::vector<ulonglong2> mu_qhinv((size_t)dnum * A * A, make_ulonglong2(0, 0));
  std::vector<uint32_t> mu_qhat((size_t)dnum * A * A * ntow * 2, 0);
  for (int d = 0; d < dnum; d++) {
    const int start = d * A;
    for (int s = 1; s <= A && start + s <= nq; s++) {
      const int b = (d * A + (s - 1)) * A;
      for (int i = 0; i < s; i++) {
        const u64 qi = mod[start + i];
        u64 prod = 1;
        for (int k = 0; k < s; k++)
          if (k != i) prod = hmul(prod, mod[start + k] % qi, qi);
        const u64 w = hinv(prod, qi);
        mu_qhinv[b + i] = make_ulonglong2(w, shoup_of(w, qi));
        for (int tw = 0; tw < ntow; tw++) {
          const u64 m = mod[tw];
          u64 v = 1;
          for (int k = 0; k < s; k++)
            if (k != i) v = hmul(v, mod[start + k] % m, m);
          mu_qhat[((size_t)(b + i) * ntow + tw) * 2 + 0] = (uint32_t)(v & ((1ull << 30) - 1));
          mu_qhat[((size_t)(b + i) * ntow + tw) * 2 + 1] = (uint32_t)(v >> 30);
        }
      }
    }
  }
  std::vector<ulonglong2> md_phinv(np), md_pinv(nq), rs_qinv((size_t)nq * nq, make_ulonglong2(0, 0));
  std::vector<uint32_t> md_phat((size_t)np * nq * 2);
  for (int k = 0; k < np; k++) {
    const u64 pk = mod[nq + k];
    u64 prod = 1;
    for (int k2 = 0; k2 < np; k2++)
      if (k2 != k) prod = hmul(prod, mod[nq + k2] % pk, pk);
    const u64 w = hinv(prod, pk);
    md_phinv[k] = make_ulonglong2(w, shoup_of(w, pk));
    for (int j = 0; j < nq; j++) {
      const u64 q = mod[j];
      u64 v = 1;
      for (int k2 = 0; k2 < np; k2++)
        if (k2 != k) v = hmul(v, mod[nq + k2] % q, q);
      md_phat[((size_t)k * nq + j) * 2 + 0] = (uint32_t)(v & ((1ull << 30) - 1));
      md_phat[((size_t)k * nq + j) * 2 + 1] = (uint32_t)(v >> 30);
    }
  }
  for (int j = 0; j < nq; j++) {
    const u64 q = mod[j];
    u64 P = 1;
    for (int k = 0; k < np; k++) P = hmul(P, mod[nq + k] % q, q);
    const u64 w = hinv(P, q);
    md_pinv[j] = make_ulonglong2(w, shoup_of(w, q));
  }
  for (int l = 1; l < nq; l++)
    for (int i = 0; i < l; i++) {
      const u64 q = mod[i];
      const u64 w = hinv(mod[l] % q, q);
      rs_qinv[(size_t)l * nq + i] = make_ulonglong2(w, shoup_of(w, q));
    }
  auto up = [&](const void* src, size_t bytes) -> void* {
    void* d = dmalloc(bytes ? bytes : 16);
    if (d && bytes) cudaMemcpy(d, src, bytes, cudaMemcpyHostToDevice);
    return d;
  };
  crt.nq = nq;
  crt.np = np;
  crt.alpha = alpha;
  crt.dnum = dnum;
  crt.ntow = ntow;
  crt.mu_qhinv = (const ulonglong2*)up(mu_qhinv.data(), sizeof(ulonglong2) * mu_qhinv.size());
  crt.mu_qhat = (const uint32_t*)up(mu_qhat.data(), sizeof(uint32_t) * mu_qhat.size());
  crt.md_phinv = (const ulonglong2*)up(md_phinv.data(), sizeof(ulonglong2) * md_phinv.size());
  crt.md_phat = (const uint32_t*)up(md_phat.data(), sizeof(uint32_t) * md_phat.size());
  crt.md_pinv = (const ulonglong2*)up(md_pinv.data(), sizeof(ulonglong2) * md_pinv.size());
  crt.rs_qinv = (const ulonglong2*)up(rs_qinv.data(), sizeof(ulonglong2) * rs_qinv.size());

  const size_t L = (size_t)N * sizeof(u64);
  ws_coeff_ = (u64*)dmalloc(L * nq);
  ws_conv_ = (u64*)dmalloc(L * dnum * ntow);
  ws_inner_ = (u64*)dmalloc(L * 2 * ntow);
  ws_md_ = (u64*)dmalloc(L * 2 * nq);
  ws_tensor_ = (u64*)dmalloc(L * 3 * nq);
  ws_top_ = (u64*)dmalloc(L * 2);
  ws_rs_ = (u64*)dmalloc(L * 2 * nq);
  if (!crt.mu_qhinv || !crt.mu_qhat || !crt.md_phinv || !crt.md_phat || !crt.md_pinv || !crt.rs_qinv ||
      !ws_coeff_ || !ws_conv_ || !ws_inner_ || !ws_md_ || !ws_tensor_ || !ws_top_ || !ws_rs_) {
    *err = "device allocation failed";
    return false;
  }
  if (cudaDeviceSynchronize() != cudaSuccess) {
    *err = std::string("device error during context set-up: ") + cudaGetErrorString(cudaGetLastError());
    return false;
  }
  return true;
}

u64* Context::alloc_limbs(size_t nlimbs, cudaStream_t s) {
  void* p = nullptr;
  if (cudaMallocAsync(&p, nlimbs * (size_t)N * sizeof(u64), s) != cudaSuccess) return nullptr;
  return (u64*)p;
}

void Context::free_limbs(u64* p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

uint32_t Context::galois_inverse(uint32_t g) const {
  u64 x = g;  // Newton iteration for the inverse modulo a power of two
  for (int i = 0; i < 6; i++) x *= 2 - (u64)g * x;
  return (uint32_t)(x & (2ull * N - 1));
}

uint32_t Context::galois_for_index(int N, int32_t index) {
  const u64 M = 2ull * N;
  if (index == 0) return 1;
  if ((u64)(int64_t)index == M - 1) return (uint32_t)(M - 1);
  const int64_t half = N / 2;  // order of 5 modulo 2N
  int64_t r = index % half;
  if (r < 0) r += half;
  u64 g = 1;
  for (int64_t k = 0; k < r; k++) g = (g * 5) % M;
  return (uint32_t)g;
}

cudaError_t Context::ntt(u64* data, int npolys, int limbs, int first_prime, long long poly_stride, bool inverse,
                         cudaStream_t s) {
  NttBatch b{};
  b.nseg = 1;
  b.total_limbs = npolys * limbs;
  NttSeg& g = b.seg[0];
  g.data = data;
  g.poly_stride = poly_stride;
  g.limbs = limbs;
  g.npolys = npolys;
  g.limb_begin = 0;
  for (int j = 0; j < limbs; j++) g.prime_of[j] = (uint8_t)(first_prime + j);
  return launch_ntt(b, tabs, inverse, s);
}

cudaError_t Context::modup(const u64* a, int t, cudaStream_t s) {
  const size_t L = (size_t)N;
  const int beta = (t + alpha - 1) / alpha;
  FGB_TRY(cudaMemcpyAsync(ws_coeff_, a, sizeof(u64) * L * t, cudaMemcpyDeviceToDevice, s));
  FGB_TRY(ntt(ws_coeff_, 1, t, 0, 0, true, s));
  KsDims k{N, logN, t, beta};
  const long long cs = (long long)ntow * N;
  FGB_TRY(launch_modup_conv(ws_coeff_, ws_conv_, cs, k, crt, d_pc, s));
  NttBatch b{};
  b.nseg = beta;
  int begin = 0;
  for (int d = 0; d < beta; d++) {
    const int start = d * alpha, sz = std::min(alpha, t - start);
    NttSeg& g = b.seg[d];
    g.data = ws_conv_ + d * cs;
    g.poly_stride = 0;
    g.npolys = 1;
    g.limbs = t - sz + np;
    g.limb_begin = begin;
    for (int jj = 0; jj < g.limbs; jj++)
      g.prime_of[jj] = (uint8_t)(jj < start ? jj : (jj < t - sz ? jj + sz : nq + (jj - (t - sz))));
    begin += g.limbs;
  }
  b.total_limbs = begin;
  FGB_TRY(launch_ntt(b, tabs, false, s));
  digits_t_ = t;
  return cudaSuccess;
}

cudaError_t Context::ks_from_digits(const u64* a, int t, const u64* key, const u64* add0, const u64* add1, u64* out,
                                    uint32_t galois_inv, cudaStream_t s) {
  const int beta = (t + alpha - 1) / alpha;
  KsDims k{N, logN, t, beta};
  const long long cs = (long long)ntow * N;
  const int ext = t + np;
  FGB_TRY(launch_ks_inner(a, ws_conv_, cs, key, ws_inner_, k, crt, d_pc, s));
  // P towers of both inner products to coefficient form
  {
    NttBatch b{};
    b.nseg = 1;
    b.total_limbs = 2 * np;
    NttSeg& g = b.seg[0];
    g.data = ws_inner_ + (size_t)t * N;
    g.poly_stride = (long long)ext * N;
    g.limbs = np;
    g.npolys = 2;
    for (int j = 0; j < np; j++) g.prime_of[j] = (uint8_t)(nq + j);
    FGB_TRY(launch_ntt(b, tabs, true, s));
  }
  FGB_TRY(launch_moddown_conv(ws_inner_, (long long)ext * N, ws_md_, (long long)t * N, 2, k, crt, d_pc, s));
  FGB_TRY(ntt(ws_md_, 2, t, 0, (long long)t * N, false, s));
  FGB_TRY(launch_moddown_epilogue(ws_inner_, (long long)ext * N, ws_md_, (long long)t * N, add0, add1, out,
                                  (long long)t * N, 2, galois_inv, k, crt, d_pc, s));
  return cudaSuccess;
}

cudaError_t Context::keyswitch(const u64* a, int t, const u64* key, const u64* add0, const u64* add1, u64* out,
                               uint32_t galois_inv, cudaStream_t s) {
  FGB_TRY(modup(a, t, s));
  return ks_from_digits(a, t, key, add0, add1, out, galois_inv, s);
}

cudaError_t Context::mult(const u64* x, const u64* y, int t, const u64* rlk, u64* out, cudaStream_t s) {
  const size_t P = (size_t)t * N;
  FGB_TRY(launch_tensor(x, y, ws_tensor_, t, N, d_pc, s));
  return keyswitch(ws_tensor_ + 2 * P, t, rlk, ws_tensor_, ws_tensor_ + P, out, 1, s);
}

cudaError_t Context::rotate(const u64* x, int t, uint32_t galois, const u64* key, u64* out, cudaStream_t s) {
  const size_t P = (size_t)t * N;
  return keyswitch(x + P, t, key, x, nullptr, out, galois_inverse(galois), s);
}

cudaError_t Context::rescale(const u64* x, int t, u64* out, cudaStream_t s) {
  if (t < 2) return cudaErrorInvalidValue;
  const size_t P = (size_t)t * N;
  FGB_TRY(cudaMemcpyAsync(ws_top_, x + (size_t)(t - 1) * N, sizeof(u64) * N, cudaMemcpyDeviceToDevice, s));
  FGB_TRY(cudaMemcpyAsync(ws_top_ + N, x + P + (size_t)(t - 1) * N, sizeof(u64) * N, cudaMemcpyDeviceToDevice, s));
  FGB_TRY(ntt(ws_top_, 2, 1, t - 1, N, true, s));
  FGB_TRY(launch_rescale_switch(ws_top_, N, ws_rs_, 2, t, N, d_pc, s));
  FGB_TRY(ntt(ws_rs_, 2, t - 1, 0, (long long)(t - 1) * N, false, s));
  FGB_TRY(launch_rescale_epilogue(x, (long long)P, ws_rs_, out, 2, t, N, crt, d_pc, s));
  return cudaSuccess;
}

}  // namespace fgb
