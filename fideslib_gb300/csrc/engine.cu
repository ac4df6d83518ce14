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
  for (auto& kv : pts)
    if (kv.second.data) cudaFree(kv.second.data);
  for (auto& kv : ext_cts)
    if (kv.second.data) cudaFree(kv.second.data);
  for (auto& kv : modups) {
    if (kv.second.c1) cudaFree(kv.second.c1);
    if (kv.second.digits) cudaFree(kv.second.digits);
  }
  for (auto& kv : lts) {
    if (kv.second.diags) cudaFree(kv.second.diags);
    if (kv.second.present_dev) cudaFree(kv.second.present_dev);
  }
  for (auto& kv : rot_keys) cudaFree(kv.second);
  if (relin_key) cudaFree(relin_key);
  for (void* p : owned_) cudaFree(p);
  if (side) cudaStreamSynchronize(side);
  if (copy_in) cudaStreamDestroy(copy_in);
  if (side) cudaStreamDestroy(side);
  for (cudaEvent_t e : side_ev)
    if (e) cudaEventDestroy(e);
  if (copy_out) cudaStreamDestroy(copy_out);
  if (chunk_alt) cudaStreamDestroy(chunk_alt);
  if (stream) cudaStreamDestroy(stream);
  // Its allocations were freed above; the pool's cached memory goes back to the device with it.
  if (pool) cudaMemPoolDestroy(pool);
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
  cudaGetDevice(&c->device);
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
  {  // the context's own stream-ordered pool on its device
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = device;
    if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
      cudaGetLastError();
      *err = "cudaMemPoolCreate failed";
      return false;
    }
    // Freed allocations stay cached in the pool (the reference's pool keeps a release threshold at the maximum,
    // src/CKKS/Context.cu:74-80).
    uint64_t thr = ~0ull;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    // Memory freed on one stream is reused on another only once the free has completed or an event orders the
    // two: the pool may not make an allocating stream wait on another stream's pending work, which would chain
    // the copy and compute streams of a pipelined host batch into one sequence.
    int no = 0;
    cudaMemPoolSetAttribute(pool, cudaMemPoolReuseAllowInternalDependencies, &no);
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
    c.negp = 0ull - p;
    c.w1ninv = hmul(hpow(hinv(psi[i], p), (u64)N / 2, p), c.ninv, p);  // psi^-brev(1) = psi^-(N/2)
    c.w1ninv_sh = shoup_of(c.w1ninv, p);
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
  // The NTT kernels read the twiddles of their last four stages (s >= logN - 4, the 16-residue groups of pass C)
  // from a transposed copy: entry m + G*nw + j (m = 2^s, nw = m / (N/16) twiddles per group G) is stored at
  // m + j*(N/16) + G, so the lanes of a warp (consecutive groups) read consecutive entries.
  std::vector<ulonglong2> fwd_t(fwd), inv_t(inv);
  const int groups = N >> 4;
  parallel_for(ntow, [&](int i) {
    const size_t base = (size_t)i * N;
    for (int s = logN - 4; s < logN; s++) {
      const int m = 1 << s, nw = m / groups;
      for (int G = 0; G < groups; G++)
        for (int j = 0; j < nw; j++) {
          fwd_t[base + m + (size_t)j * groups + G] = fwd[base + m + (size_t)G * nw + j];
          inv_t[base + m + (size_t)j * groups + G] = inv[base + m + (size_t)G * nw + j];
        }
    }
  });
  ulonglong2* d_psi = (ulonglong2*)dmalloc(sizeof(ulonglong2) * fwd.size());
  ulonglong2* d_fwd = (ulonglong2*)dmalloc(sizeof(ulonglong2) * fwd.size());
  ulonglong2* d_inv = (ulonglong2*)dmalloc(sizeof(ulonglong2) * inv.size());
  if (!d_psi || !d_fwd || !d_inv) {
    *err = "device allocation failed";
    return false;
  }
  cudaMemcpy(d_psi, fwd.data(), sizeof(ulonglong2) * fwd.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(d_fwd, fwd_t.data(), sizeof(ulonglong2) * fwd.size(), cudaMemcpyHostToDevice);
  cudaMemcpy(d_inv, inv_t.data(), sizeof(ulonglong2) * inv.size(), cudaMemcpyHostToDevice);
  psi_brev = d_psi;
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
  std::vector<ulonglong2> md_phinv(np), md_pinv(nq), md_pmodq(nq),
      rs_qinv((size_t)nq * nq, make_ulonglong2(0, 0));
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
    md_pmodq[j] = make_ulonglong2(P, shoup_of(P, q));
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
  crt.md_pmodq = (const ulonglong2*)up(md_pmodq.data(), sizeof(ulonglong2) * md_pmodq.size());
  crt.rs_qinv = (const ulonglong2*)up(rs_qinv.data(), sizeof(ulonglong2) * rs_qinv.size());

  if (!crt.mu_qhinv || !crt.mu_qhat || !crt.md_phinv || !crt.md_phat || !crt.md_pinv || !crt.md_pmodq ||
      !crt.rs_qinv) {
    *err = "device allocation failed";
    return false;
  }
  ring_.N = N;
  ring_.logN = logN;
  if (cudaDeviceSynchronize() != cudaSuccess) {
    *err = std::string("device error during context set-up: ") + cudaGetErrorString(cudaGetLastError());
    return false;
  }
  if (tune_ntt(tabs, own_stream, ntt_tune_ms) != cudaSuccess) {  // pick the forward NTT kernel for this ring
    *err = std::string("NTT tuning failed: ") + cudaGetErrorString(cudaGetLastError());
    return false;
  }
  return true;
}

cudaError_t Context::tune_ks(const KsBatch& kb, cudaStream_t s) {
  // Every tile writes the same inner products, so the batch's own launch is timed once per tile that the ring
  // allows (a thread block covers 512 * iters coefficients) and the caller's launch follows with the fastest.
  cudaEvent_t ev[2] = {nullptr, nullptr};
  cudaError_t e = cudaEventCreate(&ev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
  if (e == cudaSuccess) e = launch_ks_inner(kb, ring_, crt, d_pc, s);  // warm-up with the current tile
  float best = 0;
  int pick = 0;
  for (int v = 0; v < kKsTileVariants && e == cudaSuccess; v++) {
    const int it = 1 << v;
    if (it > N / 512) continue;
    crt.ks_iters = it;
    e = cudaEventRecord(ev[0], s);
    if (e == cudaSuccess) e = launch_ks_inner(kb, ring_, crt, d_pc, s);
    if (e == cudaSuccess) e = cudaEventRecord(ev[1], s);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
    float el = 0;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&el, ev[0], ev[1]);
    if (e != cudaSuccess) break;
    ks_tune_ms[v] = el;
    if (pick == 0 || el < best) {
      best = el;
      pick = it;
    }
  }
  crt.ks_iters = pick;  // 0 (the kernel's default) if nothing was timed
  for (cudaEvent_t x : ev)
    if (x) cudaEventDestroy(x);
  ks_tuned = true;
  return e;
}

u64* Context::alloc_limbs(size_t nlimbs, cudaStream_t s) {
  const size_t bytes = nlimbs * (size_t)N * sizeof(u64);
  std::lock_guard<std::mutex> lk(mem_mu_);
  if (mem_limit && mem_in_use + bytes > mem_limit) return nullptr;  // the caller reports FIDES_ENOMEM
  void* p = nullptr;
  if (cudaMallocFromPoolAsync(&p, bytes, pool, s) != cudaSuccess) {
    cudaGetLastError();  // a failed allocation must not surface as a later launch error
    return nullptr;
  }
  mem_in_use += bytes;
  mem_sizes_[p] = bytes;
  return (u64*)p;
}

void Context::free_limbs(u64* p, cudaStream_t s) {
  if (!p) return;
  cudaFreeAsync(p, s);
  std::lock_guard<std::mutex> lk(mem_mu_);
  auto it = mem_sizes_.find(p);
  if (it != mem_sizes_.end()) {
    mem_in_use -= it->second;
    mem_sizes_.erase(it);
  }
}

int Context::residues_out_of_range(const u64* x, long long rows, int period, int tq) {
  if (!d_bad) {
    d_bad = (int*)dmalloc(sizeof(int));
    if (!d_bad) return -1;
  }
  int bad = 0;
  if (cudaMemsetAsync(d_bad, 0, sizeof(int), stream) != cudaSuccess ||
      launch_range_check(x, rows, logN, period, tq, nq, d_pc, d_bad, stream) != cudaSuccess ||
      cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
      cudaStreamSynchronize(stream) != cudaSuccess)
    return -1;
  return bad ? 1 : 0;
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
  u64 g = 1, b = 5;
  for (; r; r >>= 1, b = b * b % M)
    if (r & 1) g = g * b % M;
  return (uint32_t)g;
}

uint32_t Context::rotation_key_galois(int32_t index, int slots) const {
  const int64_t half = N / 2;
  const uint32_t conj = (uint32_t)(2ull * N - 1);
  if ((int64_t)index == (int64_t)conj) return rot_keys.count(conj) ? conj : 0;
  const bool sparse = slots > 0 && slots < half;
  int64_t idx = index;
  if (sparse) {  // Ciphertext::normalyzeIndex: modulo slots, the upper half taken as negative rotations
    idx %= slots;
    if (idx < 0) idx += slots;
    if (idx > slots / 2) idx += half - slots;
  }
  idx %= half;
  if (idx < 0) idx += half;
  uint32_t g = galois_for_index(N, (int32_t)idx);
  if (rot_keys.count(g)) return g;
  if (sparse)  // ContextData::GetRotationKey: a key of an index congruent modulo slots
    for (int64_t i = 1; i < half / slots; i++) {
      g = galois_for_index(N, (int32_t)((idx + i * slots) % half));
      if (rot_keys.count(g)) return g;
    }
  return 0;
}

namespace {

// Accumulates NTT jobs and launches whenever kMaxNttJobs are queued.
struct NttQueue {
  const DeviceTables& tabs;
  bool inverse;
  cudaStream_t s;
  NttBatch b{};
  cudaError_t err = cudaSuccess;
  // lazy: outputs left in [0, 4p), for transforms whose readers reduce them: the basis conversions (their Shoup
  // product by the Qhat^-1 / Phat^-1 factor takes any 64-bit input), the ModDown epilogue, the key inner product
  // of at most three digits
  NttQueue(const DeviceTables& t, bool inv, cudaStream_t st, bool lazy = false) : tabs(t), inverse(inv), s(st) {
    b.lazy_out = lazy ? 1 : 0;
  }
  void add(const u64* src, u64* dst, long long ss, long long ds, int limbs, int npolys, const uint8_t* prime_of) {
    if (err != cudaSuccess || limbs <= 0 || npolys <= 0) return;
    if (b.njobs == kMaxNttJobs) flush();
    ntt_add_job(b, src, dst, ss, ds, limbs, npolys, prime_of);
  }
  void flush() {
    if (err == cudaSuccess && b.njobs > 0) err = launch_ntt(b, tabs, inverse, s);
    b.njobs = 0;
    b.limb_begin[0] = 0;
  }
};

}  // namespace

cudaError_t Context::ntt(const u64* src, u64* dst, int npolys, int limbs, int first_prime, long long poly_stride,
                         bool inverse, cudaStream_t s) {
  NttQueue q(tabs, inverse, s);
  uint8_t pm[64];
  for (int j = 0; j < limbs; j++) pm[j] = (uint8_t)(first_prime + j);
  q.add(src, dst, poly_stride, poly_stride, limbs, npolys, pm);
  q.flush();
  return q.err;
}

cudaError_t Context::modup(const u64* const* a, const int* ts, u64* const* coeff, u64* const* conv, int ng,
                           cudaStream_t s) {
  const size_t NN = (size_t)N;
  cudaError_t err = cudaSuccess;
  uint8_t pm[64];
  // 1) INTT of every input into its coefficient buffer (read only by the conversion: left in [0, 4p))
  {
    NttQueue q(tabs, true, s, true);
    for (int g = 0; g < ng; g++) {
      for (int j = 0; j < ts[g]; j++) pm[j] = (uint8_t)j;
      q.add(a[g], coeff[g], 0, 0, ts[g], 1, pm);
    }
    q.flush();
    err = q.err;
  }
  // 2) ModUp basis conversion, 3) NTT of the converted rows
  for (int g0 = 0; g0 < ng && err == cudaSuccess; g0 += kMaxJobs) {
    KsBatch kb{};
    for (int g = g0; g < ng && kb.njobs < kMaxJobs; g++) {
      KsJob& j = kb.jobs[kb.njobs++];
      j = KsJob{};
      j.a = a[g];
      j.coeff = coeff[g];
      j.conv = conv[g];
      j.t = ts[g];
    }
    err = launch_modup_conv(kb, ring_, crt, d_pc, s);
  }
  if (err == cudaSuccess) {
    // The converted digits are read only by the key inner product.  With at most three digits it accumulates four
    // 30-bit-slice products per term, which stay exact for digit values below 2^62, so the transform may leave them
    // in [0, 4p) (beta * (2^32 * 2^30) < 2^64 for beta <= 3); with more digits they are fully reduced.
    NttQueue q(tabs, false, s, dnum <= 3);
    for (int g = 0; g < ng; g++) {
      const int t = ts[g], beta = (t + alpha - 1) / alpha;
      for (int d = 0; d < beta; d++) {
        const int start = d * alpha, sz = std::min(alpha, t - start), rows = t - sz + np;
        for (int jj = 0; jj < rows; jj++)
          pm[jj] = (uint8_t)(jj < start ? jj : (jj < t - sz ? jj + sz : nq + (jj - (t - sz))));
        u64* c = conv[g] + (size_t)d * (t + np) * NN;
        q.add(c, c, 0, 0, rows, 1, pm);
      }
    }
    q.flush();
    err = q.err;
  }
  return err;
}

cudaError_t Context::keyswitch_batch(const KsReq* reqs_in, int n, cudaStream_t s) {
  const KsReq* reqs = reqs_in;
  std::vector<KsReq> by_key;
  if (n >= kKsSplit && reqs[0].ext_mode == 0) {  // (the double-hoisted transforms measured faster unsplit)
    // the first half ends at a request boundary that no ModUp group (same a, t, digits) straddles
    auto split_at = [&](const KsReq* r) {
      auto same = [&](int i, int k) { return r[i].a == r[k].a && r[i].t == r[k].t && r[i].digits == r[k].digits; };
      int h = n / 2;
      for (; h < n; h++) {
        bool straddles = false;
        for (int i = 0; i < h && !straddles; i++)
          for (int k = h; k < n && !straddles; k++) straddles = same(i, k);
        if (!straddles) break;
      }
      return h;
    };
    // Requests ordered by key first, so that the requests of one key land in one half and its inner products read
    // the key from HBM once (the launcher groups a half's jobs by key); if that order leaves no clean split (ModUp
    // groups spread over several keys), the given order is tried.
    by_key.assign(reqs, reqs + n);
    std::stable_sort(by_key.begin(), by_key.end(),
                     [](const KsReq& x, const KsReq& y) { return std::less<const u64*>()(x.key, y.key); });
    int h = split_at(by_key.data());
    if (h < n) {
      reqs = by_key.data();
    } else {
      h = split_at(reqs);
    }
    if (h < n) {
      cudaError_t err = cudaSuccess;
      if (!side) err = cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking);
      for (int k = 0; k < 2 && err == cudaSuccess; k++)
        if (!side_ev[k]) err = cudaEventCreateWithFlags(&side_ev[k], cudaEventDisableTiming);
      if (err == cudaSuccess) err = cudaEventRecord(side_ev[0], s);
      if (err == cudaSuccess) err = cudaStreamWaitEvent(side, side_ev[0], 0);
      if (err != cudaSuccess) return err;
      const cudaError_t e1 = keyswitch_run(reqs, h, s);
      const cudaError_t e2 = keyswitch_run(reqs + h, n - h, side);
      err = cudaEventRecord(side_ev[1], side);
      if (err == cudaSuccess) err = cudaStreamWaitEvent(s, side_ev[1], 0);
      return e1 != cudaSuccess ? e1 : e2 != cudaSuccess ? e2 : err;
    }
  }
  return keyswitch_run(reqs, n, s);
}

cudaError_t Context::keyswitch_run(const KsReq* reqs, int n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const size_t NN = (size_t)N;
  // ModUp groups: requests with the same input (and no precomputed digits) share the digits.
  std::vector<int> group_of(n);
  std::vector<int> gfirst;
  for (int i = 0; i < n; i++) {
    int g = -1;
    for (size_t k = 0; k < gfirst.size(); k++) {
      const KsReq& f = reqs[gfirst[k]];
      if (f.a == reqs[i].a && f.t == reqs[i].t && f.digits == reqs[i].digits) {
        g = (int)k;
        break;
      }
    }
    if (g < 0) {
      g = (int)gfirst.size();
      gfirst.push_back(i);
    }
    group_of[i] = g;
  }
  const int ng = (int)gfirst.size();
  size_t total = 0;
  std::vector<size_t> g_off(ng), r_off(n);
  for (int g = 0; g < ng; g++) {
    const int t = reqs[gfirst[g]].t, beta = (t + alpha - 1) / alpha;
    g_off[g] = total;
    if (!reqs[gfirst[g]].digits) total += (size_t)t + (size_t)beta * (t + np);
  }
  for (int i = 0; i < n; i++) {
    const int t = reqs[i].t;
    r_off[i] = total;
    total += (size_t)2 * (t + np) + (reqs[i].ext_mode ? 0 : (size_t)2 * t);
  }
  u64* ws = alloc_limbs(total, s);
  if (!ws) return cudaErrorMemoryAllocation;
  auto coeff_of = [&](int g) { return ws + g_off[g] * NN; };
  auto conv_of = [&](int g) {
    const KsReq& f = reqs[gfirst[g]];
    return f.digits ? const_cast<u64*>(f.digits) : ws + (g_off[g] + f.t) * NN;
  };
  auto inner_of = [&](int i) { return ws + r_off[i] * NN; };
  auto md_of = [&](int i) { return ws + (r_off[i] + 2 * (size_t)(reqs[i].t + np)) * NN; };
  std::vector<const u64*> ma;
  std::vector<int> mt;
  std::vector<u64*> mcoeff, mconv;
  for (int g = 0; g < ng; g++) {
    const KsReq& f = reqs[gfirst[g]];
    if (f.digits) continue;  // precomputed (fides_fast_rotation_precompute)
    ma.push_back(f.a);
    mt.push_back(f.t);
    mcoeff.push_back(coeff_of(g));
    mconv.push_back(conv_of(g));
  }
  cudaError_t err = modup(ma.data(), mt.data(), mcoeff.data(), mconv.data(), (int)ma.size(), s);
  // 4) inner products; then 5) INTT of the P rows, 6) ModDown conversion, 7) NTT, 8) epilogue for the ordinary
  // requests, or the extended-basis epilogue for the double-hoisted ones
  for (int i0 = 0; i0 < n && err == cudaSuccess; i0 += kMaxJobs) {
    KsBatch kb{}, md{}, ex{};
    for (int i = i0; i < n && kb.njobs < kMaxJobs; i++) {
      const KsReq& r = reqs[i];
      KsJob& j = kb.jobs[kb.njobs++];
      j.a = r.a;
      j.add0 = r.add0;
      j.add1 = r.add1;
      j.key = r.key;
      j.coeff = coeff_of(group_of[i]);
      j.conv = conv_of(group_of[i]);
      j.inner = inner_of(i);
      j.md = r.ext_mode ? nullptr : md_of(i);
      j.out = r.out;
      j.t = r.t;
      j.galois_inv = r.galois_inv;
      j.polys = 2;
      j.ext_mode = r.ext_mode;
      KsBatch& dst = r.ext_mode ? ex : md;
      dst.jobs[dst.njobs++] = j;
    }
    if (!ks_tuned && kb.njobs >= kKsTuneJobs) err = tune_ks(kb, s);  // the first batch of this size tunes the tile
    if (err == cudaSuccess) err = launch_ks_inner(kb, ring_, crt, d_pc, s);
    if (err == cudaSuccess) err = moddown_jobs(md, s);
    if (err == cudaSuccess) err = launch_ext_epilogue(ex, ring_, crt, d_pc, s);
  }
  free_limbs(ws, s);
  return err;
}

cudaError_t Context::moddown_jobs(const KsBatch& kb, cudaStream_t s) {
  if (kb.njobs <= 0) return cudaSuccess;
  const size_t NN = (size_t)N;
  uint8_t pm[64];
  cudaError_t err;
  {  // the P rows to coefficient form, read only by the ModDown conversion: left in [0, 4p)
    NttQueue q(tabs, true, s, true);
    for (int k = 0; k < np; k++) pm[k] = (uint8_t)(nq + k);
    for (int b = 0; b < kb.njobs; b++) {
      const KsJob& j = kb.jobs[b];
      u64* p = j.inner + (size_t)j.t * NN;
      q.add(p, p, (long long)(j.t + np) * N, (long long)(j.t + np) * N, np, j.polys ? j.polys : 2, pm);
    }
    q.flush();
    err = q.err;
  }
  if (err == cudaSuccess) err = launch_moddown_conv(kb, ring_, crt, d_pc, s);
  if (err == cudaSuccess) {
    NttQueue q(tabs, false, s, true);  // read only by the epilogue, which takes [0, 4p)
    for (int b = 0; b < kb.njobs; b++) {
      const KsJob& j = kb.jobs[b];
      for (int k = 0; k < j.t; k++) pm[k] = (uint8_t)k;
      q.add(j.md, j.md, (long long)j.t * N, (long long)j.t * N, j.t, j.polys ? j.polys : 2, pm);
    }
    q.flush();
    err = q.err;
  }
  if (err == cudaSuccess) err = launch_moddown_epilogue(kb, ring_, crt, d_pc, s);
  return err;
}

cudaError_t Context::moddown_batch(const MdReq* reqs, int n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const size_t NN = (size_t)N;
  std::vector<size_t> off(n);
  size_t total = 0;
  for (int i = 0; i < n; i++) {
    off[i] = total;
    total += (size_t)reqs[i].polys * reqs[i].t;
  }
  u64* ws = alloc_limbs(total, s);
  if (!ws) return cudaErrorMemoryAllocation;
  cudaError_t err = cudaSuccess;
  for (int i0 = 0; i0 < n && err == cudaSuccess; i0 += kMaxJobs) {
    KsBatch kb{};
    for (int i = i0; i < n && kb.njobs < kMaxJobs; i++) {
      KsJob& j = kb.jobs[kb.njobs++];
      j.inner = reqs[i].x;
      j.md = ws + off[i] * NN;
      j.out = reqs[i].out;
      j.t = reqs[i].t;
      j.polys = reqs[i].polys;
      j.galois_inv = 1;
    }
    err = moddown_jobs(kb, s);
  }
  free_limbs(ws, s);
  return err;
}

cudaError_t Context::mult_batch(const MultReq* reqs, int n, const u64* rlk, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const size_t NN = (size_t)N;
  size_t total = 0;
  std::vector<size_t> off(n);
  for (int i = 0; i < n; i++) {
    off[i] = total;
    total += (size_t)3 * reqs[i].t;
  }
  u64* ws = alloc_limbs(total, s);
  if (!ws) return cudaErrorMemoryAllocation;
  cudaError_t err = cudaSuccess;
  for (int i0 = 0; i0 < n && err == cudaSuccess; i0 += kMaxJobs) {
    TensorBatch tb{};
    for (int i = i0; i < n && tb.njobs < kMaxJobs; i++)
      tb.jobs[tb.njobs++] = TensorJob{reqs[i].x, reqs[i].y, ws + off[i] * NN, reqs[i].t};
    err = launch_tensor(tb, ring_, nq, d_pc, s);
  }
  if (err == cudaSuccess) {
    std::vector<KsReq> ks(n);
    for (int i = 0; i < n; i++) {
      u64* d = ws + off[i] * NN;
      const size_t P = (size_t)reqs[i].t * NN;
      ks[i] = KsReq{d + 2 * P, reqs[i].t, rlk, d, d + P, reqs[i].out, 1u};
    }
    err = keyswitch_batch(ks.data(), n, s);
  }
  free_limbs(ws, s);
  return err;
}

cudaError_t Context::rescale_batch(const RescaleReq* reqs, int n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const size_t NN = (size_t)N;
  for (int i = 0; i < n; i++)
    if (reqs[i].t < 2) return cudaErrorInvalidValue;
  u64* ws = alloc_limbs((size_t)2 * n, s);  // the top tower of both polys, coefficient form
  if (!ws) return cudaErrorMemoryAllocation;
  cudaError_t err = cudaSuccess;
  uint8_t pm[64];
  for (int i0 = 0; i0 < n && err == cudaSuccess; i0 += kMaxNttJobs) {
    const int i1 = std::min(n, i0 + kMaxNttJobs);
    {  // top towers of both polys to coefficient form (out of place)
      NttQueue q(tabs, true, s);
      for (int i = i0; i < i1; i++) {
        pm[0] = (uint8_t)(reqs[i].t - 1);
        q.add(reqs[i].x + (size_t)(reqs[i].t - 1) * NN, ws + (size_t)2 * i * NN, (long long)reqs[i].t * N, N, 1, 2,
              pm);
      }
      q.flush();
      err = q.err;
    }
    if (err != cudaSuccess) break;
    // the switch of the top tower into every q_i, the NTT and (x_i - .) q_l^-1 in one launch
    NttBatch nb{};
    NttEpi ep;
    for (int i = i0; i < i1; i++) {
      const int t = reqs[i].t;
      for (int k = 0; k < t - 1; k++) pm[k] = (uint8_t)k;
      ntt_add_job(nb, ws + (size_t)2 * i * NN, nullptr, N, 0, t - 1, 2, pm);
      ep.jobs[i - i0] = NttEpiJob{reqs[i].x, reqs[i].out, crt.rs_qinv + (size_t)(t - 1) * nq, t, t - 1, t - 1};
    }
    err = launch_ntt_epi(nb, ep, tabs, s);
  }
  free_limbs(ws, s);
  return err;
}

cudaError_t Context::add_batch(const AddReq* reqs, int n, cudaStream_t s) {
  cudaError_t err = cudaSuccess;
  for (int i0 = 0; i0 < n && err == cudaSuccess; i0 += kMaxJobs) {
    AddBatch ab{};
    for (int i = i0; i < n && ab.njobs < kMaxJobs; i++)
      ab.jobs[ab.njobs++] = AddJob{reqs[i].x, reqs[i].y, reqs[i].out, reqs[i].t, reqs[i].sub ? 1 : 0};
    err = launch_addsub(ab, ring_, nq, d_pc, s);
  }
  return err;
}

namespace {
int32_t slot_mod(int64_t r, int N) {  // rotation index reduced modulo N/2 (the order of 5 modulo 2N)
  const int64_t h = N / 2;
  r %= h;
  return (int32_t)(r < 0 ? r + h : r);
}
}  // namespace

std::vector<int32_t> DevLT::baby_rotations(int N) const {
  std::vector<int32_t> r;
  for (int b = 1; b < bs; b++) r.push_back(slot_mod((int64_t)b * stride, N));
  return r;
}

std::vector<int32_t> DevLT::giant_rotations(int N) const {
  std::vector<int32_t> r;
  for (int g = 0; g < gs; g++) r.push_back(slot_mod(base + (int64_t)g * bs * stride, N));
  return r;
}

cudaError_t Context::linear_transform(const u64* x, int t, const DevLT& lt, u64* out, cudaStream_t s) {
  return linear_transform_batch(&x, 1, t, lt, &out, s);
}

// Inner sums of n inputs: one job per (input, chunk of at most kDotG consecutive giant steps), kMaxJobs jobs per
// launch; rot0(i) / rot1(i) are input i's baby-step ciphertexts b = 0 / b = 1 (the rest follow at db.rot_stride),
// out(i, g) its inner sum of giant step g (chunks write consecutive giant steps at db.out_stride).
template <class R0, class R1, class O>
static cudaError_t inner_sums(DotBatch& db, int n, int gs, R0 rot0, R1 rot1, O out, const Ring& ring,
                              const PrimeConst* pc, cudaStream_t s) {
  cudaError_t err = cudaSuccess;
  db.njobs = 0;
  for (int i = 0; i < n && err == cudaSuccess; i++)
    for (int g = 0; g < gs && err == cudaSuccess; g += kDotG) {
      db.jobs[db.njobs++] = DotJob{out(i, g), rot0(i), rot1(i), g, std::min(kDotG, gs - g), 0ull};
      if (db.njobs == kMaxJobs) {
        err = launch_ptdot(db, ring, pc, s);
        db.njobs = 0;
      }
    }
  if (err == cudaSuccess && db.njobs) err = launch_ptdot(db, ring, pc, s);
  return err;
}

cudaError_t Context::linear_transform_batch(const u64* const* xs, int n, int t, const DevLT& lt, u64* const* outs,
                                            cudaStream_t s) {
  if (lt.ext) return linear_transform_ext_batch(xs, n, t, lt, outs, s);
  const size_t NN = (size_t)N, CT = (size_t)2 * t * NN;
  const int bs = lt.bs, gs = lt.gs;
  if (n <= 0) return cudaSuccess;
  if (t > lt.t || gs > kMaxJobs) return cudaErrorInvalidValue;
  const std::vector<int32_t> baby_r = lt.baby_rotations(N), giant_r = lt.giant_rotations(N);
  std::vector<int> active;  // giant steps with at least one diagonal
  for (int g = 0; g < gs; g++) {
    bool any = false;
    for (int b = 0; b < bs; b++) any = any || lt.present[(size_t)g * bs + b];
    if (any) active.push_back(g);
  }
  const size_t per = (size_t)(bs - 1 + 2 * gs);  // ciphertext slots of workspace per input
  u64* ws = alloc_limbs((size_t)2 * t * per * n, s);
  if (!ws) return cudaErrorMemoryAllocation;
  auto baby = [&](int i, int b) { return ws + ((size_t)i * per + (b - 1)) * CT; };   // b = 1..bs-1
  auto inner = [&](int i, int g) { return ws + ((size_t)i * per + (bs - 1) + g) * CT; };
  auto giant = [&](int i, int k) { return ws + ((size_t)i * per + (bs - 1) + gs + k) * CT; };
  cudaError_t err = cudaSuccess;
  {  // baby steps: rotations of every input by b*stride, one shared ModUp per input (a zero rotation is a copy)
    std::vector<KsReq> rq;
    for (int i = 0; i < n && err == cudaSuccess; i++)
      for (int b = 1; b < bs && err == cudaSuccess; b++) {
        if (baby_r[b - 1] == 0) {
          err = cudaMemcpyAsync(baby(i, b), xs[i], CT * sizeof(u64), cudaMemcpyDeviceToDevice, s);
          continue;
        }
        const uint32_t g = galois_for_index(N, baby_r[b - 1]);
        auto it = rot_keys.find(g);
        if (it == rot_keys.end()) err = cudaErrorInvalidValue;
        else rq.push_back({xs[i] + (size_t)t * NN, t, it->second, xs[i], nullptr, baby(i, b), galois_inverse(g)});
      }
    if (err == cudaSuccess) err = keyswitch_batch(rq.data(), (int)rq.size(), s);
  }
  if (err == cudaSuccess) {  // inner sums: one job per (input, chunk of kDotG giant steps)
    DotBatch db{};
    db.rot_stride = (long long)CT;
    db.out_stride = (long long)CT;
    db.pt_base = lt.diags;
    db.pt_stride = (long long)lt.rows * N;
    db.present = lt.present.data();
    db.bs = bs;
    db.t = t;
    err = inner_sums(db, n, gs, [&](int i) { return xs[i]; }, [&](int i) { return bs > 1 ? baby(i, 1) : nullptr; },
                     [&](int i, int g) { return inner(i, g); }, ring_, d_pc, s);
  }
  std::vector<int> nrot(n, 0);
  std::vector<std::vector<const u64*>> plain(n);
  if (err == cudaSuccess) {  // giant-step rotations of every input, one batch
    std::vector<KsReq> rq;
    for (int i = 0; i < n && err == cudaSuccess; i++)
      for (int g : active) {
        const u64* in = inner(i, g);
        if (giant_r[g] == 0) {
          plain[i].push_back(in);
          continue;
        }
        const uint32_t gl = galois_for_index(N, giant_r[g]);
        auto it = rot_keys.find(gl);
        if (it == rot_keys.end()) {
          err = cudaErrorInvalidValue;
          break;
        }
        rq.push_back({in + (size_t)t * NN, t, it->second, in, nullptr, giant(i, nrot[i]++), galois_inverse(gl)});
      }
    if (err == cudaSuccess) err = keyswitch_batch(rq.data(), (int)rq.size(), s);
  }
  // sums: rotated terms sit contiguously at giant(i, 0..); the first unrotated one is the sum's `first`
  // operand, further ones (offsets that coincide modulo N/2) are appended after the rotated terms
  SumBatch sb{};
  for (int i = 0; i < n && err == cudaSuccess; i++) {
    int k = nrot[i];
    for (size_t p = 1; p < plain[i].size() && err == cudaSuccess; p++, k++)
      err = cudaMemcpyAsync(giant(i, k), plain[i][p], CT * sizeof(u64), cudaMemcpyDeviceToDevice, s);
    if (err != cudaSuccess) break;
    if (k == 0 && plain[i].empty()) {
      err = cudaMemsetAsync(outs[i], 0, CT * sizeof(u64), s);
      continue;
    }
    sb.jobs[sb.njobs++] = SumJob{giant(i, 0), (long long)CT, k, plain[i].empty() ? nullptr : plain[i][0], outs[i], t};
    if (sb.njobs == kMaxJobs) {
      err = launch_sum(sb, ring_, d_pc, s);
      sb.njobs = 0;
    }
  }
  if (err == cudaSuccess && sb.njobs) err = launch_sum(sb, ring_, d_pc, s);
  free_limbs(ws, s);
  return err;
}

cudaError_t Context::linear_transform_ext_batch(const u64* const* xs, int n, int t, const DevLT& lt,
                                                u64* const* outs, cudaStream_t s) {
  const size_t NN = (size_t)N, E = (size_t)2 * (t + np) * NN;  // one ciphertext in the extended basis
  const int bs = lt.bs, gs = lt.gs;
  if (n <= 0) return cudaSuccess;
  if (t > lt.t || gs > kMaxJobs) return cudaErrorInvalidValue;
  const std::vector<int32_t> baby_r = lt.baby_rotations(N), giant_r = lt.giant_rotations(N);
  std::vector<int> active;  // giant steps with at least one diagonal
  for (int g = 0; g < gs; g++) {
    bool any = false;
    for (int b = 0; b < bs; b++) any = any || lt.present[(size_t)g * bs + b];
    if (any) active.push_back(g);
  }
  const int na = (int)active.size();
  // per input: bs baby ciphertexts (b = 0 is the input lifted by P), gs inner sums, na rotated sums, the total
  // (all extended), and na ModDowned c1 polys (t limbs each)
  const size_t per = (size_t)(bs + gs + na + 1) * E + (size_t)na * t * NN;
  u64* ws = alloc_limbs(per * n / NN, s);
  if (!ws) return cudaErrorMemoryAllocation;
  auto at = [&](int i) { return ws + (size_t)i * per; };
  auto baby = [&](int i, int b) { return at(i) + (size_t)b * E; };
  auto inner = [&](int i, int g) { return at(i) + (size_t)(bs + g) * E; };
  auto rotd = [&](int i, int k) { return at(i) + (size_t)(bs + gs + k) * E; };
  auto total = [&](int i) { return at(i) + (size_t)(bs + gs + na) * E; };
  auto c1d = [&](int i, int k) { return at(i) + (size_t)(bs + gs + na + 1) * E + (size_t)k * t * NN; };
  cudaError_t err = cudaSuccess;
  {  // b = 0: (P x0, P x1) on the Q rows, zero on the special rows
    KsBatch kb{};
    for (int i = 0; i < n && err == cudaSuccess; i++) {
      KsJob& j = kb.jobs[kb.njobs++];
      j.add0 = xs[i];
      j.add1 = xs[i] + (size_t)t * NN;
      j.out = baby(i, 0);
      j.t = t;
      j.galois_inv = 1;
      j.ext_mode = 1;
      if (kb.njobs == kMaxJobs || i == n - 1) {
        err = launch_ext_epilogue(kb, ring_, crt, d_pc, s);
        kb.njobs = 0;
      }
    }
  }
  if (err == cudaSuccess) {  // baby steps: one shared ModUp per input, no ModDown
    std::vector<KsReq> rq;
    for (int i = 0; i < n && err == cudaSuccess; i++)
      for (int b = 1; b < bs && err == cudaSuccess; b++) {
        if (baby_r[b - 1] == 0) {
          err = cudaMemcpyAsync(baby(i, b), baby(i, 0), E * sizeof(u64), cudaMemcpyDeviceToDevice, s);
          continue;
        }
        const uint32_t g = galois_for_index(N, baby_r[b - 1]);
        auto it = rot_keys.find(g);
        if (it == rot_keys.end()) {
          err = cudaErrorInvalidValue;
          break;
        }
        KsReq r{xs[i] + (size_t)t * NN, t, it->second, xs[i], nullptr, baby(i, b), galois_inverse(g)};
        r.ext_mode = 1;
        rq.push_back(r);
      }
    if (err == cudaSuccess) err = keyswitch_batch(rq.data(), (int)rq.size(), s);
  }
  if (err == cudaSuccess) {  // inner sums in the extended basis
    DotBatch db{};
    db.rot_stride = (long long)E;
    db.out_stride = (long long)E;
    db.pt_base = lt.diags;
    db.pt_stride = (long long)lt.rows * N;
    db.present = lt.present.data();
    db.bs = bs;
    db.t = t;
    db.np = np;
    db.nq = nq;
    db.pt_prow = lt.t;
    err = inner_sums(db, n, gs, [&](int i) { return baby(i, 0); },
                     [&](int i) { return bs > 1 ? baby(i, 1) : nullptr; }, [&](int i, int g) { return inner(i, g); },
                     ring_, d_pc, s);
  }
  // giant steps: ModDown of each sum's c1, then its rotation without ModDown (c0 stays extended)
  std::vector<int> nrot(n, 0);
  std::vector<std::vector<const u64*>> plain(n);
  std::vector<MdReq> md;
  std::vector<KsReq> rq;
  for (int i = 0; i < n && err == cudaSuccess; i++)
    for (int k = 0; k < na; k++) {
      const int g = active[k];
      if (giant_r[g] == 0) {
        plain[i].push_back(inner(i, g));
        continue;
      }
      const uint32_t gl = galois_for_index(N, giant_r[g]);
      auto it = rot_keys.find(gl);
      if (it == rot_keys.end()) {
        err = cudaErrorInvalidValue;
        break;
      }
      md.push_back(MdReq{inner(i, g) + (size_t)(t + np) * NN, t, 1, c1d(i, k)});
      KsReq r{c1d(i, k), t, it->second, inner(i, g), nullptr, rotd(i, nrot[i]++), galois_inverse(gl)};
      r.ext_mode = 2;
      rq.push_back(r);
    }
  if (err == cudaSuccess) err = moddown_batch(md.data(), (int)md.size(), s);
  if (err == cudaSuccess) err = keyswitch_batch(rq.data(), (int)rq.size(), s);
  // totals (rotated terms contiguous at rotd(i, 0..), the first unrotated one as `first`), then one ModDown each
  SumBatch sb{};
  sb.nq = nq;
  std::vector<MdReq> fin;
  for (int i = 0; i < n && err == cudaSuccess; i++) {
    int k = nrot[i];
    for (size_t p = 1; p < plain[i].size() && err == cudaSuccess; p++, k++)
      err = cudaMemcpyAsync(rotd(i, k), plain[i][p], E * sizeof(u64), cudaMemcpyDeviceToDevice, s);
    if (err != cudaSuccess) break;
    if (k == 0 && plain[i].empty()) {
      err = cudaMemsetAsync(outs[i], 0, (size_t)2 * t * NN * sizeof(u64), s);
      continue;
    }
    sb.jobs[sb.njobs++] = SumJob{rotd(i, 0), (long long)E, k, plain[i].empty() ? nullptr : plain[i][0], total(i), t,
                                 np};
    fin.push_back(MdReq{total(i), t, 2, outs[i]});
    if (sb.njobs == kMaxJobs) {
      err = launch_sum(sb, ring_, d_pc, s);
      sb.njobs = 0;
    }
  }
  if (err == cudaSuccess && sb.njobs) err = launch_sum(sb, ring_, d_pc, s);
  if (err == cudaSuccess) err = moddown_batch(fin.data(), (int)fin.size(), s);
  free_limbs(ws, s);
  return err;
}

cudaError_t Context::mult_monomial(const u64* x, int t, unsigned k, u64* out, cudaStream_t s) {
  MonoBatch mb{};
  mb.jobs[0] = MonoJob{x, out, t, k & (2u * N - 1)};
  mb.njobs = 1;
  return launch_monomial(mb, ring_, d_pc, psi_brev, s);
}

cudaError_t Context::mod_raise(const u64* x, int t_in, int T, u64* out, cudaStream_t s) {
  const size_t NN = (size_t)N;
  u64* ws = alloc_limbs(2, s);
  if (!ws) return cudaErrorMemoryAllocation;
  cudaError_t err;
  {
    NttQueue q(tabs, true, s);
    uint8_t pm[1] = {0};
    q.add(x, ws, (long long)t_in * N, N, 1, 2, pm);  // tower 0 of both polys to coefficient form
    q.flush();
    err = q.err;
  }
  if (err == cudaSuccess) {
    RaiseBatch rb{};
    rb.jobs[0] = RaiseJob{ws, out, T};
    rb.njobs = 1;
    err = launch_raise_switch(rb, ring_, d_pc, s);
  }
  if (err == cudaSuccess) err = ntt(out, out, 2, T, 0, (long long)T * N, false, s);
  (void)NN;
  free_limbs(ws, s);
  return err;
}

}  // namespace fgb
