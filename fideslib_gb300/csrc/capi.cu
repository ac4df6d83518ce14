// extern "C" boundary of the engine (declarations and contract: include/fideslib_gb300.h).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "../../include/fideslib_gb300.h"
#include "autoscale.hpp"
#include "engine.hpp"

struct fides_ctx {
  fgb::Context* c;
};

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char* where) {
  g_err = std::string(where) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? FIDES_ENOMEM : FIDES_ECUDA;
}

#define CK(call, where)                            \
  do {                                             \
    cudaError_t e_ = (call);                       \
    if (e_ != cudaSuccess) return cuda_fail(e_, where); \
  } while (0)

fgb::DevCt* find_ct(fides_ctx* ctx, uint32_t h) {
  auto it = ctx->c->cts.find(h);
  return it == ctx->c->cts.end() ? nullptr : &it->second;
}

fgb::DevPt* find_pt(fides_ctx* ctx, uint32_t h) {
  auto it = ctx->c->pts.find(h);
  return it == ctx->c->pts.end() ? nullptr : &it->second;
}

uint32_t register_ct(fides_ctx* ctx, const fgb::DevCt& ct) {
  uint32_t h = ctx->c->next_handle++;
  if (ctx->c->next_handle == 0) ctx->c->next_handle = 1;
  ctx->c->cts[h] = ct;
  return h;
}

int new_ct(fides_ctx* ctx, int t, const fgb::DevCt& like, fgb::DevCt* out) {
  *out = like;
  out->t = t;
  out->data = ctx->c->alloc_limbs((size_t)2 * t, ctx->c->stream);
  if (!out->data) return fail(FIDES_ENOMEM, "ciphertext allocation failed");
  return FIDES_OK;
}

bool valid_ctx(fides_ctx* ctx) { return ctx && ctx->c; }

// The ModUp kernel keeps one digit's towers in registers: at most 32 towers per digit.
int check_ks_shape(fides_ctx* ctx) {
  if (ctx->c->alpha > 32) return fail(FIDES_EINVAL, "key switching supports at most 32 towers per digit (raise dnum)");
  return FIDES_OK;
}

// Opt-in validation of a freshly loaded object (fides_ctx_set_input_check): every residue below its prime.
int check_loaded(fgb::Context* c, const fgb::u64* x, long long rows, int period, int tq, const char* what) {
  if (!c->input_check) return FIDES_OK;
  const int r = c->residues_out_of_range(x, rows, period, tq);
  if (r < 0) return fail(FIDES_ECUDA, std::string(what) + ": residue check failed");
  if (r > 0) return fail(FIDES_EINVAL, std::string(what) + " has a residue that is not below its tower's prime");
  return FIDES_OK;
}

}  // namespace

namespace fgb {
// Lets other translation units of the library report through fides_last_error().
int set_last_error(int code, const char* msg) { return fail(code, msg); }
// For the request server: makes `s` the stream that later calls on ctx order their work on and returns the
// previous one, without synchronising it (fides_ctx_set_stream does); the caller orders the two streams itself.
cudaStream_t swap_ctx_stream(fides_ctx* ctx, cudaStream_t s) {
  cudaStream_t old = ctx->c->stream;
  ctx->c->stream = s;
  return old;
}
}  // namespace fgb

extern "C" {

const char* fides_last_error(void) { return g_err.c_str(); }
const char* fides_version(void) { return "fideslib_gb300 0.1 (sm_103a)"; }

int fides_ctx_ntt_tuning(fides_ctx* ctx, int32_t* variant, float* ms) {
  if (!valid_ctx(ctx)) return fail(FIDES_EINVAL, "null context");
  const fgb::DeviceTables& t = ctx->c->tabs;
  if (variant) {
    variant[0] = t.fwd_variant_tiny;
    variant[1] = t.fwd_variant_small;
    variant[2] = t.fwd_variant;
    variant[3] = t.inv_variant_tiny;
    variant[4] = t.inv_variant_small;
    variant[5] = t.inv_variant;
  }
  if (ms)
    for (int i = 0; i < fgb::kNttSizeClasses * (fgb::kNttFwdVariants + fgb::kNttInvVariants); i++)
      ms[i] = ctx->c->ntt_tune_ms[i];
  return FIDES_OK;
}

int fides_ctx_ks_tuning(fides_ctx* ctx, int32_t* iters, float* ms) {
  if (!valid_ctx(ctx)) return fail(FIDES_EINVAL, "null context");
  if (iters) *iters = ctx->c->crt.ks_iters > 0 ? ctx->c->crt.ks_iters : std::min(4, ctx->c->N / 512);
  if (ms)
    for (int v = 0; v < fgb::Context::kKsTileVariants; v++) ms[v] = ctx->c->ks_tune_ms[v];
  return FIDES_OK;
}

int fides_ctx_ks_tuning_set(fides_ctx* ctx, int32_t iters) {
  if (!valid_ctx(ctx)) return fail(FIDES_EINVAL, "null context");
  if ((iters != 1 && iters != 2 && iters != 4 && iters != 8 && iters != 16) || iters > ctx->c->N / 512)
    return fail(FIDES_EINVAL, "coefficient pairs per thread must be 1, 2, 4, 8 or 16 and at most N / 512");
  cudaStreamSynchronize(ctx->c->stream);
  ctx->c->crt.ks_iters = iters;
  ctx->c->ks_tuned = true;  // no later tuning overrides the caller's choice
  return FIDES_OK;
}

int fides_ctx_set_mem_limit(fides_ctx* ctx, uint64_t bytes) {
  if (!valid_ctx(ctx)) return fail(FIDES_EINVAL, "null context");
  ctx->c->mem_limit = (size_t)bytes;
  return FIDES_OK;
}

int fides_ctx_mem_in_use(fides_ctx* ctx, uint64_t* bytes) {
  if (!valid_ctx(ctx) || !bytes) return fail(FIDES_EINVAL, "null argument");
  *bytes = ctx->c->mem_in_use;
  return FIDES_OK;
}

int fides_ctx_set_input_check(fides_ctx* ctx, int enable) {
  if (!valid_ctx(ctx)) return fail(FIDES_EINVAL, "null context");
  ctx->c->input_check = enable != 0;
  return FIDES_OK;
}

int fides_ctx_ntt_tuning_set(fides_ctx* ctx, int32_t fwd_variant, int32_t inv_variant) {
  if (!valid_ctx(ctx)) return fail(FIDES_EINVAL, "null context");
  if (fwd_variant < 0 || fwd_variant >= fgb::kNttFwdVariants || inv_variant < 0 ||
      inv_variant >= fgb::kNttInvVariants)
    return fail(FIDES_EINVAL, "forward and inverse variants must be 0, 1 or 2");
  if (ctx->c->logN < 13 && (fwd_variant != 1 || inv_variant != 0))
    return fail(FIDES_EINVAL, "below N = 2^13 only forward variant 1 and inverse variant 0 exist");
  cudaStreamSynchronize(ctx->c->stream);
  fgb::DeviceTables& t = ctx->c->tabs;
  t.fwd_variant = t.fwd_variant_small = t.fwd_variant_tiny = fwd_variant;
  t.inv_variant = t.inv_variant_small = t.inv_variant_tiny = t.inv_variant_ks = inv_variant;
  return FIDES_OK;
}

int fides_find_primes(uint32_t bits, uint32_t count, uint64_t two_n, const uint64_t* exclude, uint32_t nexclude,
                      uint64_t* out) {
  if (!out || bits < 2 || bits > 62 || two_n < 2) return 0;
  typedef unsigned __int128 u128;
  auto mulmod = [](uint64_t a, uint64_t b, uint64_t m) { return (uint64_t)((u128)a * b % m); };
  auto powmod = [&](uint64_t a, uint64_t e, uint64_t m) {
    uint64_t r = 1 % m;
    for (a %= m; e; e >>= 1, a = mulmod(a, a, m))
      if (e & 1) r = mulmod(r, a, m);
    return r;
  };
  auto is_prime = [&](uint64_t n) {
    if (n < 2) return false;
    for (uint64_t q : {2ull, 3ull, 5ull, 7ull, 11ull, 13ull, 17ull, 19ull, 23ull, 29ull, 31ull, 37ull})
      if (n % q == 0) return n == q;
    uint64_t d = n - 1;
    int r = 0;
    while (!(d & 1)) {
      d >>= 1;
      r++;
    }
    for (uint64_t a : {2ull, 325ull, 9375ull, 28178ull, 450775ull, 9780504ull, 1795265022ull}) {
      if (!(a %= n)) continue;
      uint64_t x = powmod(a, d, n);
      if (x == 1 || x == n - 1) continue;
      bool comp = true;
      for (int k = 1; k < r && comp; k++)
        if ((x = mulmod(x, x, n)) == n - 1) comp = false;
      if (comp) return false;
    }
    return true;
  };
  const uint64_t top = (1ull << bits) - 1;
  uint64_t c = top - top % two_n + 1;
  if (c > top) c -= two_n;
  uint32_t found = 0;
  for (; found < count && c > two_n; c -= two_n) {
    bool skip = false;
    for (uint32_t i = 0; i < nexclude && !skip; i++) skip = exclude[i] == c;
    for (uint32_t i = 0; i < found && !skip; i++) skip = out[i] == c;
    if (!skip && is_prime(c)) out[found++] = c;
  }
  return (int)found;
}

int fides_ctx_create(const fides_params* p, fides_ctx** out) {
  if (!p || !out || !p->moduli) return fail(FIDES_EINVAL, "null argument");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return fail(FIDES_ENODEV, "no CUDA device");
  std::string err;
  fgb::Context* c = fgb::Context::create((int)p->log_n, (int)p->nq, (int)p->np, (int)p->dnum, (const fgb::u64*)p->moduli,
                                                (const fgb::u64*)p->roots, &err);
  if (!c) return fail(FIDES_EINVAL, err);
  if (c->set_scaling(p->scaling_technique, p->scaling_factor_real, p->scaling_factor_real_big, p->mod_reduce_factor,
                     p->default_scale, &err) != FIDES_OK) {
    delete c;
    return fail(FIDES_EINVAL, err);
  }
  *out = new fides_ctx{c};
  return FIDES_OK;
}

int fides_ctx_scaling(const fides_ctx* ctx, int32_t* technique, double* sf, double* big, double* mrf) {
  if (!ctx || !ctx->c) return fail(FIDES_EINVAL, "null context");
  const fgb::Context* c = ctx->c;
  if (technique) *technique = c->technique;
  for (int l = 0; l < c->nq; l++) {
    if (sf) sf[l] = c->sf[l];
    if (big) big[l] = c->big[l];
    if (mrf) mrf[l] = c->mrf[l];
  }
  return FIDES_OK;
}

int fides_ctx_destroy(fides_ctx* ctx) {
  if (!ctx) return FIDES_OK;
  delete ctx->c;
  delete ctx;
  return FIDES_OK;
}

int fides_ctx_moduli(const fides_ctx* ctx, uint64_t* moduli, uint64_t* roots) {
  if (!ctx || !ctx->c) return fail(FIDES_EINVAL, "null context");
  const fgb::Context* c = ctx->c;
  for (int i = 0; i < c->ntow; i++) {
    if (moduli) moduli[i] = c->mod[i];
    if (roots) roots[i] = c->psi[i];
  }
  return FIDES_OK;
}

int fides_ctx_get_shape(const fides_ctx* ctx, fides_ctx_shape* shape) {
  if (!ctx || !ctx->c || !shape) return fail(FIDES_EINVAL, "null argument");
  const fgb::Context* c = ctx->c;
  *shape = fides_ctx_shape{(uint32_t)c->N, (uint32_t)c->logN, (uint32_t)c->nq, (uint32_t)c->np, (uint32_t)c->dnum,
                           (uint32_t)c->alpha};
  return FIDES_OK;
}

uint32_t fides_galois_element(const fides_ctx* ctx, int32_t index) {
  if (!ctx || !ctx->c) return 0;
  return fgb::Context::galois_for_index(ctx->c->N, index);
}

int fides_synchronize(fides_ctx* ctx) {
  if (!valid_ctx(ctx)) return fail(FIDES_EINVAL, "null context");
  CK(cudaStreamSynchronize(ctx->c->stream), "synchronize");
  return FIDES_OK;
}

void* fides_ctx_stream(fides_ctx* ctx) { return valid_ctx(ctx) ? (void*)ctx->c->stream : nullptr; }

int fides_ctx_set_stream(fides_ctx* ctx, void* stream) {
  if (!valid_ctx(ctx)) return fail(FIDES_EINVAL, "null context");
  fgb::Context* c = ctx->c;
  CK(cudaStreamSynchronize(c->stream), "set stream");
  c->stream = stream ? (cudaStream_t)stream : c->own_stream;
  return FIDES_OK;
}

uint64_t fides_kernel_launches(void) { return fgb::launch_count(); }

int fides_ntt_batch_device(fides_ctx* ctx, uint64_t* data, uint32_t npolys, uint32_t limbs, uint32_t first_prime,
                           int inverse, void* stream) {
  if (!valid_ctx(ctx) || !data) return fail(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  if (limbs == 0 || npolys == 0) return FIDES_OK;
  if (limbs > 64 || first_prime + limbs > (uint32_t)c->ntow) return fail(FIDES_EINVAL, "tower range out of bounds");
  if ((uintptr_t)data % 16) return fail(FIDES_EINVAL, "device data must be 16-byte aligned");
  cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
  CK(c->ntt((const fgb::u64*)data, (fgb::u64*)data, (int)npolys, (int)limbs, (int)first_prime, (long long)limbs * c->N, inverse != 0, s),
     "ntt launch");
  return FIDES_OK;
}

int fides_ntt_batch_host(fides_ctx* ctx, uint64_t* data, uint32_t npolys, uint32_t limbs, uint32_t first_prime,
                         int inverse) {
  if (!valid_ctx(ctx) || !data) return fail(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  const size_t bytes = (size_t)npolys * limbs * c->N * sizeof(uint64_t);
  if (bytes == 0) return FIDES_OK;
  fgb::u64* d = c->alloc_limbs((size_t)npolys * limbs, c->stream);
  if (!d) return fail(FIDES_ENOMEM, "device allocation failed");
  CK(cudaMemcpyAsync(d, data, bytes, cudaMemcpyHostToDevice, c->stream), "H2D");
  int rc = fides_ntt_batch_device(ctx, (uint64_t*)d, npolys, limbs, first_prime, inverse, c->stream);
  if (rc == FIDES_OK) {
    CK(cudaMemcpyAsync(data, d, bytes, cudaMemcpyDeviceToHost, c->stream), "D2H");
  }
  c->free_limbs(d, c->stream);
  CK(cudaStreamSynchronize(c->stream), "synchronize");
  return rc;
}

// A key refused by the input check is not loaded: its slot is freed and left null (the caller drops the entry).
static int load_key(fides_ctx* ctx, const uint64_t* key, bool device, fgb::u64** slot) {
  fgb::Context* c = ctx->c;
  const size_t bytes = (size_t)2 * c->dnum * c->ntow * c->N * sizeof(uint64_t);
  if (!*slot) {
    void* p = nullptr;
    CK(cudaMalloc(&p, bytes), "key allocation");
    *slot = (fgb::u64*)p;
  }
  CK(cudaMemcpyAsync(*slot, key, bytes, device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->stream),
     "key copy");
  if (int rc = check_loaded(c, *slot, (long long)2 * c->dnum * c->ntow, c->ntow, c->ntow, "key")) {
    cudaFree(*slot);
    *slot = nullptr;
    return rc;
  }
  CK(fgb::launch_key_split(*slot, bytes / sizeof(uint64_t), c->stream), "key layout");
  CK(cudaStreamSynchronize(c->stream), "key copy");
  return FIDES_OK;
}

int fides_load_eval_mult_key(fides_ctx* ctx, const uint64_t* key) {
  if (!valid_ctx(ctx) || !key) return fail(FIDES_EINVAL, "null argument");
  return load_key(ctx, key, false, &ctx->c->relin_key);
}

int fides_load_eval_mult_key_device(fides_ctx* ctx, const uint64_t* dev_key) {
  if (!valid_ctx(ctx) || !dev_key) return fail(FIDES_EINVAL, "null argument");
  return load_key(ctx, dev_key, true, &ctx->c->relin_key);
}

int fides_load_rotation_key(fides_ctx* ctx, uint32_t galois, const uint64_t* key) {
  if (!valid_ctx(ctx) || !key) return fail(FIDES_EINVAL, "null argument");
  if ((galois & 1) == 0 || galois >= 2u * ctx->c->N) return fail(FIDES_EINVAL, "Galois element must be odd and < 2N");
  fgb::u64*& slot = ctx->c->rot_keys[galois];
  const int rc = load_key(ctx, key, false, &slot);
  if (!slot) ctx->c->rot_keys.erase(galois);
  return rc;
}

int fides_load_rotation_key_device(fides_ctx* ctx, uint32_t galois, const uint64_t* dev_key) {
  if (!valid_ctx(ctx) || !dev_key) return fail(FIDES_EINVAL, "null argument");
  if ((galois & 1) == 0 || galois >= 2u * ctx->c->N) return fail(FIDES_EINVAL, "Galois element must be odd and < 2N");
  fgb::u64*& slot = ctx->c->rot_keys[galois];
  const int rc = load_key(ctx, dev_key, true, &slot);
  if (!slot) ctx->c->rot_keys.erase(galois);
  return rc;
}

// Switch keys share the rotation-key table under tagged ids that no Galois element (< 2N <= 2^17) can take.
constexpr uint32_t kSwitchKeyTag = 0x80000000u;

int fides_load_switch_key(fides_ctx* ctx, uint32_t key_id, const uint64_t* key) {
  if (!valid_ctx(ctx) || !key) return fail(FIDES_EINVAL, "null argument");
  if (key_id & kSwitchKeyTag) return fail(FIDES_EINVAL, "switch key id must be < 2^31");
  fgb::u64*& slot = ctx->c->rot_keys[kSwitchKeyTag | key_id];
  const int rc = load_key(ctx, key, false, &slot);
  if (!slot) ctx->c->rot_keys.erase(kSwitchKeyTag | key_id);
  return rc;
}

int fides_load_switch_key_device(fides_ctx* ctx, uint32_t key_id, const uint64_t* dev_key) {
  if (!valid_ctx(ctx) || !dev_key) return fail(FIDES_EINVAL, "null argument");
  if (key_id & kSwitchKeyTag) return fail(FIDES_EINVAL, "switch key id must be < 2^31");
  fgb::u64*& slot = ctx->c->rot_keys[kSwitchKeyTag | key_id];
  const int rc = load_key(ctx, dev_key, true, &slot);
  if (!slot) ctx->c->rot_keys.erase(kSwitchKeyTag | key_id);
  return rc;
}

static int ct_load_impl(fides_ctx* ctx, const uint64_t* data, const fides_ct_meta* meta, uint32_t* handle,
                        bool device) {
  if (!valid_ctx(ctx) || !data || !meta || !handle) return fail(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  if (meta->towers < 1 || meta->towers > (uint32_t)c->nq) return fail(FIDES_EINVAL, "towers out of range");
  fgb::DevCt ct;
  ct.t = (int)meta->towers;
  ct.scale = meta->scale;
  ct.noise_deg = (int)meta->noise_deg;
  ct.slots = (int)meta->slots;
  ct.data = c->alloc_limbs((size_t)2 * ct.t, c->stream);
  if (!ct.data) return fail(FIDES_ENOMEM, "ciphertext allocation failed");
  CK(cudaMemcpyAsync(ct.data, data, (size_t)2 * ct.t * c->N * sizeof(uint64_t),
                     device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->stream),
     "ciphertext copy");
  if (int rc = check_loaded(c, ct.data, 2 * ct.t, ct.t, ct.t, "ciphertext")) {
    c->free_limbs(ct.data, c->stream);
    return rc;
  }
  *handle = register_ct(ctx, ct);
  return FIDES_OK;
}

int fides_ct_load(fides_ctx* ctx, const uint64_t* data, const fides_ct_meta* meta, uint32_t* handle) {
  return ct_load_impl(ctx, data, meta, handle, false);
}

int fides_ct_load_device(fides_ctx* ctx, const uint64_t* dev_data, const fides_ct_meta* meta, uint32_t* handle) {
  return ct_load_impl(ctx, dev_data, meta, handle, true);
}

int fides_ct_meta_get(fides_ctx* ctx, uint32_t handle, fides_ct_meta* meta) {
  if (!valid_ctx(ctx) || !meta) return fail(FIDES_EINVAL, "null argument");
  fgb::DevCt* ct = find_ct(ctx, handle);
  bool ext = false;
  if (!ct) {
    auto it = ctx->c->ext_cts.find(handle);
    if (it == ctx->c->ext_cts.end()) return fail(FIDES_EINVAL, "unknown ciphertext handle");
    ct = &it->second;
    ext = true;
  }
  meta->towers = (uint32_t)ct->t;
  meta->noise_deg = (uint32_t)ct->noise_deg;
  meta->slots = (uint32_t)ct->slots;
  meta->reserved = ext ? (uint32_t)ctx->c->np : 0;
  meta->scale = ct->scale;
  return FIDES_OK;
}

int fides_ct_store(fides_ctx* ctx, uint32_t handle, uint64_t* data, fides_ct_meta* meta) {
  if (!valid_ctx(ctx) || !data) return fail(FIDES_EINVAL, "null argument");
  fgb::DevCt* ct = find_ct(ctx, handle);
  if (!ct) return fail(FIDES_EINVAL, "unknown ciphertext handle");
  fgb::Context* c = ctx->c;
  CK(cudaMemcpyAsync(data, ct->data, (size_t)2 * ct->t * c->N * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                     c->stream),
     "ciphertext store");
  CK(cudaStreamSynchronize(c->stream), "ciphertext store");
  if (meta) return fides_ct_meta_get(ctx, handle, meta);
  return FIDES_OK;
}

int fides_ct_free(fides_ctx* ctx, uint32_t handle) {
  if (!valid_ctx(ctx)) return fail(FIDES_EINVAL, "null context");
  for (auto* map : {&ctx->c->cts, &ctx->c->ext_cts}) {
    auto it = map->find(handle);
    if (it == map->end()) continue;
    ctx->c->free_limbs(it->second.data, ctx->c->stream);
    map->erase(it);
    return FIDES_OK;
  }
  return fail(FIDES_EINVAL, "unknown ciphertext handle");
}

// Plaintext jobs, kMaxJobs per launch.
static cudaError_t launch_plain_jobs(fgb::Context* c, const fgb::PtJob* jobs, size_t n) {
  const fgb::Ring ring{c->N, c->logN};
  for (size_t k0 = 0; k0 < n; k0 += fgb::kMaxJobs) {
    fgb::PtBatch pb{};
    pb.njobs = (int)std::min(n - k0, (size_t)fgb::kMaxJobs);
    for (int k = 0; k < pb.njobs; k++) pb.jobs[k] = jobs[k0 + k];
    const cudaError_t e = fgb::launch_ptop(pb, ring, c->d_pc, c->stream);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Validates one request and prepares its output ciphertext; the compute is issued by run_batch.
struct Pending {
  fgb::DevCt out;
  const fgb::DevCt* a = nullptr;
  const fgb::DevCt* b = nullptr;
  const fgb::DevPt* pt = nullptr;  // *_PLAIN requests
  uint32_t galois_inv = 1;  // automorphism applied after the key switch (1 = none)
  const fgb::u64* key = nullptr;
};

// Aligned operands (AutoScaler: the scaling technique's adjustments, or the FIXEDMANUAL tower cut) replace the
// registered ones when given.
static int prepare(fides_ctx* ctx, const fides_op& op, Pending* pd, const fgb::DevCt* Aov = nullptr,
                   const fgb::DevCt* Bov = nullptr) {
  fgb::Context* c = ctx->c;
  const fgb::DevCt* A = Aov ? Aov : find_ct(ctx, op.a);
  if (!A) return fail(FIDES_EINVAL, "unknown ciphertext handle " + std::to_string(op.a));
  const fgb::DevCt* B = nullptr;
  if (op.op == FIDES_OP_ADD || op.op == FIDES_OP_SUB || op.op == FIDES_OP_MULT) {
    B = Bov ? Bov : find_ct(ctx, op.b);
    if (!B) return fail(FIDES_EINVAL, "unknown ciphertext handle " + std::to_string(op.b));
    if (A->t != B->t) return fail(FIDES_EINVAL, "operands have different tower counts");
  }
  const bool plain = op.op == FIDES_OP_MULT_PLAIN || op.op == FIDES_OP_ADD_PLAIN || op.op == FIDES_OP_SUB_PLAIN;
  if (plain) {
    pd->pt = find_pt(ctx, op.b);
    if (!pd->pt) return fail(FIDES_EINVAL, "unknown plaintext handle " + std::to_string(op.b));
    if (pd->pt->t < A->t) return fail(FIDES_EINVAL, "plaintext has fewer towers than the ciphertext");
  }
  pd->a = A;
  pd->b = B;
  int t_out = A->t;
  fgb::DevCt meta = *A;
  switch (op.op) {
    case FIDES_OP_ADD:
    case FIDES_OP_SUB:
      meta.noise_deg = A->noise_deg > B->noise_deg ? A->noise_deg : B->noise_deg;
      break;
    case FIDES_OP_MULT:
    case FIDES_OP_SQUARE: {
      if (!c->relin_key) return fail(FIDES_ENOKEY, "no relinearisation key loaded");
      if (int rc = check_ks_shape(ctx)) return rc;
      const fgb::DevCt* Y = op.op == FIDES_OP_SQUARE ? A : B;
      meta.noise_deg = A->noise_deg + Y->noise_deg;
      meta.scale = A->scale * Y->scale;
      pd->b = Y;
      break;
    }
    case FIDES_OP_MULT_PLAIN:
      meta.scale = A->scale * pd->pt->scale;
      meta.noise_deg = A->noise_deg + 1;
      break;
    case FIDES_OP_ADD_PLAIN:
    case FIDES_OP_SUB_PLAIN:
      break;
    case FIDES_OP_RESCALE:
      if (A->t < 2) return fail(FIDES_EINVAL, "cannot rescale a ciphertext with one tower");
      t_out = A->t - 1;
      meta.noise_deg = A->noise_deg > 1 ? A->noise_deg - 1 : 1;
      meta.scale = A->scale / (double)c->mod[A->t - 1];
      break;
    case FIDES_OP_ROTATE:
    case FIDES_OP_AUTOMORPHISM:
    case FIDES_OP_KEY_SWITCH: {
      const bool ks = op.op == FIDES_OP_KEY_SWITCH;
      if (ks && ((uint32_t)op.index & kSwitchKeyTag)) return fail(FIDES_EINVAL, "switch key id must be < 2^31");
      if (op.op == FIDES_OP_AUTOMORPHISM && (((uint32_t)op.index & 1) == 0 || (uint32_t)op.index >= 2u * c->N))
        return fail(FIDES_EINVAL, "Galois element must be odd and < 2N");
      uint32_t g = op.op == FIDES_OP_ROTATE ? c->rotation_key_galois(op.index, A->slots)
                   : ks                     ? kSwitchKeyTag | (uint32_t)op.index
                                            : (uint32_t)op.index;
      if (op.op == FIDES_OP_ROTATE && g == 0)
        return fail(FIDES_ENOKEY, "no rotation key for index " + std::to_string(op.index) + " (Galois element " +
                                      std::to_string(fgb::Context::galois_for_index(c->N, op.index)) + ")");
      auto it = c->rot_keys.find(g);
      if (it == c->rot_keys.end())
        return fail(FIDES_ENOKEY, ks ? "no switch key with id " + std::to_string(op.index)
                                     : "no rotation key for Galois element " + std::to_string(g));
      if (int rc = check_ks_shape(ctx)) return rc;
      pd->galois_inv = ks ? 1u : c->galois_inverse(g);
      pd->key = it->second;
      break;
    }
    default:
      return fail(FIDES_EINVAL, "unknown op code " + std::to_string(op.op));
  }
  meta.t = t_out;
  meta.data = c->alloc_limbs((size_t)2 * t_out, c->stream);
  if (!meta.data) return fail(FIDES_ENOMEM, "ciphertext allocation failed");
  pd->out = meta;
  return FIDES_OK;
}

// Runs a set of independent requests as one batch per op family: every ciphertext of a family goes through
// each pipeline stage in a single launch.
// align = false skips the operand alignment (the engine's own composites, which keep their operands at matching
// levels and scales themselves).
static int run_batch(fides_ctx* ctx, fides_op* ops, uint32_t n, bool align = true) {
  fgb::Context* c = ctx->c;
  std::vector<Pending> pd(n);
  // Operand alignment first (its temporaries live until the batch's launches are queued, then are freed
  // stream-ordered): binary ops whose operands differ in towers, or any operand under an automatic technique.
  fgb::AutoScaler scaler(c, c->stream);
  std::vector<fgb::DevCt> adj_a(n), adj_b(n);
  std::vector<char> adjusted(n, 0);
  for (uint32_t i = 0; i < n; i++) {
    const int code = ops[i].op;
    const bool binary = code == FIDES_OP_ADD || code == FIDES_OP_SUB || code == FIDES_OP_MULT;
    const bool unary = code == FIDES_OP_SQUARE || code == FIDES_OP_MULT_PLAIN;
    if (!align || (!binary && !(unary && c->technique != FIDES_FIXEDMANUAL))) continue;
    const fgb::DevCt* A = find_ct(ctx, ops[i].a);
    const fgb::DevCt* B = binary ? find_ct(ctx, ops[i].b) : nullptr;
    if (!A || (binary && !B)) continue;  // prepare() reports the unknown handle
    if (binary && c->technique == FIDES_FIXEDMANUAL && A->t == B->t) continue;
    adj_a[i] = *A;
    int rc = FIDES_OK;
    if (binary) {
      adj_b[i] = *B;
      rc = scaler.prepare_binary(code, adj_a[i], adj_b[i]);
    } else {
      rc = scaler.prepare_unary(adj_a[i]);
    }
    if (rc) return rc;
    adjusted[i] = 1;
  }
  for (uint32_t i = 0; i < n; i++) {
    int rc = adjusted[i] ? prepare(ctx, ops[i], &pd[i], &adj_a[i], ops[i].op == FIDES_OP_SQUARE ||
                                                                       ops[i].op == FIDES_OP_MULT_PLAIN
                                                                   ? nullptr
                                                                   : &adj_b[i])
                         : prepare(ctx, ops[i], &pd[i]);
    if (rc) {
      for (uint32_t k = 0; k < i; k++) c->free_limbs(pd[k].out.data, c->stream);
      return rc;
    }
  }
  std::vector<fgb::Context::AddReq> adds;
  std::vector<fgb::Context::MultReq> mults;
  std::vector<fgb::Context::RescaleReq> rescales;
  std::vector<fgb::Context::KsReq> rots;
  std::vector<fgb::PtJob> ptops;
  const size_t NN = (size_t)c->N;
  for (uint32_t i = 0; i < n; i++) {
    const Pending& p = pd[i];
    const int t = p.a->t;
    switch (ops[i].op) {
      case FIDES_OP_ADD:
      case FIDES_OP_SUB:
        adds.push_back({p.a->data, p.b->data, t, p.out.data, ops[i].op == FIDES_OP_SUB});
        break;
      case FIDES_OP_MULT:
      case FIDES_OP_SQUARE:
        mults.push_back({p.a->data, p.b->data, t, p.out.data});
        break;
      case FIDES_OP_RESCALE:
        rescales.push_back({p.a->data, t, p.out.data});
        break;
      case FIDES_OP_MULT_PLAIN:
      case FIDES_OP_ADD_PLAIN:
      case FIDES_OP_SUB_PLAIN:
        ptops.push_back({p.a->data, p.pt->data, p.out.data, t, ops[i].op - FIDES_OP_MULT_PLAIN});
        break;
      default:
        rots.push_back({p.a->data + (size_t)t * NN, t, p.key, p.a->data, nullptr, p.out.data, p.galois_inv});
    }
  }
  cudaError_t e = c->add_batch(adds.data(), (int)adds.size(), c->stream);
  if (e == cudaSuccess) e = launch_plain_jobs(c, ptops.data(), ptops.size());
  if (e == cudaSuccess) e = c->rescale_batch(rescales.data(), (int)rescales.size(), c->stream);
  if (e == cudaSuccess) e = c->mult_batch(mults.data(), (int)mults.size(), c->relin_key, c->stream);
  if (e == cudaSuccess) e = c->keyswitch_batch(rots.data(), (int)rots.size(), c->stream);
  if (e != cudaSuccess) {
    for (uint32_t k = 0; k < n; k++) c->free_limbs(pd[k].out.data, c->stream);
    return cuda_fail(e, "batch");
  }
  for (uint32_t i = 0; i < n; i++) ops[i].out = register_ct(ctx, pd[i].out);
  return FIDES_OK;
}

// Pipelined batch from and to host memory: chunk k's inputs are copied in on one stream while earlier chunks compute
// and chunk k-2's results are copied out on another, so the copy engines run beside the kernels.  Consecutive
// chunks compute on two streams (the context stream and chunk_alt), so one chunk's launches fill the SMs that the
// other's leave idle.  Inputs and outputs must be pinned host memory for the copies to be asynchronous.  Device
// memory comes from the stream-ordered pool, whose reuse across the streams follows their event dependencies.
int fides_eval_batch_host(fides_ctx* ctx, fides_host_op* ops, uint32_t n, uint32_t chunk) {
  if (!valid_ctx(ctx) || (!ops && n)) return fail(FIDES_EINVAL, "null argument");
  if (n == 0) return FIDES_OK;
  fgb::Context* c = ctx->c;
  for (uint32_t i = 0; i < n; i++) {
    const fides_host_op& o = ops[i];
    const bool binary = o.op == FIDES_OP_ADD || o.op == FIDES_OP_SUB || o.op == FIDES_OP_MULT;
    if (!o.a || !o.out || (binary && !o.b)) return fail(FIDES_EINVAL, "null host buffer in request " + std::to_string(i));
    if (o.op == FIDES_OP_BOOTSTRAP) return fail(FIDES_EINVAL, "bootstrap requests go through the server");
    if (o.op >= FIDES_OP_MULT_PLAIN && o.op <= FIDES_OP_SUB_PLAIN)
      return fail(FIDES_EINVAL, "plaintext requests take resident plaintext handles: use fides_eval_batch");
    if (o.meta.towers < 1 || o.meta.towers > (uint32_t)c->nq) return fail(FIDES_EINVAL, "towers out of range");
  }
  if (!c->copy_in) CK(cudaStreamCreateWithFlags(&c->copy_in, cudaStreamNonBlocking), "copy stream");
  if (!c->copy_out) CK(cudaStreamCreateWithFlags(&c->copy_out, cudaStreamNonBlocking), "copy stream");
  if (!c->chunk_alt) CK(cudaStreamCreateWithFlags(&c->chunk_alt, cudaStreamNonBlocking), "compute stream");
  const size_t limb = (size_t)c->N * sizeof(uint64_t);
  cudaStream_t const main_stream = c->stream;
  std::vector<cudaEvent_t> events;
  auto event = [&]() {
    cudaEvent_t e;
    cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    events.push_back(e);
    return e;
  };
  int rc = FIDES_OK;
  std::vector<fides_op> fo(n);
  std::vector<uint32_t> bounds{0};  // chunk k = requests bounds[k] .. bounds[k+1]-1
  if (chunk == 0 && n >= 16) {      // automatic: chunks of 8, the first and the last of 4 (shorter fill and drain)
    bounds.push_back(4);
    while (bounds.back() + 12 <= n) bounds.push_back(bounds.back() + 8);
    if (n - bounds.back() > 4) bounds.push_back(n - 4);
    bounds.push_back(n);
  } else {
    const uint32_t c = chunk ? chunk : n;
    for (uint32_t k = c; k < n; k += c) bounds.push_back(k);
    bounds.push_back(n);
  }
  {  // the second compute stream starts after the work already queued on the context stream
    cudaEvent_t ev0 = event();
    cudaEventRecord(ev0, main_stream);
    cudaStreamWaitEvent(c->chunk_alt, ev0, 0);
  }
  for (size_t ci = 0; ci + 1 < bounds.size() && rc == FIDES_OK; ci++) {
    const uint32_t k0 = bounds[ci], k1 = bounds[ci + 1];
    c->stream = (ci & 1) ? c->chunk_alt : main_stream;  // every call below orders its work on this chunk's stream
    // copy in (input handles are registered now; their memory is ready once ev_in has passed)
    std::vector<uint32_t> inputs;
    for (uint32_t i = k0; i < k1 && rc == FIDES_OK; i++) {
      const fides_host_op& o = ops[i];
      const bool binary = o.op == FIDES_OP_ADD || o.op == FIDES_OP_SUB || o.op == FIDES_OP_MULT;
      uint32_t hab[2] = {0, 0};
      for (int w = 0; w < (binary ? 2 : 1) && rc == FIDES_OK; w++) {
        fgb::DevCt ct;
        ct.t = (int)o.meta.towers;
        ct.scale = o.meta.scale;
        ct.noise_deg = (int)o.meta.noise_deg;
        ct.slots = (int)o.meta.slots;
        ct.data = c->alloc_limbs((size_t)2 * ct.t, c->copy_in);
        if (!ct.data) {
          rc = fail(FIDES_ENOMEM, "input allocation failed");
          break;
        }
        const cudaError_t e = cudaMemcpyAsync(ct.data, w ? o.b : o.a, 2 * ct.t * limb, cudaMemcpyHostToDevice,
                                              c->copy_in);
        hab[w] = register_ct(ctx, ct);
        inputs.push_back(hab[w]);
        if (e != cudaSuccess) rc = cuda_fail(e, "input copy");
      }
      fo[i] = fides_op{o.op, hab[0], hab[1], o.index, 0};
    }
    cudaEvent_t ev_in = event();
    cudaEventRecord(ev_in, c->copy_in);
    cudaStreamWaitEvent(c->stream, ev_in, 0);
    if (rc == FIDES_OK) rc = run_batch(ctx, fo.data() + k0, k1 - k0);
    for (uint32_t h : inputs) fides_ct_free(ctx, h);  // stream-ordered after the batch
    if (rc != FIDES_OK) break;
    // copy out after the batch, results freed on the copy stream once copied
    cudaEvent_t ev_done = event();
    cudaEventRecord(ev_done, c->stream);
    cudaStreamWaitEvent(c->copy_out, ev_done, 0);
    for (uint32_t i = k0; i < k1; i++) {
      auto it = c->cts.find(fo[i].out);
      fgb::DevCt& r = it->second;
      ops[i].out_meta = fides_ct_meta{(uint32_t)r.t, (uint32_t)r.noise_deg, (uint32_t)r.slots, 0, r.scale};
      const cudaError_t e = cudaMemcpyAsync(ops[i].out, r.data, 2 * r.t * limb, cudaMemcpyDeviceToHost, c->copy_out);
      if (e != cudaSuccess && rc == FIDES_OK) rc = cuda_fail(e, "result copy");
      c->free_limbs(r.data, c->copy_out);
      c->cts.erase(it);
    }
  }
  c->stream = main_stream;
  {  // later work on the context stream follows both compute streams
    cudaEvent_t ev1 = event();
    cudaEventRecord(ev1, c->chunk_alt);
    cudaStreamWaitEvent(main_stream, ev1, 0);
  }
  const cudaError_t e1 = cudaStreamSynchronize(c->copy_out), e2 = cudaStreamSynchronize(c->stream);
  for (cudaEvent_t e : events) cudaEventDestroy(e);
  if (rc == FIDES_OK && (e1 != cudaSuccess || e2 != cudaSuccess)) rc = cuda_fail(e1 ? e1 : e2, "host batch");
  return rc;
}

static int one(fides_ctx* ctx, int32_t code, uint32_t a, uint32_t b, int32_t index, uint32_t* out) {
  if (!valid_ctx(ctx) || !out) return fail(FIDES_EINVAL, "null argument");
  fides_op op{code, a, b, index, 0};
  int rc = run_batch(ctx, &op, 1);
  if (rc == FIDES_OK) *out = op.out;
  return rc;
}

int fides_eval_batch(fides_ctx* ctx, fides_op* ops, uint32_t n) {
  if (!valid_ctx(ctx) || (n && !ops)) return fail(FIDES_EINVAL, "null argument");
  return run_batch(ctx, ops, n);
}

}  // extern "C"

namespace fgb {
// fides_eval_batch without the scaling technique's operand alignment: the bootstrap and polynomial-evaluation
// composites track levels and scales exactly themselves, so their recipe is the same under every technique.
int eval_batch_exact(fides_ctx* ctx, fides_op* ops, uint32_t n) {
  if (!valid_ctx(ctx) || (n && !ops)) return fail(FIDES_EINVAL, "null argument");
  return run_batch(ctx, ops, n, false);
}
}  // namespace fgb

extern "C" {

int fides_eval_add(fides_ctx* ctx, uint32_t a, uint32_t b, uint32_t* out) { return one(ctx, FIDES_OP_ADD, a, b, 0, out); }
int fides_eval_sub(fides_ctx* ctx, uint32_t a, uint32_t b, uint32_t* out) { return one(ctx, FIDES_OP_SUB, a, b, 0, out); }
int fides_eval_mult(fides_ctx* ctx, uint32_t a, uint32_t b, uint32_t* out) { return one(ctx, FIDES_OP_MULT, a, b, 0, out); }
int fides_eval_square(fides_ctx* ctx, uint32_t a, uint32_t* out) { return one(ctx, FIDES_OP_SQUARE, a, 0, 0, out); }
int fides_rescale(fides_ctx* ctx, uint32_t a, uint32_t* out) { return one(ctx, FIDES_OP_RESCALE, a, 0, 0, out); }
int fides_eval_rotate(fides_ctx* ctx, uint32_t a, int32_t index, uint32_t* out) {
  return one(ctx, FIDES_OP_ROTATE, a, 0, index, out);
}
int fides_eval_automorphism(fides_ctx* ctx, uint32_t a, uint32_t galois, uint32_t* out) {
  return one(ctx, FIDES_OP_AUTOMORPHISM, a, 0, (int32_t)galois, out);
}

int fides_fast_rotation_precompute(fides_ctx* ctx, uint32_t a, uint32_t* pre) {
  if (!valid_ctx(ctx) || !pre) return fail(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  fgb::DevCt* A = find_ct(ctx, a);
  if (!A) return fail(FIDES_EINVAL, "unknown ciphertext handle " + std::to_string(a));
  if (int rc = check_ks_shape(ctx)) return rc;
  const int t = A->t, beta = (t + c->alpha - 1) / c->alpha;
  fgb::DevModUp m;
  m.t = t;
  m.c1 = c->alloc_limbs((size_t)t, c->stream);
  m.digits = c->alloc_limbs((size_t)beta * (t + c->np), c->stream);
  fgb::u64* scratch = c->alloc_limbs((size_t)t, c->stream);
  auto release = [&]() {
    c->free_limbs(m.c1, c->stream);
    c->free_limbs(m.digits, c->stream);
    c->free_limbs(scratch, c->stream);
  };
  if (!m.c1 || !m.digits || !scratch) {
    release();
    return fail(FIDES_ENOMEM, "precomputation allocation failed");
  }
  const size_t NN = (size_t)c->N;
  cudaError_t e = cudaMemcpyAsync(m.c1, A->data + (size_t)t * NN, (size_t)t * NN * sizeof(fgb::u64),
                                  cudaMemcpyDeviceToDevice, c->stream);
  const fgb::u64* in = m.c1;
  if (e == cudaSuccess) e = c->modup(&in, &t, &scratch, &m.digits, 1, c->stream);
  c->free_limbs(scratch, c->stream);
  if (e != cudaSuccess) {
    c->free_limbs(m.c1, c->stream);
    c->free_limbs(m.digits, c->stream);
    return cuda_fail(e, "fast rotation precompute");
  }
  const uint32_t h = c->next_handle++;
  c->modups[h] = m;
  *pre = h;
  return FIDES_OK;
}

int fides_eval_fast_rotation_precomputed(fides_ctx* ctx, uint32_t a, uint32_t pre, int32_t index, uint32_t* out) {
  if (!valid_ctx(ctx) || !out) return fail(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  fgb::DevCt* A = find_ct(ctx, a);
  auto it = c->modups.find(pre);
  if (!A || it == c->modups.end()) return fail(FIDES_EINVAL, "unknown ciphertext or precomputation handle");
  const fgb::DevModUp& M = it->second;
  if (M.t != A->t) return fail(FIDES_EINVAL, "precomputation was made at a different tower count");
  const uint32_t g = c->rotation_key_galois(index, A->slots);
  auto kt = c->rot_keys.find(g);
  if (kt == c->rot_keys.end()) return fail(FIDES_ENOKEY, "no rotation key for index " + std::to_string(index));
  fgb::DevCt r;
  int rc = new_ct(ctx, A->t, *A, &r);
  if (rc) return rc;
  fgb::Context::KsReq q{M.c1, A->t, kt->second, A->data, nullptr, r.data, c->galois_inverse(g), M.digits};
  const cudaError_t e = c->keyswitch_batch(&q, 1, c->stream);
  if (e != cudaSuccess) {
    c->free_limbs(r.data, c->stream);
    return cuda_fail(e, "fast rotation");
  }
  *out = register_ct(ctx, r);
  return FIDES_OK;
}

int fides_precompute_free(fides_ctx* ctx, uint32_t pre) {
  if (!valid_ctx(ctx)) return fail(FIDES_EINVAL, "null context");
  auto it = ctx->c->modups.find(pre);
  if (it == ctx->c->modups.end()) return fail(FIDES_EINVAL, "unknown precomputation handle");
  ctx->c->free_limbs(it->second.c1, ctx->c->stream);
  ctx->c->free_limbs(it->second.digits, ctx->c->stream);
  ctx->c->modups.erase(it);
  return FIDES_OK;
}

int fides_eval_key_switch(fides_ctx* ctx, uint32_t a, uint32_t key_id, uint32_t* out) {
  return one(ctx, FIDES_OP_KEY_SWITCH, a, 0, (int32_t)key_id, out);
}

int fides_eval_fast_rotation(fides_ctx* ctx, uint32_t a, uint32_t n, const int32_t* indices, uint32_t* outs) {
  if (!valid_ctx(ctx) || (n && (!indices || !outs))) return fail(FIDES_EINVAL, "null argument");
  std::vector<fides_op> ops(n);
  for (uint32_t i = 0; i < n; i++) ops[i] = fides_op{FIDES_OP_ROTATE, a, 0, indices[i], 0};
  int rc = run_batch(ctx, ops.data(), n);  // same input: one shared ModUp
  if (rc == FIDES_OK)
    for (uint32_t i = 0; i < n; i++) outs[i] = ops[i].out;
  return rc;
}


// ---------------------------------------------------------------------------------------------------------
// Plaintexts, scalars, level management, ModRaise and linear transforms (bootstrap building blocks)
// ---------------------------------------------------------------------------------------------------------

namespace {

// Residue of round(v) mod q for |v| < 2^126, exact for the double value: v = m * 2^e with a 53-bit integer m.
uint64_t double_residue(double v, uint64_t q) {
  typedef unsigned __int128 u128;
  const bool neg = v < 0;
  double a = neg ? -v : v;
  a = std::nearbyint(a);
  int e = 0;
  const double fr = std::frexp(a, &e);  // a = fr * 2^e, fr in [0.5, 1)
  uint64_t r;
  if (e <= 63) {
    r = (uint64_t)a % q;
  } else {
    const uint64_t m = (uint64_t)std::ldexp(fr, 53);  // a = m * 2^(e-53)
    uint64_t p2 = 1 % q, b = 2 % q;
    for (int k = e - 53; k > 0; k >>= 1) {
      if (k & 1) p2 = (uint64_t)((u128)p2 * b % q);
      b = (uint64_t)((u128)b * b % q);
    }
    r = (uint64_t)((u128)(m % q) * p2 % q);
  }
  return neg && r ? q - r : r;
}

uint64_t shoup_const(uint64_t w, uint64_t q) { return (uint64_t)(((unsigned __int128)w << 64) / q); }

// One scalar constant set: residues of round(mul_v) (or of the integer k when `integer`) and round(add_v).
void make_set(fgb::Context* c, double mul_v, double add_v, bool integer, int64_t k, fgb::ScalarSet* set) {
  for (int j = 0; j < c->nq; j++) {
    const uint64_t q = c->mod[j];
    uint64_t m = double_residue(mul_v, q);
    if (integer && (k > (1ll << 52) || k < -(1ll << 52))) {
      const uint64_t r = (uint64_t)(k < 0 ? -(k + 1) : k) % q;
      m = k < 0 ? (q - 1 - r) % q : r;
    }
    set->mul[j] = m;
    set->mul_sh[j] = shoup_const(m, q);
    set->add[j] = add_v == 0.0 ? 0 : double_residue(add_v, q);
  }
}

// Scalar jobs in launches of up to kMaxJobs jobs and kMaxScalarSets constant sets; consecutive jobs with the same
// set index (into `sets`) share one copy of it.
cudaError_t launch_scalar_jobs(fgb::Context* c, const fgb::ScalarJob* jobs, const fgb::ScalarSet* sets, size_t n) {
  const fgb::Ring ring{c->N, c->logN};
  fgb::ScalarBatch sb{};
  int nsets = 0, last = -1;  // sets copied into sb; source index of the last one
  auto flush = [&]() {
    const cudaError_t e = sb.njobs ? fgb::launch_scalar(sb, ring, c->d_pc, c->stream) : cudaSuccess;
    sb.njobs = 0;
    nsets = 0;
    last = -1;
    return e;
  };
  for (size_t k = 0; k < n; k++) {
    if (sb.njobs == fgb::kMaxJobs || (jobs[k].set != last && nsets == fgb::kMaxScalarSets)) {
      const cudaError_t e = flush();
      if (e != cudaSuccess) return e;
    }
    if (jobs[k].set != last) {
      sb.sets[nsets++] = sets[jobs[k].set];
      last = jobs[k].set;
    }
    sb.jobs[sb.njobs] = jobs[k];
    sb.jobs[sb.njobs++].set = nsets - 1;
  }
  return flush();
}

int scalar_op(fides_ctx* ctx, uint32_t a, const fgb::ScalarSet& set, fgb::DevCt meta, uint32_t* out) {
  fgb::Context* c = ctx->c;
  fgb::DevCt* A = find_ct(ctx, a);
  if (!A) return fail(FIDES_EINVAL, "unknown ciphertext handle");
  fgb::DevCt r;
  int rc = new_ct(ctx, A->t, meta, &r);
  if (rc) return rc;
  const fgb::ScalarJob job{A->data, r.data, A->t, 0};
  CK(launch_scalar_jobs(c, &job, &set, 1), "scalar op");
  *out = register_ct(ctx, r);
  return FIDES_OK;
}

}  // namespace

int fides_pt_load(fides_ctx* ctx, const uint64_t* data, uint32_t towers, double scale, uint32_t* handle) {
  if (!valid_ctx(ctx) || !data || !handle) return fail(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  if (towers < 1 || towers > (uint32_t)c->nq) return fail(FIDES_EINVAL, "towers out of range");
  fgb::DevPt p;
  p.t = (int)towers;
  p.scale = scale;
  p.data = c->alloc_limbs(towers, c->stream);
  if (!p.data) return fail(FIDES_ENOMEM, "plaintext allocation failed");
  CK(cudaMemcpyAsync(p.data, data, (size_t)towers * c->N * sizeof(uint64_t), cudaMemcpyHostToDevice, c->stream),
     "plaintext copy");
  if (int rc = check_loaded(c, p.data, p.t, p.t, p.t, "plaintext")) {
    c->free_limbs(p.data, c->stream);
    return rc;
  }
  const uint32_t h = c->next_handle++;
  c->pts[h] = p;
  *handle = h;
  return FIDES_OK;
}

int fides_pt_store(fides_ctx* ctx, uint32_t handle, uint64_t* data) {
  if (!valid_ctx(ctx) || !data) return fail(FIDES_EINVAL, "null argument");
  fgb::DevPt* P = find_pt(ctx, handle);
  if (!P) return fail(FIDES_EINVAL, "unknown plaintext handle");
  CK(cudaMemcpyAsync(data, P->data, (size_t)P->t * ctx->c->N * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                     ctx->c->stream),
     "plaintext copy");
  CK(cudaStreamSynchronize(ctx->c->stream), "plaintext copy");
  return FIDES_OK;
}

int fides_pt_free(fides_ctx* ctx, uint32_t handle) {
  if (!valid_ctx(ctx)) return fail(FIDES_EINVAL, "null context");
  auto it = ctx->c->pts.find(handle);
  if (it == ctx->c->pts.end()) return fail(FIDES_EINVAL, "unknown plaintext handle");
  ctx->c->free_limbs(it->second.data, ctx->c->stream);
  ctx->c->pts.erase(it);
  return FIDES_OK;
}

int fides_eval_mult_plain(fides_ctx* ctx, uint32_t a, uint32_t pt, uint32_t* out) {
  return one(ctx, FIDES_OP_MULT_PLAIN, a, pt, 0, out);
}
int fides_eval_add_plain(fides_ctx* ctx, uint32_t a, uint32_t pt, uint32_t* out) {
  return one(ctx, FIDES_OP_ADD_PLAIN, a, pt, 0, out);
}
int fides_eval_sub_plain(fides_ctx* ctx, uint32_t a, uint32_t pt, uint32_t* out) {
  return one(ctx, FIDES_OP_SUB_PLAIN, a, pt, 0, out);
}

int fides_eval_mult_int(fides_ctx* ctx, uint32_t a, int64_t k, uint32_t* out) {
  if (!valid_ctx(ctx) || !out) return fail(FIDES_EINVAL, "null argument");
  fgb::DevCt* A = find_ct(ctx, a);
  if (!A) return fail(FIDES_EINVAL, "unknown ciphertext handle");
  fgb::ScalarSet set;
  make_set(ctx->c, (double)k, 0.0, true, k, &set);
  return scalar_op(ctx, a, set, *A, out);
}

int fides_eval_mult_scalar(fides_ctx* ctx, uint32_t a, double v, double scale, uint32_t* out) {
  if (!valid_ctx(ctx) || !out) return fail(FIDES_EINVAL, "null argument");
  return fides_eval_many_to_one(ctx, FIDES_OP_MULT_SCALAR, 1, 1, &a, nullptr, &v, &scale, out);
}

int fides_eval_add_scalar(fides_ctx* ctx, uint32_t a, double v, uint32_t* out) {
  if (!valid_ctx(ctx) || !out) return fail(FIDES_EINVAL, "null argument");
  return fides_eval_many_to_one(ctx, FIDES_OP_ADD_SCALAR, 1, 1, &a, nullptr, &v, nullptr, out);
}

int fides_eval_many_to_one(fides_ctx* ctx, int32_t op, uint32_t nb, uint32_t stride, const uint32_t* a,
                           const uint32_t* b, const double* values, const double* scales, uint32_t* outs) {
  if (!valid_ctx(ctx)) return fail(FIDES_EINVAL, "null context");
  const size_t n = (size_t)nb * stride;
  if (n == 0) return FIDES_OK;
  const bool cts = op == FIDES_OP_ADD || op == FIDES_OP_SUB;
  const bool pts = op == FIDES_OP_MULT_PLAIN || op == FIDES_OP_ADD_PLAIN || op == FIDES_OP_SUB_PLAIN;
  const bool scalar = op == FIDES_OP_MULT_SCALAR || op == FIDES_OP_ADD_SCALAR || op == FIDES_OP_MULT_INT;
  if (!cts && !pts && !scalar) return fail(FIDES_EINVAL, "op code " + std::to_string(op) + " has no many-to-one form");
  if (!a || ((cts || pts) && !b) || (scalar && !values) || (op == FIDES_OP_MULT_SCALAR && !scales))
    return fail(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  const bool in_place = outs == nullptr;
  std::vector<fgb::DevCt*> A(n);
  for (size_t k = 0; k < n; k++)
    if (!(A[k] = find_ct(ctx, a[k]))) return fail(FIDES_EINVAL, "unknown ciphertext handle " + std::to_string(a[k]));
  if (in_place) {
    std::vector<uint32_t> sorted(a, a + n);
    std::sort(sorted.begin(), sorted.end());
    if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end())
      return fail(FIDES_EINVAL, "a ciphertext appears twice in an in-place many-to-one op");
    if (cts)
      for (uint32_t i = 0; i < nb; i++)
        if (std::binary_search(sorted.begin(), sorted.end(), b[i]))
          return fail(FIDES_EINVAL, "an in-place many-to-one op cannot read one of the ciphertexts it writes");
  }
  // Validate the operands and work out the result metadata.
  std::vector<fgb::DevCt> R(n);
  std::vector<const fgb::DevCt*> B(cts ? nb : 0);
  std::vector<const fgb::DevPt*> P(pts ? nb : 0);
  for (uint32_t i = 0; i < nb; i++) {
    if (cts && !(B[i] = find_ct(ctx, b[i]))) return fail(FIDES_EINVAL, "unknown ciphertext handle " + std::to_string(b[i]));
    if (pts && !(P[i] = find_pt(ctx, b[i]))) return fail(FIDES_EINVAL, "unknown plaintext handle " + std::to_string(b[i]));
    if (op == FIDES_OP_MULT_INT && (values[i] != std::nearbyint(values[i]) || std::fabs(values[i]) >= 9007199254740992.0))
      return fail(FIDES_EINVAL, "MULT_INT values must be integers below 2^53 in magnitude");
    for (uint32_t j = 0; j < stride; j++) {
      const size_t k = (size_t)i * stride + j;
      fgb::DevCt m = *A[k];
      if (cts) {
        if (B[i]->t != m.t) return fail(FIDES_EINVAL, "operands have different tower counts");
        m.noise_deg = std::max(m.noise_deg, B[i]->noise_deg);
      }
      if (pts && P[i]->t < m.t) return fail(FIDES_EINVAL, "plaintext has fewer towers than the ciphertext");
      if (op == FIDES_OP_MULT_PLAIN || op == FIDES_OP_MULT_SCALAR) {
        m.scale *= op == FIDES_OP_MULT_PLAIN ? P[i]->scale : scales[i];
        m.noise_deg += 1;
      }
      R[k] = m;
    }
  }
  if (!in_place)
    for (size_t k = 0; k < n; k++) {
      R[k].data = c->alloc_limbs((size_t)2 * R[k].t, c->stream);
      if (!R[k].data) {
        for (size_t q = 0; q < k; q++) c->free_limbs(R[q].data, c->stream);
        return fail(FIDES_ENOMEM, "ciphertext allocation failed");
      }
    }
  cudaError_t e = cudaSuccess;
  if (cts) {
    std::vector<fgb::Context::AddReq> adds(n);
    for (size_t k = 0; k < n; k++)
      adds[k] = {A[k]->data, B[k / stride]->data, A[k]->t, R[k].data, op == FIDES_OP_SUB};
    e = c->add_batch(adds.data(), (int)n, c->stream);
  } else if (pts) {
    std::vector<fgb::PtJob> jobs(n);
    for (size_t k = 0; k < n; k++)
      jobs[k] = fgb::PtJob{A[k]->data, P[k / stride]->data, R[k].data, A[k]->t, op - FIDES_OP_MULT_PLAIN};
    e = launch_plain_jobs(c, jobs.data(), n);
  } else {
    // One constant set per group, or per (group, ciphertext scale) for ADD_SCALAR, whose constant is
    // round(v * scale of the ciphertext).
    std::vector<fgb::ScalarSet> sets;
    std::vector<fgb::ScalarJob> jobs(n);
    double last_scale = 0.0;
    for (size_t k = 0; k < n; k++) {
      const uint32_t i = (uint32_t)(k / stride);
      const bool first = k % stride == 0;
      if (first || (op == FIDES_OP_ADD_SCALAR && A[k]->scale != last_scale)) {
        sets.emplace_back();
        if (op == FIDES_OP_MULT_SCALAR) make_set(c, values[i] * scales[i], 0.0, false, 0, &sets.back());
        else if (op == FIDES_OP_MULT_INT) make_set(c, values[i], 0.0, true, (int64_t)values[i], &sets.back());
        else make_set(c, 1.0, values[i] * A[k]->scale, false, 0, &sets.back());
        last_scale = A[k]->scale;
      }
      jobs[k] = fgb::ScalarJob{A[k]->data, R[k].data, A[k]->t, (int)sets.size() - 1};
    }
    e = launch_scalar_jobs(c, jobs.data(), sets.data(), n);
  }
  if (e != cudaSuccess) {
    if (!in_place)
      for (size_t k = 0; k < n; k++) c->free_limbs(R[k].data, c->stream);
    return cuda_fail(e, "many-to-one op");
  }
  for (size_t k = 0; k < n; k++) {
    if (in_place) *A[k] = R[k];
    else outs[k] = register_ct(ctx, R[k]);
  }
  return FIDES_OK;
}

int fides_eval_linear_wsum(fides_ctx* ctx, uint32_t m, uint32_t n_terms, const uint32_t* cts, const double* weights,
                           const double* scales, uint32_t* outs) {
  if (!valid_ctx(ctx)) return fail(FIDES_EINVAL, "null context");
  if (m == 0) return FIDES_OK;
  if (!cts || !weights || !scales || !outs) return fail(FIDES_EINVAL, "null argument");
  if (n_terms < 1 || n_terms > 2 * fgb::kMaxWsumTerms) return fail(FIDES_EINVAL, "n_terms must be in [1, 16]");
  fgb::Context* c = ctx->c;
  const size_t total = (size_t)m * n_terms;
  std::vector<const fgb::DevCt*> A(total);
  for (size_t k = 0; k < total; k++) {
    if (!(A[k] = find_ct(ctx, cts[k]))) return fail(FIDES_EINVAL, "unknown ciphertext handle " + std::to_string(cts[k]));
    if (A[k]->noise_deg != 1) return fail(FIDES_EINVAL, "weighted-sum terms must have noise degree 1");
  }
  std::vector<fgb::DevCt> R(m);
  for (uint32_t i = 0; i < m; i++) {
    fgb::DevCt r = *A[i];
    for (uint32_t k = 1; k < n_terms; k++) r.t = std::min(r.t, A[(size_t)k * m + i]->t);
    r.scale = A[i]->scale * scales[i];
    r.noise_deg = 2;
    r.data = c->alloc_limbs((size_t)2 * r.t, c->stream);
    if (!r.data) {
      for (uint32_t q = 0; q < i; q++) c->free_limbs(R[q].data, c->stream);
      return fail(FIDES_ENOMEM, "ciphertext allocation failed");
    }
    R[i] = r;
  }
  // Elements whose constant columns (scales[k*m + i] over k) agree share one launch's constant set; terms go
  // in chunks of kMaxWsumTerms, later chunks accumulating into the output.
  const fgb::Ring ring{c->N, c->logN};
  auto same_set = [&](uint32_t x, uint32_t y) {
    for (uint32_t k = 0; k < n_terms; k++)
      if (scales[(size_t)k * m + x] != scales[(size_t)k * m + y]) return false;
    return true;
  };
  cudaError_t e = cudaSuccess;
  for (uint32_t k0 = 0; k0 < n_terms && e == cudaSuccess; k0 += fgb::kMaxWsumTerms) {
    const uint32_t nk = std::min<uint32_t>(fgb::kMaxWsumTerms, n_terms - k0);
    fgb::WsumBatch wb{};
    auto flush = [&]() {
      const cudaError_t x = wb.njobs ? fgb::launch_wsum(wb, ring, c->d_pc, c->stream) : cudaSuccess;
      wb.njobs = 0;
      return x;
    };
    uint32_t lead = 0;  // element whose constants the batch carries
    for (uint32_t i = 0; i < m && e == cudaSuccess; i++) {
      if (wb.njobs == fgb::kMaxJobs || (wb.njobs && !same_set(lead, i))) e = flush();
      if (e != cudaSuccess) break;
      if (wb.njobs == 0) {
        lead = i;
        wb.nterms = (int)nk;
        wb.accumulate = k0 > 0;
        for (uint32_t k = 0; k < nk; k++)
          for (int j = 0; j < c->nq; j++) {
            const uint64_t w = double_residue(weights[k0 + k] * scales[(size_t)(k0 + k) * m + i], c->mod[j]);
            wb.set.mul[k][j] = w;
            wb.set.mul_sh[k][j] = shoup_const(w, c->mod[j]);
          }
      }
      fgb::WsumJob& J = wb.jobs[wb.njobs++];
      for (uint32_t k = 0; k < nk; k++) {
        J.term[k] = A[(size_t)(k0 + k) * m + i]->data;
        J.term_t[k] = A[(size_t)(k0 + k) * m + i]->t;
      }
      J.out = R[i].data;
      J.t = R[i].t;
    }
    if (e == cudaSuccess) e = flush();
  }
  if (e != cudaSuccess) {
    for (uint32_t i = 0; i < m; i++) c->free_limbs(R[i].data, c->stream);
    return cuda_fail(e, "weighted sum");
  }
  for (uint32_t i = 0; i < m; i++) outs[i] = register_ct(ctx, R[i]);
  return FIDES_OK;
}

int fides_level_reduce(fides_ctx* ctx, uint32_t a, uint32_t towers, uint32_t* out) {
  if (!valid_ctx(ctx) || !out) return fail(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  fgb::DevCt* A = find_ct(ctx, a);
  if (!A) return fail(FIDES_EINVAL, "unknown ciphertext handle");
  if (towers < 1 || (int)towers > A->t) return fail(FIDES_EINVAL, "towers must be in [1, current towers]");
  fgb::DevCt r;
  int rc = new_ct(ctx, (int)towers, *A, &r);
  if (rc) return rc;
  const size_t row = (size_t)towers * c->N * sizeof(uint64_t);
  CK(cudaMemcpy2DAsync(r.data, row, A->data, (size_t)A->t * c->N * sizeof(uint64_t), row, 2, cudaMemcpyDeviceToDevice,
                       c->stream),
     "level reduce");
  *out = register_ct(ctx, r);
  return FIDES_OK;
}

int fides_mod_raise(fides_ctx* ctx, uint32_t a, uint32_t towers, uint32_t* out) {
  if (!valid_ctx(ctx) || !out) return fail(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  fgb::DevCt* A = find_ct(ctx, a);
  if (!A) return fail(FIDES_EINVAL, "unknown ciphertext handle");
  if (towers < 1 || (int)towers > c->nq) return fail(FIDES_EINVAL, "towers out of range");
  fgb::DevCt r;
  int rc = new_ct(ctx, (int)towers, *A, &r);
  if (rc) return rc;
  CK(c->mod_raise(A->data, A->t, (int)towers, r.data, c->stream), "mod raise");
  *out = register_ct(ctx, r);
  return FIDES_OK;
}

int fides_lt_create(fides_ctx* ctx, uint32_t bs, uint32_t gs, uint32_t towers, const uint64_t* diags,
                    const uint8_t* present, double scale, uint32_t* handle) {
  return fides_lt_create_strided(ctx, bs, gs, 1, 0, towers, diags, present, scale, handle);
}

static int lt_create(fides_ctx* ctx, uint32_t bs, uint32_t gs, int32_t stride, int32_t base, uint32_t towers, bool ext,
                     const uint64_t* diags, const uint8_t* present, double scale, uint32_t* handle) {
  if (!valid_ctx(ctx) || !diags || !present || !handle) return fail(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  if (bs < 1 || bs > 16 || gs < 1 || gs > (uint32_t)fgb::kMaxJobs || towers < 1 || towers > (uint32_t)c->nq)
    return fail(FIDES_EINVAL, "need 1 <= bs <= 16, 1 <= gs <= 64, 1 <= towers <= nq");
  if (bs > 1 && stride == 0) return fail(FIDES_EINVAL, "stride must be nonzero");
  fgb::DevLT lt;
  lt.bs = (int)bs;
  lt.gs = (int)gs;
  lt.stride = (int)stride;
  lt.base = (int)base;
  lt.t = (int)towers;
  lt.ext = ext;
  lt.rows = (int)towers + (ext ? c->np : 0);
  lt.scale = scale;
  lt.present.assign(present, present + (size_t)bs * gs);
  const size_t bytes = (size_t)bs * gs * lt.rows * c->N * sizeof(uint64_t);
  void* d = nullptr;
  void* pd = nullptr;
  CK(cudaMalloc(&d, bytes), "linear transform allocation");
  if (cudaMalloc(&pd, (size_t)bs * gs) != cudaSuccess) {
    cudaFree(d);
    return fail(FIDES_ENOMEM, "linear transform allocation failed");
  }
  lt.diags = (fgb::u64*)d;
  lt.present_dev = (uint8_t*)pd;
  cudaError_t e = cudaMemcpyAsync(d, diags, bytes, cudaMemcpyDefault, c->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(pd, present, (size_t)bs * gs, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) {
    cudaFree(d);
    cudaFree(pd);
    return cuda_fail(e, "linear transform copy");
  }
  const uint32_t h = c->next_handle++;
  c->lts[h] = std::move(lt);
  *handle = h;
  return FIDES_OK;
}

int fides_lt_create_strided(fides_ctx* ctx, uint32_t bs, uint32_t gs, int32_t stride, int32_t base, uint32_t towers,
                            const uint64_t* diags, const uint8_t* present, double scale, uint32_t* handle) {
  return lt_create(ctx, bs, gs, stride, base, towers, false, diags, present, scale, handle);
}

int fides_lt_create_strided_ext(fides_ctx* ctx, uint32_t bs, uint32_t gs, int32_t stride, int32_t base,
                                uint32_t towers, const uint64_t* diags, const uint8_t* present, double scale,
                                uint32_t* handle) {
  return lt_create(ctx, bs, gs, stride, base, towers, true, diags, present, scale, handle);
}

int fides_lt_free(fides_ctx* ctx, uint32_t handle) {
  if (!valid_ctx(ctx)) return fail(FIDES_EINVAL, "null context");
  auto it = ctx->c->lts.find(handle);
  if (it == ctx->c->lts.end()) return fail(FIDES_EINVAL, "unknown linear transform handle");
  cudaStreamSynchronize(ctx->c->stream);
  cudaFree(it->second.diags);
  cudaFree(it->second.present_dev);
  ctx->c->lts.erase(it);
  return FIDES_OK;
}

int fides_eval_linear_transform(fides_ctx* ctx, uint32_t a, uint32_t lt, uint32_t* out) {
  return fides_eval_linear_transform_batch(ctx, 1, &a, lt, out);
}

int fides_eval_linear_transform_batch(fides_ctx* ctx, uint32_t n, const uint32_t* cts, uint32_t lt, uint32_t* outs) {
  if (!valid_ctx(ctx) || !cts || !outs) return fail(FIDES_EINVAL, "null argument");
  if (n == 0) return FIDES_OK;
  fgb::Context* c = ctx->c;
  auto it = c->lts.find(lt);
  if (it == c->lts.end()) return fail(FIDES_EINVAL, "unknown linear transform handle");
  if (int rc0 = check_ks_shape(ctx)) return rc0;
  const fgb::DevLT& L = it->second;
  std::vector<fgb::DevCt*> A(n);
  for (uint32_t i = 0; i < n; i++) {
    A[i] = find_ct(ctx, cts[i]);
    if (!A[i]) return fail(FIDES_EINVAL, "unknown ciphertext handle " + std::to_string(cts[i]));
    if (A[i]->t != A[0]->t) return fail(FIDES_EINVAL, "batched transform inputs must have the same tower count");
  }
  const int t = A[0]->t;
  if (t > L.t) return fail(FIDES_EINVAL, "ciphertext has more towers than the transform's diagonals");
  for (int32_t r : L.baby_rotations(c->N))
    if (r && !c->rot_keys.count(fgb::Context::galois_for_index(c->N, r)))
      return fail(FIDES_ENOKEY, "missing baby-step rotation key for index " + std::to_string(r));
  const std::vector<int32_t> giant = L.giant_rotations(c->N);
  for (int g = 0; g < L.gs; g++) {
    bool any = false;
    for (int b = 0; b < L.bs; b++) any = any || L.present[(size_t)g * L.bs + b];
    if (any && giant[g] && !c->rot_keys.count(fgb::Context::galois_for_index(c->N, giant[g])))
      return fail(FIDES_ENOKEY, "missing giant-step rotation key for index " + std::to_string(giant[g]));
  }
  std::vector<fgb::DevCt> R(n);
  std::vector<const fgb::u64*> xs(n);
  std::vector<fgb::u64*> ys(n);
  for (uint32_t i = 0; i < n; i++) {
    fgb::DevCt meta = *A[i];
    meta.scale = A[i]->scale * L.scale;
    meta.noise_deg = A[i]->noise_deg + 1;
    int rc = new_ct(ctx, t, meta, &R[i]);
    if (rc) {
      for (uint32_t k = 0; k < i; k++) c->free_limbs(R[k].data, c->stream);
      return rc;
    }
    xs[i] = A[i]->data;
    ys[i] = R[i].data;
  }
  const cudaError_t e = c->linear_transform_batch(xs.data(), (int)n, t, L, ys.data(), c->stream);
  if (e != cudaSuccess) {
    for (uint32_t k = 0; k < n; k++) c->free_limbs(R[k].data, c->stream);
    return cuda_fail(e, "linear transform");
  }
  for (uint32_t i = 0; i < n; i++) outs[i] = register_ct(ctx, R[i]);
  return FIDES_OK;
}

int fides_eval_mult_monomial(fides_ctx* ctx, uint32_t a, uint32_t k, uint32_t* out) {
  if (!valid_ctx(ctx) || !out) return fail(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  fgb::DevCt* A = find_ct(ctx, a);
  if (!A) return fail(FIDES_EINVAL, "unknown ciphertext handle " + std::to_string(a));
  fgb::DevCt r;
  int rc = new_ct(ctx, A->t, *A, &r);
  if (rc) return rc;
  CK(c->mult_monomial(A->data, A->t, k, r.data, c->stream), "monomial multiplication");
  *out = register_ct(ctx, r);
  return FIDES_OK;
}


// ---------------------------------------------------------------------------------------------------------
// Extended-basis ciphertexts (EvalFastRotationExt / KeySwitchDown)
// ---------------------------------------------------------------------------------------------------------

static uint32_t register_ext(fides_ctx* ctx, const fgb::DevCt& ct) {
  uint32_t h = ctx->c->next_handle++;
  if (ctx->c->next_handle == 0) ctx->c->next_handle = 1;
  ctx->c->ext_cts[h] = ct;
  return h;
}

static fgb::DevCt* find_ext(fides_ctx* ctx, uint32_t h) {
  auto it = ctx->c->ext_cts.find(h);
  return it == ctx->c->ext_cts.end() ? nullptr : &it->second;
}

int fides_eval_fast_rotation_ext(fides_ctx* ctx, uint32_t a, uint32_t pre, uint32_t n, const int32_t* indices,
                                 int32_t add_first, uint32_t* outs) {
  if (!valid_ctx(ctx) || (n && (!indices || !outs))) return fail(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  fgb::DevCt* A = find_ct(ctx, a);
  if (!A) return fail(FIDES_EINVAL, "unknown ciphertext handle " + std::to_string(a));
  const fgb::DevModUp* M = nullptr;
  if (pre) {
    auto it = c->modups.find(pre);
    if (it == c->modups.end()) return fail(FIDES_EINVAL, "unknown precomputation handle");
    if (it->second.t != A->t) return fail(FIDES_EINVAL, "precomputation was made at a different tower count");
    M = &it->second;
  }
  if (int rc = check_ks_shape(ctx)) return rc;
  const int t = A->t;
  const size_t NN = (size_t)c->N, rows = (size_t)2 * (t + c->np);
  std::vector<fgb::DevCt> res(n);
  std::vector<fgb::Context::KsReq> rq;
  fgb::KsBatch lift{};
  int rc = FIDES_OK;
  for (uint32_t i = 0; i < n && rc == FIDES_OK; i++) {
    res[i] = *A;
    res[i].data = c->alloc_limbs(rows, c->stream);
    if (!res[i].data) {
      rc = fail(FIDES_ENOMEM, "ciphertext allocation failed");
      break;
    }
    const uint32_t g = fgb::Context::galois_for_index(c->N, indices[i]);
    if (g == 1) {  // no rotation: the input itself, lifted by P
      fgb::KsJob& j = lift.jobs[lift.njobs++];
      j.add0 = add_first ? A->data : nullptr;
      j.add1 = A->data + (size_t)t * NN;
      j.out = res[i].data;
      j.t = t;
      j.galois_inv = 1;
      j.ext_mode = 1;
      if (lift.njobs == fgb::kMaxJobs) rc = fail(FIDES_EINVAL, "at most 64 zero rotations per call");
      continue;
    }
    auto kt = c->rot_keys.find(g);
    if (kt == c->rot_keys.end()) {
      rc = fail(FIDES_ENOKEY, "no rotation key for Galois element " + std::to_string(g));
      break;
    }
    fgb::Context::KsReq r{M ? M->c1 : A->data + (size_t)t * NN, t, kt->second, add_first ? A->data : nullptr, nullptr,
                          res[i].data, c->galois_inverse(g), M ? M->digits : nullptr};
    r.ext_mode = 1;
    rq.push_back(r);
  }
  cudaError_t e = cudaSuccess;
  if (rc == FIDES_OK) {
    const fgb::Ring ring{c->N, c->logN};
    e = fgb::launch_ext_epilogue(lift, ring, c->crt, c->d_pc, c->stream);
    if (e == cudaSuccess) e = c->keyswitch_batch(rq.data(), (int)rq.size(), c->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "fast rotation (extended basis)");
  }
  if (rc != FIDES_OK) {
    for (auto& r : res) c->free_limbs(r.data, c->stream);
    return rc;
  }
  for (uint32_t i = 0; i < n; i++) outs[i] = register_ext(ctx, res[i]);
  return FIDES_OK;
}

int fides_ext_add(fides_ctx* ctx, uint32_t a, uint32_t b, uint32_t* out) {
  if (!valid_ctx(ctx) || !out) return fail(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  fgb::DevCt* A = find_ext(ctx, a);
  fgb::DevCt* B = find_ext(ctx, b);
  if (!A || !B) return fail(FIDES_EINVAL, "unknown extended-basis ciphertext handle");
  if (A->t != B->t) return fail(FIDES_EINVAL, "operands have different tower counts");
  fgb::DevCt r = *A;
  r.noise_deg = std::max(A->noise_deg, B->noise_deg);
  r.data = c->alloc_limbs((size_t)2 * (A->t + c->np), c->stream);
  if (!r.data) return fail(FIDES_ENOMEM, "ciphertext allocation failed");
  fgb::SumBatch sb{};
  sb.nq = c->nq;
  sb.njobs = 1;
  sb.jobs[0] = fgb::SumJob{B->data, 0, 1, A->data, r.data, A->t, c->np};
  const fgb::Ring ring{c->N, c->logN};
  const cudaError_t e = fgb::launch_sum(sb, ring, c->d_pc, c->stream);
  if (e != cudaSuccess) {
    c->free_limbs(r.data, c->stream);
    return cuda_fail(e, "extended-basis add");
  }
  *out = register_ext(ctx, r);
  return FIDES_OK;
}

int fides_pt_load_ext(fides_ctx* ctx, const uint64_t* data, uint32_t towers, double scale, uint32_t* handle) {
  if (!valid_ctx(ctx) || !data || !handle) return fail(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  if (towers < 1 || towers > (uint32_t)c->nq) return fail(FIDES_EINVAL, "towers out of range");
  fgb::DevPt p;
  p.t = (int)towers;
  p.prows = c->np;
  p.scale = scale;
  const size_t rows = (size_t)towers + c->np;
  p.data = c->alloc_limbs(rows, c->stream);
  if (!p.data) return fail(FIDES_ENOMEM, "plaintext allocation failed");
  CK(cudaMemcpyAsync(p.data, data, rows * c->N * sizeof(uint64_t), cudaMemcpyDefault, c->stream), "plaintext copy");
  if (int rc = check_loaded(c, p.data, (long long)rows, (int)rows, p.t, "plaintext")) {
    c->free_limbs(p.data, c->stream);
    return rc;
  }
  const uint32_t h = c->next_handle++;
  c->pts[h] = p;
  *handle = h;
  return FIDES_OK;
}

int fides_ext_mult_plain(fides_ctx* ctx, uint32_t a, uint32_t pt, uint32_t* out) {
  if (!valid_ctx(ctx) || !out) return fail(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  fgb::DevCt* A = find_ext(ctx, a);
  fgb::DevPt* P = find_pt(ctx, pt);
  if (!A || !P) return fail(FIDES_EINVAL, "unknown extended-basis ciphertext or plaintext handle");
  if (P->prows != c->np) return fail(FIDES_EINVAL, "the plaintext has no special-prime rows (fides_pt_load_ext)");
  if (P->t < A->t) return fail(FIDES_EINVAL, "plaintext has fewer towers than the ciphertext");
  fgb::DevCt r = *A;
  r.scale = A->scale * P->scale;
  r.noise_deg = A->noise_deg + 1;
  r.data = c->alloc_limbs((size_t)2 * (A->t + c->np), c->stream);
  if (!r.data) return fail(FIDES_ENOMEM, "ciphertext allocation failed");
  static const uint8_t kOne[1] = {1};
  fgb::DotBatch db{};
  db.pt_base = P->data;
  db.pt_stride = (long long)(P->t + P->prows) * c->N;
  db.present = kOne;
  db.bs = 1;
  db.t = A->t;
  db.np = c->np;
  db.nq = c->nq;
  db.pt_prow = P->t;
  db.njobs = 1;
  db.jobs[0] = fgb::DotJob{r.data, A->data, nullptr, 0, 1, 0ull};
  const fgb::Ring ring{c->N, c->logN};
  const cudaError_t e = fgb::launch_ptdot(db, ring, c->d_pc, c->stream);
  if (e != cudaSuccess) {
    c->free_limbs(r.data, c->stream);
    return cuda_fail(e, "extended-basis plaintext product");
  }
  *out = register_ext(ctx, r);
  return FIDES_OK;
}

int fides_key_switch_down(fides_ctx* ctx, uint32_t a, uint32_t* out) {
  if (!valid_ctx(ctx) || !out) return fail(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  fgb::DevCt* A = find_ext(ctx, a);
  if (!A) return fail(FIDES_EINVAL, "unknown extended-basis ciphertext handle");
  const size_t rows = (size_t)2 * (A->t + c->np);
  fgb::u64* tmp = c->alloc_limbs(rows, c->stream);  // the ModDown leaves its input's special rows in coefficient form
  fgb::DevCt r;
  int rc = new_ct(ctx, A->t, *A, &r);
  if (rc || !tmp) {
    c->free_limbs(tmp, c->stream);
    if (!rc) c->free_limbs(r.data, c->stream);
    return rc ? rc : fail(FIDES_ENOMEM, "workspace allocation failed");
  }
  cudaError_t e = cudaMemcpyAsync(tmp, A->data, rows * c->N * sizeof(uint64_t), cudaMemcpyDeviceToDevice, c->stream);
  const fgb::Context::MdReq m{tmp, A->t, 2, r.data};
  if (e == cudaSuccess) e = c->moddown_batch(&m, 1, c->stream);
  c->free_limbs(tmp, c->stream);
  if (e != cudaSuccess) {
    c->free_limbs(r.data, c->stream);
    return cuda_fail(e, "key switch down");
  }
  *out = register_ct(ctx, r);
  return FIDES_OK;
}

int fides_ext_store(fides_ctx* ctx, uint32_t h, uint64_t* data, fides_ct_meta* meta) {
  if (!valid_ctx(ctx) || !data) return fail(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  fgb::DevCt* A = find_ext(ctx, h);
  if (!A) return fail(FIDES_EINVAL, "unknown extended-basis ciphertext handle");
  CK(cudaMemcpyAsync(data, A->data, (size_t)2 * (A->t + c->np) * c->N * sizeof(uint64_t), cudaMemcpyDeviceToHost,
                     c->stream),
     "ciphertext store");
  CK(cudaStreamSynchronize(c->stream), "ciphertext store");
  if (meta) *meta = fides_ct_meta{(uint32_t)A->t, (uint32_t)A->noise_deg, (uint32_t)A->slots, 0, A->scale};
  return FIDES_OK;
}

}  // extern "C"
