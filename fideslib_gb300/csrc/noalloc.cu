// Allocation-free rotation: fides_eval_rotate_noalloc (declared in include/fideslib_gb300.h).
//
// Some callers cannot allocate device memory on their request path: a process whose GPU memory is entirely
// pre-reserved by its own caching allocator, or a latency-critical caller that cannot afford cudaMalloc's
// implicit device synchronisation.  For them this entry point runs the same key-switch pipeline as
// fides_eval_automorphism, but its workspace lives in the fixed file-scope array below instead of the
// stream-ordered pool, and it calls no cudaMalloc, cudaFree or other allocating routine.
//
// Limits and sharing rules:
//   * the workspace of one rotation at t towers is t + beta(t+np) + 2(t+np) + 2t limbs of 8N bytes; requests
//     larger than kNoAllocScratchBytes (32 MiB) are rejected with FIDES_EINVAL;
//   * every GPU that loads the library holds the 32 MiB array until the process exits;
//   * all calls share the one array, and it keeps the contents of the last call.  Nothing in the pipeline needs
//     it zeroed (every region is fully written before it is read), so it is never cleared;
//   * calls whose GPU work overlaps (different streams, or different host threads) race on the array: order
//     them on one stream;
//   * the context's device must be the current device (FIDES_EINVAL otherwise): the array's address differs per
//     device, and the context's stream and tables live on its own device;
//   * the first call on a device looks up the array's device address with cudaGetSymbolAddress while that
//     device is current; make that first call before any stream capture.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/fideslib_gb300.h"
#include "engine.hpp"

struct fides_ctx {
  fgb::Context* c;
};

namespace fgb {
int set_last_error(int code, const char* msg);
}

namespace {

constexpr size_t kNoAllocScratchBytes = 32ull << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned long long g_noalloc_scratch[kNoAllocScratchBytes / sizeof(unsigned long long)];

std::mutex g_setup_mu;
fgb::u64* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the context's device `want`, which must be the current device: the
// array's address is per device, and the context's stream and tables live on `want` (looked up once per device).
int scratch_for_device(int want, fgb::u64** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fgb::set_last_error(FIDES_ENODEV, "no current CUDA device for the no-alloc scratch");
  if (dev != want)
    return fgb::set_last_error(FIDES_EINVAL,
                               "the current CUDA device is not the context's device; make the context's device "
                               "current before calling fides_eval_rotate_noalloc");
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return fgb::set_last_error(FIDES_ECUDA, "cudaGetSymbolAddress of the no-alloc scratch failed");
    g_scratch_ptr[dev] = (fgb::u64*)p;
  }
  *out = g_scratch_ptr[dev];
  return FIDES_OK;
}

bool overlaps(const void* a, size_t na, const void* b, size_t nb) {
  const char *pa = (const char*)a, *pb = (const char*)b;
  return pa < pb + nb && pb < pa + na;
}

}  // namespace

extern "C" int fides_eval_rotate_noalloc(fides_ctx* ctx, const uint64_t* dev_in, uint32_t towers, uint32_t galois,
                                         uint64_t* dev_out, void* stream) {
  using fgb::u64;
  if (!ctx || !ctx->c || !dev_in || !dev_out) return fgb::set_last_error(FIDES_EINVAL, "null argument");
  if ((uintptr_t)dev_in % 16 || (uintptr_t)dev_out % 16)  // the kernels read and write 16-byte vectors
    return fgb::set_last_error(FIDES_EINVAL, "device buffers must be 16-byte aligned");
  fgb::Context* c = ctx->c;
  const int t = (int)towers;
  if (t < 1 || t > c->nq) return fgb::set_last_error(FIDES_EINVAL, "towers out of range");
  if (c->alpha > 32) return fgb::set_last_error(FIDES_EINVAL, "at most 32 towers per digit");
  const int np = c->np, nq = c->nq, alpha = c->alpha, beta = (t + alpha - 1) / alpha;
  const size_t NN = (size_t)c->N;
  const size_t limbs = (size_t)t + (size_t)beta * (t + np) + 2 * (size_t)(t + np) + 2 * (size_t)t;
  if (limbs * NN * sizeof(u64) > kNoAllocScratchBytes)
    return fgb::set_last_error(FIDES_EINVAL,
                               "request needs more than the 32 MiB no-alloc scratch (t + beta(t+np) + 2(t+np) + 2t "
                               "limbs of 8N bytes); use fides_eval_automorphism");
  const size_t ct_bytes = 2 * (size_t)t * NN * sizeof(u64);
  if (overlaps(dev_in, ct_bytes, dev_out, ct_bytes))
    return fgb::set_last_error(FIDES_EINVAL, "output must not overlap the input");
  if ((galois & 1) == 0 || galois >= 2u * (uint32_t)c->N)
    return fgb::set_last_error(FIDES_EINVAL, "Galois element must be odd and < 2N");
  auto it = c->rot_keys.find(galois);
  if (it == c->rot_keys.end()) return fgb::set_last_error(FIDES_ENOKEY, "no rotation key for this Galois element");
  u64* ws = nullptr;
  if (int rc = scratch_for_device(c->device, &ws)) return rc;
  cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;

  const u64* a = (const u64*)dev_in + (size_t)t * NN;  // c1
  u64* coeff = ws;
  u64* conv = coeff + (size_t)t * NN;
  u64* inner = conv + (size_t)beta * (t + np) * NN;
  u64* md = inner + 2 * (size_t)(t + np) * NN;
  const fgb::Ring ring{c->N, c->logN};
  uint8_t pm[64];
  cudaError_t e = cudaSuccess;

  fgb::KsBatch kb{};
  kb.njobs = 1;
  fgb::KsJob& j = kb.jobs[0];
  j.a = a;
  j.add0 = (const u64*)dev_in;
  j.add1 = nullptr;
  j.key = it->second;
  j.coeff = coeff;
  j.conv = conv;
  j.inner = inner;
  j.md = md;
  j.out = (u64*)dev_out;
  j.t = t;
  j.galois_inv = c->galois_inverse(galois);

  {  // INTT of c1 into the coefficient workspace
    fgb::NttBatch nb{};
    for (int k = 0; k < t; k++) pm[k] = (uint8_t)k;
    fgb::ntt_add_job(nb, a, coeff, 0, 0, t, 1, pm);
    e = fgb::launch_ntt(nb, c->tabs, true, s);
  }
  if (e == cudaSuccess) e = fgb::launch_modup_conv(kb, ring, c->crt, c->d_pc, s);
  if (e == cudaSuccess) {  // NTT of every converted digit row
    fgb::NttBatch nb{};
    for (int d = 0; d < beta; d++) {
      const int start = d * alpha, sz = (alpha < t - start) ? alpha : t - start, rows = t - sz + np;
      for (int jj = 0; jj < rows; jj++)
        pm[jj] = (uint8_t)(jj < start ? jj : (jj < t - sz ? jj + sz : nq + (jj - (t - sz))));
      u64* cv = conv + (size_t)d * (t + np) * NN;
      fgb::ntt_add_job(nb, cv, cv, 0, 0, rows, 1, pm);
    }
    e = fgb::launch_ntt(nb, c->tabs, false, s);
  }
  if (e == cudaSuccess) e = fgb::launch_ks_inner(kb, ring, c->crt, c->d_pc, s);
  if (e == cudaSuccess) {  // P rows of both inner products to coefficient form
    fgb::NttBatch nb{};
    for (int k = 0; k < np; k++) pm[k] = (uint8_t)(nq + k);
    u64* p = inner + (size_t)t * NN;
    fgb::ntt_add_job(nb, p, p, (long long)(t + np) * c->N, (long long)(t + np) * c->N, np, 2, pm);
    e = fgb::launch_ntt(nb, c->tabs, true, s);
  }
  if (e == cudaSuccess) e = fgb::launch_moddown_conv(kb, ring, c->crt, c->d_pc, s);
  if (e == cudaSuccess) {
    fgb::NttBatch nb{};
    for (int k = 0; k < t; k++) pm[k] = (uint8_t)k;
    fgb::ntt_add_job(nb, md, md, (long long)t * c->N, (long long)t * c->N, t, 2, pm);
    e = fgb::launch_ntt(nb, c->tabs, false, s);
  }
  if (e == cudaSuccess) e = fgb::launch_moddown_epilogue(kb, ring, c->crt, c->d_pc, s);
  if (e != cudaSuccess) return fgb::set_last_error(FIDES_ECUDA, cudaGetErrorString(e));
  return FIDES_OK;
}
