// CKKS encoding and decoding on the GPU (C ABI: fides_pt_encode, fides_pt_decode, fides_lt_create_slots).
//
// Reference counterpart: OpenFHE's MakeCKKSPackedPlaintext / Decode, which the reference calls on the CPU before
// LoadPlaintext (api/CryptoContext.cpp:488-535) and for its bootstrap precomputation (RawCiphertext.cu
// AddBootstrapPrecomputation).  Convention (the evaluation order the engine uses everywhere): n slots z, packed
// coefficients w = U_n^-1 z with U_n[j][k] = xi^(5^j k), xi = exp(i pi / 2n); the plaintext polynomial has
// m[k gap] = Re(w_k), m[(n + k) gap] = Im(w_k) (gap = N / 2n, every other coefficient zero), and its residues are
// round(scale * m) mod q_i in evaluation form.  U_n is applied as the special FFT U_n = S_n ... S_2 P (P the
// bit-reversal permutation, S_len the butterfly stage (u, v) -> (u + w_j v, u - w_j v), w_j =
// exp(2 pi i (5^j mod 4 len) / (4 len))), one launch per stage over every vector of a batch, in FP64.
// Decoding reconstructs coefficients from towers 0 and 1 (exact CRT in 128 bits), so it needs
// |round(scale * m)| < q_0 q_1 / 2 (q_0 / 2 for a one-tower plaintext).
#include <cuda_runtime.h>

#include <cmath>
#include <complex>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/fideslib_gb300.h"
#include "arith.cuh"
#include "engine.hpp"

struct fides_ctx {
  fgb::Context* c;
};

namespace fgb {
int set_last_error(int code, const char* msg);
}

namespace {

using fgb::u64;
constexpr int kT = 256;

__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Stage S_len (inverse = false) or S_len^-1 over `nv` vectors of n values: one thread per butterfly.
__global__ void fft_stage_kernel(double2* __restrict__ a, int nv, int n, int len, const double2* __restrict__ roots,
                                 const uint32_t* __restrict__ rot, int inverse) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int half = n / 2;
  if (idx >= (long long)nv * half) return;
  const int v = (int)(idx / half), r = (int)(idx % half), h = len / 2, j = r % h;
  double2* x = a + (size_t)v * n + (size_t)(r / h) * len + j;
  const double2 w = roots[(size_t)(rot[j] & (4u * len - 1)) * (n / len)];
  const double2 u = x[0], y = x[h];
  if (!inverse) {
    const double2 t = cmul(w, y);
    x[0] = make_double2(u.x + t.x, u.y + t.y);
    x[h] = make_double2(u.x - t.x, u.y - t.y);
  } else {  // u' = (u + y) / 2, v' = (u - y) conj(w) / 2
    x[0] = make_double2(0.5 * (u.x + y.x), 0.5 * (u.y + y.y));
    const double2 d = make_double2(0.5 * (u.x - y.x), 0.5 * (u.y - y.y));
    x[h] = cmul(d, make_double2(w.x, -w.y));
  }
}

__device__ __forceinline__ uint32_t brev_bits(uint32_t x, int bits) { return bits ? __brev(x) >> (32 - bits) : 0; }

// Encode placement: out[v][j][c] = round(scale m_c) mod m_j with m from the FFT output y (w_k = y[brev(k)]);
// row j < tq is Q tower j, row tq + k the special prime nq + k (t rows in all).
__global__ void encode_place_kernel(const double2* __restrict__ y, int nv, int n, int logn, int N, double scale, int t,
                                    int tq, int nq, const fgb::PrimeConst* __restrict__ pc, u64* __restrict__ out,
                                    int* __restrict__ overflow) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)nv * N) return;
  const int v = (int)(idx / N), c = (int)(idx % N), gap = N / (2 * n);
  double val = 0.0;
  if (c % gap == 0) {
    const int k = c / gap;
    val = k < n ? y[(size_t)v * n + brev_bits(k, logn)].x : y[(size_t)v * n + brev_bits(k - n, logn)].y;
  }
  const double r = nearbyint(val * scale);
  if (!(fabs(r) < 4611686018427387904.0)) {  // 2^62 (also catches NaN)
    atomicExch(overflow, 1);
    for (int j = 0; j < t; j++) out[((size_t)v * t + j) * N + c] = 0;
    return;
  }
  const long long iv = (long long)r;
  const u64 mag = (u64)(iv < 0 ? -iv : iv);
  for (int j = 0; j < t; j++) {
    const u64 q = pc[j < tq ? j : nq + (j - tq)].p, m = mag % q;
    out[((size_t)v * t + j) * N + c] = (iv < 0 && m) ? q - m : m;
  }
}

// Decode gather: coefficient-form towers 0 (and 1) -> centred values -> w_k, written permuted (a[i] = w[brev(i)]).
__global__ void decode_gather_kernel(const u64* __restrict__ coeff, int t, int n, int logn, int N, double inv_scale,
                                     const fgb::PrimeConst* __restrict__ pc, u64 q0inv_mod_q1, u64 q0inv_sh,
                                     double2* __restrict__ a) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const int gap = N / (2 * n);
  double part[2];
  for (int s = 0; s < 2; s++) {
    const int c = (k + s * n) * gap;
    const u64 q0 = pc[0].p, x0 = coeff[c];
    double val;
    if (t == 1) {
      val = x0 > q0 / 2 ? -(double)(q0 - x0) : (double)x0;
    } else {  // x = x0 + q0 * ((x1 - x0) q0^-1 mod q1), centred modulo q0 q1
      const u64 q1 = pc[1].p, x1 = coeff[N + c];
      const u64 x0m = x0 % q1;
      const u64 d = x1 >= x0m ? x1 - x0m : x1 + q1 - x0m;
      const u64 h = fgb::shoup(d, q0inv_mod_q1, q0inv_sh, q1);
      const unsigned __int128 Q = (unsigned __int128)q0 * q1;
      const unsigned __int128 X = (unsigned __int128)h * q0 + x0;
      if (X > Q / 2) {
        const unsigned __int128 m = Q - X;
        val = -((double)(u64)(m >> 64) * 18446744073709551616.0 + (double)(u64)m);
      } else {
        val = (double)(u64)(X >> 64) * 18446744073709551616.0 + (double)(u64)X;
      }
    }
    part[s] = val * inv_scale;
  }
  a[brev_bits(k, logn)] = make_double2(part[0], part[1]);
}

struct FftTables {
  double2* roots = nullptr;  // exp(2 pi i k / 4n), k < 4n
  uint32_t* rot = nullptr;   // 5^j mod 4n, j < n/2
};

std::mutex g_tab_mu;
std::map<std::pair<int, int>, FftTables> g_tabs;  // per (device, n), shared by every context; kept for the process

int tables_for(int n, FftTables* out) {
  std::lock_guard<std::mutex> lk(g_tab_mu);
  int dev = 0;
  cudaGetDevice(&dev);
  auto key = std::make_pair(dev, n);
  auto it = g_tabs.find(key);
  if (it != g_tabs.end()) {
    *out = it->second;
    return FIDES_OK;
  }
  std::vector<double2> roots(4 * (size_t)n);
  for (int k = 0; k < 4 * n; k++) {
    const double th = 2.0 * M_PI * (double)k / (4.0 * n);
    roots[k] = make_double2(std::cos(th), std::sin(th));
  }
  std::vector<uint32_t> rot(std::max(1, n / 2));
  uint64_t g = 1;
  for (size_t j = 0; j < rot.size(); j++) {
    rot[j] = (uint32_t)g;
    g = g * 5 % (4ull * n);
  }
  FftTables T;
  if (cudaMalloc(&T.roots, roots.size() * sizeof(double2)) != cudaSuccess ||
      cudaMalloc(&T.rot, rot.size() * sizeof(uint32_t)) != cudaSuccess)
    return fgb::set_last_error(FIDES_ENOMEM, "encoding table allocation failed");
  cudaMemcpy(T.roots, roots.data(), roots.size() * sizeof(double2), cudaMemcpyHostToDevice);
  cudaMemcpy(T.rot, rot.data(), rot.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
  g_tabs[key] = T;
  *out = T;
  return FIDES_OK;
}

int check_slots(fgb::Context* c, uint32_t slots) {
  if (slots < 1 || (slots & (slots - 1)) || slots > (uint32_t)c->N / 2)
    return fgb::set_last_error(FIDES_EINVAL, "slots must be a power of two <= N/2");
  return FIDES_OK;
}

int ilog2(uint32_t x) {
  int l = 0;
  while ((1u << l) < x) l++;
  return l;
}

// Encodes nv vectors (host re/im, [nv][slots]) into out ([nv][rows][N] device, evaluation form): rows = towers Q
// towers, followed by the np special primes when `ext`.
int encode_many(fgb::Context* c, const double* re, const double* im, int nv, uint32_t slots, double scale, int towers,
                bool ext, u64* out) {
  const int n = (int)slots, N = c->N, rows = towers + (ext ? c->np : 0);
  FftTables T;
  if (int rc = tables_for(n, &T)) return rc;
  std::vector<double2> host((size_t)nv * n);
  for (size_t i = 0; i < host.size(); i++) host[i] = make_double2(re[i], im ? im[i] : 0.0);
  double2* a = nullptr;
  int* ovf = nullptr;
  if (cudaMallocFromPoolAsync(&a, host.size() * sizeof(double2), c->pool, c->stream) != cudaSuccess ||
      cudaMallocFromPoolAsync(&ovf, sizeof(int), c->pool, c->stream) != cudaSuccess)
    return fgb::set_last_error(FIDES_ENOMEM, "encoding workspace allocation failed");
  cudaError_t e = cudaMemcpyAsync(a, host.data(), host.size() * sizeof(double2), cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(ovf, 0, sizeof(int), c->stream);
  const long long bfly = (long long)nv * (n / 2);
  for (int len = n; len >= 2 && e == cudaSuccess; len >>= 1) {  // S_n^-1 first, ..., S_2^-1 last
    fft_stage_kernel<<<(unsigned)((bfly + kT - 1) / kT), kT, 0, c->stream>>>(a, nv, n, len, T.roots, T.rot, 1);
    fgb::count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    const long long total = (long long)nv * N;
    encode_place_kernel<<<(unsigned)((total + kT - 1) / kT), kT, 0, c->stream>>>(a, nv, n, ilog2(n), N, scale, rows,
                                                                                 towers, c->nq, c->d_pc, out, ovf);
    fgb::count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = c->ntt(out, out, nv, towers, 0, (long long)rows * N, false, c->stream);
  if (e == cudaSuccess && ext)
    e = c->ntt(out + (size_t)towers * N, out + (size_t)towers * N, nv, c->np, c->nq, (long long)rows * N, false,
               c->stream);
  int hovf = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hovf, ovf, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
  cudaFreeAsync(a, c->stream);
  cudaFreeAsync(ovf, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fgb::set_last_error(FIDES_ECUDA, cudaGetErrorString(e));
  if (hovf) return fgb::set_last_error(FIDES_EINVAL, "encoded coefficient exceeds 2^62: lower the scale");
  return FIDES_OK;
}

}  // namespace

extern "C" {

int fides_pt_encode(fides_ctx* ctx, const double* re, const double* im, uint32_t slots, double scale, uint32_t towers,
                    uint32_t* handle) {
  if (!ctx || !ctx->c || !re || !handle) return fgb::set_last_error(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  if (int rc = check_slots(c, slots)) return rc;
  if (towers < 1 || towers > (uint32_t)c->nq) return fgb::set_last_error(FIDES_EINVAL, "towers out of range");
  fgb::DevPt p;
  p.t = (int)towers;
  p.scale = scale;
  p.data = c->alloc_limbs(towers, c->stream);
  if (!p.data) return fgb::set_last_error(FIDES_ENOMEM, "plaintext allocation failed");
  if (int rc = encode_many(c, re, im, 1, slots, scale, (int)towers, false, p.data)) {
    c->free_limbs(p.data, c->stream);
    return rc;
  }
  const uint32_t h = c->next_handle++;
  c->pts[h] = p;
  *handle = h;
  return FIDES_OK;
}

int fides_pt_decode(fides_ctx* ctx, uint32_t pt, uint32_t slots, double* re, double* im) {
  if (!ctx || !ctx->c || !re || !im) return fgb::set_last_error(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  auto it = c->pts.find(pt);
  if (it == c->pts.end()) return fgb::set_last_error(FIDES_EINVAL, "unknown plaintext handle");
  if (int rc = check_slots(c, slots)) return rc;
  const fgb::DevPt& P = it->second;
  const int n = (int)slots, N = c->N, t = P.t >= 2 ? 2 : 1;
  FftTables T;
  if (int rc = tables_for(n, &T)) return rc;
  u64 q0inv = 0, q0inv_sh = 0;
  if (t == 2) {
    const u64 q0 = c->mod[0], q1 = c->mod[1];
    u64 x = q0 % q1, r = 1;  // q0^(q1-2) mod q1
    for (u64 e = q1 - 2; e; e >>= 1) {
      if (e & 1) r = (u64)((unsigned __int128)r * x % q1);
      x = (u64)((unsigned __int128)x * x % q1);
    }
    q0inv = r;
    q0inv_sh = (u64)(((unsigned __int128)r << 64) / q1);
  }
  u64* coeff = c->alloc_limbs(t, c->stream);
  double2* a = nullptr;
  if (!coeff || cudaMallocFromPoolAsync(&a, (size_t)n * sizeof(double2), c->pool, c->stream) != cudaSuccess) {
    c->free_limbs(coeff, c->stream);
    return fgb::set_last_error(FIDES_ENOMEM, "decoding workspace allocation failed");
  }
  cudaError_t e = c->ntt(P.data, coeff, 1, t, 0, (long long)t * N, true, c->stream);
  if (e == cudaSuccess) {
    decode_gather_kernel<<<(n + kT - 1) / kT, kT, 0, c->stream>>>(coeff, t, n, ilog2(n), N, 1.0 / P.scale, c->d_pc,
                                                                  q0inv, q0inv_sh, a);
    fgb::count_launch();
    e = cudaGetLastError();
  }
  for (int len = 2; len <= n && e == cudaSuccess; len <<= 1) {  // S_2 first, ..., S_n last
    fft_stage_kernel<<<(n / 2 + kT - 1) / kT, kT, 0, c->stream>>>(a, 1, n, len, T.roots, T.rot, 0);
    fgb::count_launch();
    e = cudaGetLastError();
  }
  std::vector<double2> host(n);
  if (e == cudaSuccess) e = cudaMemcpyAsync(host.data(), a, (size_t)n * sizeof(double2), cudaMemcpyDeviceToHost, c->stream);
  cudaFreeAsync(a, c->stream);
  c->free_limbs(coeff, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fgb::set_last_error(FIDES_ECUDA, cudaGetErrorString(e));
  for (int k = 0; k < n; k++) {
    re[k] = host[k].x;
    im[k] = host[k].y;
  }
  return FIDES_OK;
}

static int lt_create_slots(fides_ctx* ctx, uint32_t bs, uint32_t gs, int32_t stride, int32_t base, uint32_t towers,
                           bool ext, const double* re, const double* im, const uint8_t* present, uint32_t slots,
                           double scale, uint32_t* handle) {
  if (!ctx || !ctx->c || !re || !im || !present || !handle) return fgb::set_last_error(FIDES_EINVAL, "null argument");
  fgb::Context* c = ctx->c;
  if (int rc = check_slots(c, slots)) return rc;
  if (towers < 1 || towers > (uint32_t)c->nq) return fgb::set_last_error(FIDES_EINVAL, "towers out of range");
  const size_t nd = (size_t)bs * gs, per = (size_t)(towers + (ext ? c->np : 0)) * c->N;
  std::vector<double> r, i;
  std::vector<size_t> idx;
  for (size_t d = 0; d < nd; d++)
    if (present[d]) {
      idx.push_back(d);
      r.insert(r.end(), re + d * slots, re + (d + 1) * slots);
      i.insert(i.end(), im + d * slots, im + (d + 1) * slots);
    }
  u64* enc = nullptr;
  if (!idx.empty() && cudaMalloc(&enc, idx.size() * per * sizeof(u64)) != cudaSuccess)
    return fgb::set_last_error(FIDES_ENOMEM, "diagonal encoding allocation failed");
  int rc = FIDES_OK;
  if (!idx.empty()) rc = encode_many(c, r.data(), i.data(), (int)idx.size(), slots, scale, (int)towers, ext, enc);
  u64* full = nullptr;
  if (rc == FIDES_OK && cudaMalloc(&full, nd * per * sizeof(u64)) != cudaSuccess)
    rc = fgb::set_last_error(FIDES_ENOMEM, "diagonal allocation failed");
  if (rc == FIDES_OK) {  // everything on the context stream (it does not synchronise with the legacy stream)
    cudaError_t e = cudaMemsetAsync(full, 0, nd * per * sizeof(u64), c->stream);
    for (size_t k = 0; k < idx.size() && e == cudaSuccess; k++)
      e = cudaMemcpyAsync(full + idx[k] * per, enc + k * per, per * sizeof(u64), cudaMemcpyDeviceToDevice, c->stream);
    const uint64_t* d = reinterpret_cast<const uint64_t*>(full);
    rc = e != cudaSuccess ? fgb::set_last_error(FIDES_ECUDA, cudaGetErrorString(e))
         : ext            ? fides_lt_create_strided_ext(ctx, bs, gs, stride, base, towers, d, present, scale, handle)
                          : fides_lt_create_strided(ctx, bs, gs, stride, base, towers, d, present, scale, handle);
  }
  cudaStreamSynchronize(c->stream);
  cudaFree(enc);
  cudaFree(full);
  return rc;
}

int fides_lt_create_slots(fides_ctx* ctx, uint32_t bs, uint32_t gs, int32_t stride, int32_t base, uint32_t towers,
                          const double* re, const double* im, const uint8_t* present, uint32_t slots, double scale,
                          uint32_t* handle) {
  return lt_create_slots(ctx, bs, gs, stride, base, towers, false, re, im, present, slots, scale, handle);
}

int fides_lt_create_slots_ext(fides_ctx* ctx, uint32_t bs, uint32_t gs, int32_t stride, int32_t base,
                              uint32_t towers, const double* re, const double* im, const uint8_t* present,
                              uint32_t slots, double scale, uint32_t* handle) {
  return lt_create_slots(ctx, bs, gs, stride, base, towers, true, re, im, present, slots, scale, handle);
}

}  // extern "C"
