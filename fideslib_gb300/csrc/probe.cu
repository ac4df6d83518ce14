// Diagnostic microbenchmarks of the GPU units that bound this engine's kernels (fides_probe_pipes, declared in
// include/fideslib_gb300.h; no counterpart in the reference).  Every kernel here works on registers only and writes
// one word per thread into a buffer sized for the grid, so the runs are bounded and fault-free; bench.py reports the
// results beside the kernels they explain:
//   * 32-bit multiply-add (IMAD) and 32x32 -> 64-bit multiply-add (IMAD.WIDE) rates: the integer pipe every 64-bit
//     modular product is built from;
//   * the Harvey/Shoup butterfly of the forward NTT (shoup_lazy4 + the lazy add / subtract, arith.cuh), in
//     butterflies per clock per SM: the ceiling of the NTT kernels' butterfly work;
//   * the legacy warp-level INT8 tensor product (mma.sync m16n8k32 s8 -> s32), the only INT8 tensor path sm_103a
//     offers (tcgen05.mma kind::i8 is not supported on sm_103a: ptxas rejects it), for an 8-bit-sliced basis
//     conversion;
//   * the spacing of back-to-back launches of an empty kernel (launch-bound chains).
#include <cuda_runtime.h>

#include "../../include/fideslib_gb300.h"
#include "arith.cuh"

namespace fgb {
int set_last_error(int code, const char* msg);
}

namespace {

using fgb::u64;

__global__ void probe_imad(int iters, unsigned* out) {
  unsigned x[8], m = threadIdx.x | 1;
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = threadIdx.x + k;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(x[k]) : "r"(m), "r"(k));
  }
  unsigned s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void probe_imad_wide(int iters, unsigned* out) {
  unsigned long long x[8];
  const unsigned m = threadIdx.x | 1;
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = threadIdx.x + k;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++)
      asm volatile("mad.wide.u32 %0, %1, %2, %0;" : "+l"(x[k]) : "r"((unsigned)x[k]), "r"(m));
  }
  unsigned long long s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = (unsigned)(s ^ (s >> 32));
}

// Eight independent forward butterflies per thread and iteration, the NTT's exact arithmetic.
__global__ void probe_butterfly(int iters, u64 p, u64 w, u64 wsh, unsigned* out) {
  const u64 negp = 0ull - p, p4 = 4 * p;
  u64 X[8], Y[8];
#pragma unroll
  for (int k = 0; k < 8; k++) {
    X[k] = (threadIdx.x * 977ull + k) % p;
    Y[k] = (threadIdx.x * 131ull + 7 * k) % p;
  }
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 8; k++) {
      const u64 x = X[k] >= 2 * p4 ? X[k] - 2 * p4 : X[k];
      const u64 t = fgb::shoup_lazy4(Y[k], w, wsh, negp);
      X[k] = x + t;
      Y[k] = x - t + p4;
    }
  }
  u64 s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += X[k] ^ Y[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = (unsigned)(s ^ (s >> 32));
}

__global__ void probe_mma_s8(int iters, unsigned* out) {
  int a0 = threadIdx.x, a1 = a0 * 3, a2 = a0 * 5, a3 = a0 * 7, b0 = a0 ^ 0x55, b1 = a0 ^ 0x33;
  int c[4][4] = {};
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 4; k++)
      asm volatile("mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                   "{%0,%1,%2,%3};"
                   : "+r"(c[k][0]), "+r"(c[k][1]), "+r"(c[k][2]), "+r"(c[k][3])
                   : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
  }
  int s = 0;
#pragma unroll
  for (int k = 0; k < 4; k++) s += c[k][0] + c[k][1] + c[k][2] + c[k][3];
  out[blockIdx.x * blockDim.x + threadIdx.x] = (unsigned)s;
}

__global__ void probe_empty() {}

}  // namespace

extern "C" int fides_probe_pipes(fides_probe_result* r) {
  if (!r) return fgb::set_last_error(FIDES_EINVAL, "null argument");
  int dev = 0, sms = 0, khz = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) ||
      cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev))
    return fgb::set_last_error(FIDES_ENODEV, "no usable CUDA device");
  const int blocks = sms * 8, threads = 256, iters = 2048;
  unsigned* out = nullptr;
  if (cudaMalloc(&out, (size_t)blocks * threads * sizeof(unsigned)) != cudaSuccess)
    return fgb::set_last_error(FIDES_ENOMEM, "probe buffer");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto timed = [&](auto launch) {
    float best = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
      cudaEventRecord(e0);
      launch();
      cudaEventRecord(e1);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep && ms < best) best = ms;  // the first run warms up
    }
    return (double)best * 1e-3;
  };
  const double lanes = (double)blocks * threads * iters * 8;
  const double per_clk_sm = 1.0 / ((double)sms * khz * 1e3);
  *r = fides_probe_result{};
  r->sms = (uint32_t)sms;
  r->clock_mhz = khz / 1e3;
  double t = timed([&] { probe_imad<<<blocks, threads>>>(iters, out); });
  r->imad32_per_clk_sm = lanes / t * per_clk_sm;
  t = timed([&] { probe_imad_wide<<<blocks, threads>>>(iters, out); });
  r->imad_wide_per_clk_sm = lanes / t * per_clk_sm;
  const u64 p = 1152921504606584833ull;  // a 60-bit prime = 1 mod 2^17
  const u64 w = 0x0123456789abcdefull % p, wsh = (u64)(((unsigned __int128)w << 64) / p);
  t = timed([&] { probe_butterfly<<<blocks, threads>>>(iters, p, w, wsh, out); });
  r->butterflies_per_clk_sm = lanes / t * per_clk_sm;
  t = timed([&] { probe_mma_s8<<<blocks, threads>>>(iters, out); });
  r->int8_mma_tops = (double)blocks * (threads / 32) * iters * 4 * 4096 * 2 / t / 1e12;
  const int chain = 1000;
  t = timed([&] {
    for (int i = 0; i < chain; i++) probe_empty<<<64, 128>>>();
  });
  r->launch_spacing_us = t / chain * 1e6;
  const cudaError_t e = cudaDeviceSynchronize();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return fgb::set_last_error(FIDES_ECUDA, cudaGetErrorString(e));
  return FIDES_OK;
}
