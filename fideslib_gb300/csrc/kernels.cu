// Element-wise and basis-conversion kernels of the CKKS key-switching pipeline.
//
// Reference counterparts: DecompAndModUpConv (src/CKKS/Conv.cu:258-407), ModDown2 (src/CKKS/Conv.cu:26-133),
// fusedDotKSK_2_ (src/CKKS/ElemenwiseBatchKernels.cu:202-275), binomialMult_/binomialSquare_
// (ElemenwiseBatchKernels.cu:1363-1510), moddown_fusion / rescale_fusion (src/NTTfusions.cuh:214-252),
// SwitchModulus (src/CKKS/Rescale.cuh:44-64) and automorph_ (src/Rotation.cuh:14-26).
//
// The basis conversions accumulate sum_i y_i * c_ij exactly: both factors are < 2^60 and are split into
// 30-bit halves, so each product is four 32x32->64 multiply-adds into four 64-bit accumulators (at most 16
// terms per accumulator before folding into a 128-bit total), then one 128-bit reduction per output.
#include <atomic>

#include "kernels.cuh"

namespace fgb {

static std::atomic<unsigned long long> g_launches{0};
void count_launch(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
unsigned long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

namespace {

constexpr int kT = 256;
constexpr u64 kMask30 = (1ull << 30) - 1;

struct Acc4 {
  u64 a0, a1, a2, a3;  // lo*lo, lo*hi, hi*lo, hi*hi
};

__device__ __forceinline__ void acc4_mac(Acc4& A, uint32_t yl, uint32_t yh, uint32_t cl, uint32_t ch) {
  A.a0 += (u64)yl * cl;
  A.a1 += (u64)yl * ch;
  A.a2 += (u64)yh * cl;
  A.a3 += (u64)yh * ch;
}

// (hi, lo) += a0 + (a1 + a2) * 2^30 + a3 * 2^60
__device__ __forceinline__ void acc4_fold(const Acc4& A, u64& hi, u64& lo) {
  u64 m = A.a1 + A.a2;
  u64 mc = m < A.a1 ? 1ull : 0ull;
  u64 l, c;
  l = lo + A.a0;
  c = l < lo;
  hi += c;
  lo = l;
  const u64 t_lo = m << 30, t_hi = (m >> 34) | (mc << 30);
  l = lo + t_lo;
  c = l < lo;
  hi += t_hi + c;
  lo = l;
  const u64 u_lo = A.a3 << 60, u_hi = A.a3 >> 4;
  l = lo + u_lo;
  c = l < lo;
  hi += u_hi + c;
  lo = l;
}

__device__ __forceinline__ uint32_t brev_n(uint32_t x, int logN) { return __brev(x) >> (32 - logN); }

// ---------------------------------------------------------------------------------------------------------
template <int MAXS>
__global__ void __launch_bounds__(kT) modup_conv_kernel(const u64* __restrict__ coeff, u64* __restrict__ conv,
                                                        long long conv_stride, KsDims k, CrtTables c,
                                                        const PrimeConst* __restrict__ pc) {
  extern __shared__ uint2 cs[];  // [s][nout] 30-bit slices of Qhat
  const int d = blockIdx.y;
  const int start = d * c.alpha;
  const int s = min(c.alpha, k.t - start);
  const int nout = k.t - s + c.np;
  const int base = (d * c.alpha + (s - 1)) * c.alpha;
  for (int idx = threadIdx.x; idx < s * nout; idx += kT) {
    const int i = idx / nout, jj = idx - i * nout;
    const int tower = jj < start ? jj : (jj < k.t - s ? jj + s : c.nq + (jj - (k.t - s)));
    const uint32_t* src = c.mu_qhat + ((size_t)(base + i) * c.ntow + tower) * 2;
    cs[idx] = make_uint2(src[0], src[1]);
  }
  __syncthreads();
  const int n = blockIdx.x * kT + threadIdx.x;
  uint32_t yl[MAXS], yh[MAXS];
#pragma unroll
  for (int i = 0; i < MAXS; i++) {
    if (i < s) {
      const ulonglong2 w = c.mu_qhinv[base + i];
      const u64 q = pc[start + i].p;
      const u64 y = shoup(coeff[(size_t)(start + i) * k.N + n], w.x, w.y, q);
      yl[i] = (uint32_t)(y & kMask30);
      yh[i] = (uint32_t)(y >> 30);
    } else {
      yl[i] = 0;
      yh[i] = 0;
    }
  }
  u64* out = conv + d * conv_stride + n;
#pragma unroll 1
  for (int jj = 0; jj < nout; jj++) {
    const int tower = jj < start ? jj : (jj < k.t - s ? jj + s : c.nq + (jj - (k.t - s)));
    u64 hi = 0, lo = 0;
#pragma unroll
    for (int i0 = 0; i0 < MAXS; i0 += 16) {
      Acc4 A{0, 0, 0, 0};
#pragma unroll
      for (int i = i0; i < i0 + 16 && i < MAXS; i++) {
        if (i < s) {
          const uint2 cc = cs[i * nout + jj];
          acc4_mac(A, yl[i], yh[i], cc.x, cc.y);
        }
      }
      acc4_fold(A, hi, lo);
    }
    out[(size_t)jj * k.N] = reduce128(hi, lo, pc[tower]);
  }
}

__global__ void __launch_bounds__(kT) ks_inner_kernel(const u64* __restrict__ a_eval, const u64* __restrict__ conv,
                                                      long long conv_stride, const u64* __restrict__ key,
                                                      u64* __restrict__ inner, KsDims k, CrtTables c,
                                                      const PrimeConst* __restrict__ pc) {
  const int j = blockIdx.y;
  const int ext = k.t + c.np;
  const int tower = j < k.t ? j : c.nq + (j - k.t);
  const int n = blockIdx.x * kT + threadIdx.x;
  const size_t N = k.N;
  U128 acc0{0, 0}, acc1{0, 0};
#pragma unroll 1
  for (int d = 0; d < k.beta; d++) {
    const int start = d * c.alpha;
    const int s = min(c.alpha, k.t - start);
    u64 D;
    if (j >= start && j < start + s) {
      D = a_eval[(size_t)j * N + n];
    } else {
      const int jj = j < start ? j : j - s;
      D = conv[d * conv_stride + (size_t)jj * N + n];
    }
    const u64 ka = key[((size_t)(0 * c.dnum + d) * c.ntow + tower) * N + n];
    const u64 kb = key[((size_t)(1 * c.dnum + d) * c.ntow + tower) * N + n];
    mac(acc0, D, kb);
    mac(acc1, D, ka);
  }
  const PrimeConst& P = pc[tower];
  inner[(size_t)j * N + n] = reduce128(acc0.hi, acc0.lo, P);
  inner[((size_t)ext + j) * N + n] = reduce128(acc1.hi, acc1.lo, P);
}

template <int MAXK>
__global__ void __launch_bounds__(kT) moddown_conv_kernel(const u64* __restrict__ inner, long long in_stride,
                                                          u64* __restrict__ conv_out, long long out_stride, KsDims k,
                                                          CrtTables c, const PrimeConst* __restrict__ pc) {
  extern __shared__ uint2 cs[];  // [np][t]
  const int np = c.np, t = k.t;
  for (int idx = threadIdx.x; idx < np * t; idx += kT) {
    const int kk = idx / t, j = idx - kk * t;
    const uint32_t* src = c.md_phat + ((size_t)kk * c.nq + j) * 2;
    cs[idx] = make_uint2(src[0], src[1]);
  }
  __syncthreads();
  const int poly = blockIdx.y;
  const int n = blockIdx.x * kT + threadIdx.x;
  const u64* x = inner + poly * in_stride + (size_t)t * k.N + n;
  uint32_t yl[MAXK], yh[MAXK];
#pragma unroll
  for (int i = 0; i < MAXK; i++) {
    if (i < np) {
      const ulonglong2 w = c.md_phinv[i];
      const u64 y = shoup(x[(size_t)i * k.N], w.x, w.y, pc[c.nq + i].p);
      yl[i] = (uint32_t)(y & kMask30);
      yh[i] = (uint32_t)(y >> 30);
    } else {
      yl[i] = 0;
      yh[i] = 0;
    }
  }
  u64* out = conv_out + poly * out_stride + n;
#pragma unroll 1
  for (int j = 0; j < t; j++) {
    u64 hi = 0, lo = 0;
#pragma unroll
    for (int i0 = 0; i0 < MAXK; i0 += 16) {
      Acc4 A{0, 0, 0, 0};
#pragma unroll
      for (int i = i0; i < i0 + 16 && i < MAXK; i++) {
        if (i < np) {
          const uint2 cc = cs[i * t + j];
          acc4_mac(A, yl[i], yh[i], cc.x, cc.y);
        }
      }
      acc4_fold(A, hi, lo);
    }
    out[(size_t)j * k.N] = reduce128(hi, lo, pc[j]);
  }
}

__global__ void __launch_bounds__(kT) moddown_epilogue_kernel(const u64* __restrict__ inner, long long in_stride,
                                                              const u64* __restrict__ conv, long long conv_stride,
                                                              const u64* __restrict__ add0,
                                                              const u64* __restrict__ add1, u64* __restrict__ out,
                                                              long long out_stride, uint32_t galois_inv, KsDims k,
                                                              CrtTables c, const PrimeConst* __restrict__ pc) {
  const int j = blockIdx.y, poly = blockIdx.z;
  const int n = blockIdx.x * kT + threadIdx.x;
  const size_t N = k.N;
  const u64 q = pc[j].p;
  const ulonglong2 w = c.md_pinv[j];
  const u64 x = inner[poly * in_stride + (size_t)j * N + n];
  const u64 y = conv[poly * conv_stride + (size_t)j * N + n];
  u64 v = shoup(sub_mod(x, y, q), w.x, w.y, q);
  const u64* add = poly == 0 ? add0 : add1;
  if (add) v = add_mod(v, add[(size_t)j * N + n], q);
  uint32_t pos = n;
  if (galois_inv != 1) {
    const uint32_t idx = brev_n(n, k.logN);
    const uint32_t jj = (uint32_t)((((2ull * idx + 1) * galois_inv) & (2ull * N - 1)) >> 1);
    pos = brev_n(jj, k.logN);
  }
  out[poly * out_stride + (size_t)j * N + pos] = v;
}

__global__ void __launch_bounds__(kT) tensor_kernel(const u64* __restrict__ x, const u64* __restrict__ y,
                                                    u64* __restrict__ d, int t, int N,
                                                    const PrimeConst* __restrict__ pc) {
  const int j = blockIdx.y;
  const size_t o = (size_t)j * N + blockIdx.x * kT + threadIdx.x;
  const size_t P = (size_t)t * N;
  const PrimeConst& c = pc[j];
  const u64 x0 = x[o], x1 = x[P + o], y0 = y[o], y1 = y[P + o];
  d[o] = mul_mod(x0, y0, c);
  d[P + o] = add_mod(mul_mod(x0, y1, c), mul_mod(x1, y0, c), c.p);
  d[2 * P + o] = mul_mod(x1, y1, c);
}

__global__ void __launch_bounds__(kT) addsub_kernel(const u64* __restrict__ x, const u64* __restrict__ y,
                                                    u64* __restrict__ out, int t, int N, int sub,
                                                    const PrimeConst* __restrict__ pc) {
  const int j = blockIdx.y, poly = blockIdx.z;
  const size_t o = ((size_t)poly * t + j) * N + blockIdx.x * kT + threadIdx.x;
  const u64 p = pc[j].p;
  out[o] = sub ? sub_mod(x[o], y[o], p) : add_mod(x[o], y[o], p);
}

__global__ void __launch_bounds__(kT) rescale_switch_kernel(const u64* __restrict__ top, long long top_stride,
                                                            u64* __restrict__ tmp, int t, int N,
                                                            const PrimeConst* __restrict__ pc) {
  const int i = blockIdx.y, poly = blockIdx.z;
  const int n = blockIdx.x * kT + threadIdx.x;
  const PrimeConst& om = pc[t - 1];
  const PrimeConst& nm = pc[i];
  // OpenFHE NativeVector::SwitchModulus: values above om/2 are lifted to v - om before reduction mod nm.
  const u64 om_mod_nm = shoup(om.p, 1ull, nm.one_sh, nm.p);
  const u64 diff = nm.p - om_mod_nm;
  u64 v = top[poly * top_stride + n];
  if (v > (om.p >> 1)) v += diff;
  v = shoup(v, 1ull, nm.one_sh, nm.p);
  tmp[((size_t)poly * (t - 1) + i) * N + n] = v;
}

__global__ void __launch_bounds__(kT) rescale_epilogue_kernel(const u64* __restrict__ x, long long x_stride,
                                                              const u64* __restrict__ tmp, u64* __restrict__ out,
                                                              int t, int N, CrtTables c,
                                                              const PrimeConst* __restrict__ pc) {
  const int i = blockIdx.y, poly = blockIdx.z;
  const int n = blockIdx.x * kT + threadIdx.x;
  const u64 q = pc[i].p;
  const ulonglong2 w = c.rs_qinv[(size_t)(t - 1) * c.nq + i];
  const u64 a = x[poly * x_stride + (size_t)i * N + n];
  const u64 b = tmp[((size_t)poly * (t - 1) + i) * N + n];
  out[((size_t)poly * (t - 1) + i) * N + n] = shoup(sub_mod(a, b, q), w.x, w.y, q);
}

__global__ void __launch_bounds__(kT) automorph_kernel(const u64* __restrict__ in, u64* __restrict__ out, int N,
                                                       int logN, uint32_t galois) {
  const int l = blockIdx.y;
  const uint32_t pos = blockIdx.x * kT + threadIdx.x;
  const uint32_t j = brev_n(pos, logN);
  const uint32_t idx = (uint32_t)((((2ull * j + 1) * galois) & (2ull * N - 1)) >> 1);
  out[(size_t)l * N + pos] = in[(size_t)l * N + brev_n(idx, logN)];
}

}  // namespace

cudaError_t launch_modup_conv(const u64* coeff, u64* conv, long long conv_stride, const KsDims& k,
                              const CrtTables& c, const PrimeConst* pc, cudaStream_t s) {
  const int maxout = k.t + c.np;
  const size_t smem = sizeof(uint2) * c.alpha * maxout;
  dim3 grid(k.N / kT, k.beta);
  if (c.alpha <= 16) {
    modup_conv_kernel<16><<<grid, kT, smem, s>>>(coeff, conv, conv_stride, k, c, pc);
  } else if (c.alpha <= 32) {
    modup_conv_kernel<32><<<grid, kT, smem, s>>>(coeff, conv, conv_stride, k, c, pc);
  } else {
    return cudaErrorInvalidValue;
  }
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_ks_inner(const u64* a_eval, const u64* conv, long long conv_stride, const u64* key, u64* inner,
                            const KsDims& k, const CrtTables& c, const PrimeConst* pc, cudaStream_t s) {
  dim3 grid(k.N / kT, k.t + c.np);
  ks_inner_kernel<<<grid, kT, 0, s>>>(a_eval, conv, conv_stride, key, inner, k, c, pc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_moddown_conv(const u64* inner, long long poly_stride_in, u64* conv_out, long long poly_stride_out,
                                int npolys, const KsDims& k, const CrtTables& c, const PrimeConst* pc,
                                cudaStream_t s) {
  const size_t smem = sizeof(uint2) * c.np * k.t;
  dim3 grid(k.N / kT, npolys);
  if (c.np <= 16) {
    moddown_conv_kernel<16><<<grid, kT, smem, s>>>(inner, poly_stride_in, conv_out, poly_stride_out, k, c, pc);
  } else if (c.np <= 32) {
    moddown_conv_kernel<32><<<grid, kT, smem, s>>>(inner, poly_stride_in, conv_out, poly_stride_out, k, c, pc);
  } else {
    return cudaErrorInvalidValue;
  }
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_moddown_epilogue(const u64* inner, long long in_stride, const u64* conv, long long conv_stride,
                                    const u64* add0, const u64* add1, u64* out, long long out_stride, int npolys,
                                    uint32_t galois_inv, const KsDims& k, const CrtTables& c, const PrimeConst* pc,
                                    cudaStream_t s) {
  dim3 grid(k.N / kT, k.t, npolys);
  moddown_epilogue_kernel<<<grid, kT, 0, s>>>(inner, in_stride, conv, conv_stride, add0, add1, out, out_stride,
                                              galois_inv, k, c, pc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_tensor(const u64* x, const u64* y, u64* d, int t, int N, const PrimeConst* pc, cudaStream_t s) {
  dim3 grid(N / kT, t);
  tensor_kernel<<<grid, kT, 0, s>>>(x, y, d, t, N, pc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_addsub(const u64* x, const u64* y, u64* out, int npolys, int t, int N, bool sub,
                          const PrimeConst* pc, cudaStream_t s) {
  dim3 grid(N / kT, t, npolys);
  addsub_kernel<<<grid, kT, 0, s>>>(x, y, out, t, N, sub ? 1 : 0, pc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_rescale_switch(const u64* top, long long top_stride, u64* tmp, int npolys, int t, int N,
                                  const PrimeConst* pc, cudaStream_t s) {
  dim3 grid(N / kT, t - 1, npolys);
  rescale_switch_kernel<<<grid, kT, 0, s>>>(top, top_stride, tmp, t, N, pc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_rescale_epilogue(const u64* x, long long x_stride, const u64* tmp, u64* out, int npolys, int t,
                                    int N, const CrtTables& c, const PrimeConst* pc, cudaStream_t s) {
  dim3 grid(N / kT, t - 1, npolys);
  rescale_epilogue_kernel<<<grid, kT, 0, s>>>(x, x_stride, tmp, out, t, N, c, pc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_automorph(const u64* in, u64* out, int nlimbs, int N, int logN, uint32_t galois, cudaStream_t s) {
  dim3 grid(N / kT, nlimbs);
  automorph_kernel<<<grid, kT, 0, s>>>(in, out, N, logN, galois);
  count_launch();
  return cudaGetLastError();
}

}  // namespace fgb
