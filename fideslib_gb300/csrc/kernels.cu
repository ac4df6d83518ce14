// Job-batched kernels of the CKKS key-switching pipeline and the element-wise ops around it.
//
// Reference counterparts: DecompAndModUpConv (src/CKKS/Conv.cu:258-407), ModDown2 (src/CKKS/Conv.cu:26-133),
// fusedDotKSK_2_ (src/CKKS/ElemenwiseBatchKernels.cu:202-275), binomialMult_/binomialSquare_
// (ElemenwiseBatchKernels.cu:1363-1510), moddown_fusion / rescale_fusion (src/NTTfusions.cuh:214-252),
// SwitchModulus (src/CKKS/Rescale.cuh:44-64), automorph_ (src/Rotation.cuh:14-26) and add_/sub_
// (src/AddSub.cu:10-123).  The reference launches these per limb batch of one ciphertext; here each launch
// covers up to kMaxJobs ciphertexts at independent levels (grid.z = job).
//
// The basis conversions accumulate sum_i y_i * c_ij exactly: both factors are < 2^60 and are split into
// 30-bit halves, so each product is four 32x32->64 multiply-adds into four 64-bit accumulators (at most 16
// terms per accumulator before folding into a 128-bit total), then one 128-bit reduction per output.
#include <algorithm>
#include <atomic>

#include "kernels.cuh"
#include "ntt.cuh"

namespace fgb {

static std::atomic<unsigned long long> g_launches{0};
void count_launch(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
unsigned long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

bool pdl_for(long long ctas) {
  static std::atomic<int> sms[64];  // SM count per device, 0 until first asked
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
  int n = sms[dev].load(std::memory_order_relaxed);
  if (n == 0) {
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return false;
    sms[dev].store(n, std::memory_order_relaxed);
  }
  return ctas < n;
}

namespace {

constexpr int kT = 256;
constexpr u64 kMask30 = (1ull << 30) - 1;

struct Acc4 {
  u64 a0, a1, a2, a3;  // lo*lo, lo*hi, hi*lo, hi*hi
};

// a += x*y (64-bit) as a 32-bit multiply-add pair with a carry chain: on GB300 this issues faster than the 32x32->64
// wide multiply-add the plain C expression compiles to (22.5 against 20.6 accumulations per clock per SM).
__device__ __forceinline__ void mac64(u64& a, uint32_t x, uint32_t y) {
  asm("{\n\t.reg .u32 l,h;\n\tmov.b64 {l,h}, %0;\n\tmad.lo.cc.u32 l, %1, %2, l;\n\t"
      "madc.hi.u32 h, %1, %2, h;\n\tmov.b64 %0, {l,h};\n\t}"
      : "+l"(a)
      : "r"(x), "r"(y));
}

__device__ __forceinline__ void acc4_mac(Acc4& A, uint32_t yl, uint32_t yh, uint32_t cl, uint32_t ch) {
  mac64(A.a0, yl, cl);
  mac64(A.a1, yl, ch);
  mac64(A.a2, yh, cl);
  mac64(A.a3, yh, ch);
}

// Three-product (Karatsuba) form of the same sum: y*c = yl*cl + (ys*cs - yl*cl - yh*ch) * 2^30 + yh*ch * 2^60 with
// ys = yl + yh and cs = cl + ch (31 bits each).  am accumulates ys*cs modulo 2^64; the middle sum it stands for,
// sum (yl*ch + yh*cl), is below 2^64 while an accumulator holds at most kAcc3Terms terms (16 cross products
// < 2^60), so am - a0 - a3 taken modulo 2^64 is exact.  One multiply-add pair fewer per term than Acc4 (three
// instead of four 32x32 products, whose high halves issue at half rate), for two more additions per term.
constexpr int kAcc3Terms = 8;
struct Acc3 {
  u64 a0, am, a3;  // lo*lo, (lo+hi)*(lo+hi) mod 2^64, hi*hi
};
__device__ __forceinline__ void acc3_mac(Acc3& A, uint32_t yl, uint32_t yh, uint32_t ys, uint32_t cl, uint32_t ch) {
  mac64(A.a0, yl, cl);
  mac64(A.am, ys, cl + ch);
  mac64(A.a3, yh, ch);
}
// (hi, lo) += a0 + (am - a0 - a3) * 2^30 + a3 * 2^60
__device__ __forceinline__ void acc3_fold(const Acc3& A, u64& hi, u64& lo) {
  const u64 m = A.am - A.a0 - A.a3;
  u64 l = lo + A.a0;
  hi += (l < lo);
  lo = l;
  l = lo + (m << 30);
  hi += (m >> 34) + (l < lo);
  lo = l;
  l = lo + (A.a3 << 60);
  hi += (A.a3 >> 4) + (l < lo);
  lo = l;
}

// (hi, lo) += a0 + (a1 + a2) * 2^30 + a3 * 2^60
__device__ __forceinline__ void acc4_fold(const Acc4& A, u64& hi, u64& lo) {
  const u64 m = A.a1 + A.a2;
  const u64 mc = m < A.a1 ? 1ull : 0ull;
  u64 l = lo + A.a0;
  hi += (l < lo);
  lo = l;
  const u64 t_lo = m << 30, t_hi = (m >> 34) | (mc << 30);
  l = lo + t_lo;
  hi += t_hi + (l < lo);
  lo = l;
  const u64 u_lo = A.a3 << 60, u_hi = A.a3 >> 4;
  l = lo + u_lo;
  hi += u_hi + (l < lo);
  lo = l;
}

__device__ __forceinline__ uint32_t brev_n(uint32_t x, int logN) { return __brev(x) >> (32 - logN); }

// Tower id of converted row jj of digit [start, start+s) at t active towers.
__device__ __forceinline__ int conv_tower(int jj, int start, int s, int t, int nq) {
  return jj < start ? jj : (jj < t - s ? jj + s : nq + (jj - (t - s)));
}

// ---------------------------------------------------------------------------------------------------------
// Basis conversion core: for NC adjacent coefficients (NC = 1 or 2), outputs sum_{i<S} y_i * c_{i,jj} mod m_jj for
// jj < nout, with the S inputs y_i (already multiplied by the Qhat^-1 / Phat^-1 factor) held in registers as 30-bit
// halves and the constants c_{i,jj} staged in shared memory as 30-bit halves (one shared load serves the NC
// coefficients).  S is a compile-time constant so no multiply-add is issued for absent towers.  Every output feeds
// a forward NTT, which accepts residues in [0, 8p), so the outputs are left unreduced in that range (the NTT's own
// output is fully reduced).  Up to 10 inputs two outputs are interleaved (unroll 2: the reduction of one overlaps the
// products of the next; the ModUp instance is held to three CTAs per SM for it): 64-rotation step 7,855 -> 7,905
// ops/s, with larger digits the extra registers spill.
template <int S, int NC, class TowerOf>
__device__ __forceinline__ void conv_rows(const uint32_t (&yl)[NC][S], const uint32_t (&yh)[NC][S], const uint2* cs,
                                          int nout, u64* out, size_t stride, const PrimeConst* __restrict__ pc,
                                          TowerOf tower_of) {
#pragma unroll(S <= 10 ? 2 : 1)
  for (int jj = 0; jj < nout; jj++) {
    u64 hi[NC], lo[NC];
#pragma unroll
    for (int k = 0; k < NC; k++) hi[k] = lo[k] = 0;
#pragma unroll
    for (int i0 = 0; i0 < S; i0 += 16) {
      Acc4 A[NC];
#pragma unroll
      for (int k = 0; k < NC; k++) A[k] = Acc4{0, 0, 0, 0};
#pragma unroll
      for (int i = i0; i < i0 + 16 && i < S; i++) {
        const uint2 cc = cs[i * nout + jj];
#pragma unroll
        for (int k = 0; k < NC; k++) acc4_mac(A[k], yl[k][i], yh[k][i], cc.x, cc.y);
      }
#pragma unroll
      for (int k = 0; k < NC; k++) acc4_fold(A[k], hi[k], lo[k]);
    }
    const PrimeConst& P = pc[tower_of(jj)];
    if constexpr (NC == 2)
      *reinterpret_cast<ulonglong2*>(out + (size_t)jj * stride) =
          make_ulonglong2(reduce128_lazy8(hi[0], lo[0], P), reduce128_lazy8(hi[1], lo[1], P));
    else
      out[(size_t)jj * stride] = reduce128_lazy8(hi[0], lo[0], P);
  }
}

// Loads NC adjacent residues of row x (16 bytes when NC = 2), multiplies them by the Shoup constant w and splits
// them into 30-bit halves.
template <int NC>
__device__ __forceinline__ void load_split(const u64* x, ulonglong2 w, u64 p, uint32_t* lo, uint32_t* hi) {
  u64 y[NC];
  if constexpr (NC == 2) {
    const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(x);
    y[0] = v.x;
    y[1] = v.y;
  } else {
    y[0] = x[0];
  }
#pragma unroll
  for (int k = 0; k < NC; k++) {
    const u64 z = shoup(y[k], w.x, w.y, p);
    lo[k] = (uint32_t)(z & kMask30);
    hi[k] = (uint32_t)(z >> 30);
  }
}

template <int S, int NC>
__device__ __forceinline__ void modup_body(const KsJob& J, const Ring& r, const CrtTables& c,
                                           const PrimeConst* __restrict__ pc, int d, int start, int t, int nout,
                                           int base, const uint2* cs) {
  const int n = (blockIdx.x * kT + threadIdx.x) * NC;
  uint32_t yl[NC][S], yh[NC][S];
#pragma unroll
  for (int i = 0; i < S; i++) {
    uint32_t lo[NC], hi[NC];
    load_split<NC>(J.coeff + (size_t)(start + i) * r.N + n, c.mu_qhinv[base + i], pc[start + i].p, lo, hi);
#pragma unroll
    for (int k = 0; k < NC; k++) {
      yl[k][i] = lo[k];
      yh[k][i] = hi[k];
    }
  }
  const int nq = c.nq;
  conv_rows<S, NC>(yl, yh, cs, nout, J.conv + (size_t)d * (t + c.np) * r.N + n, (size_t)r.N, pc,
                   [=](int jj) { return conv_tower(jj, start, S, t, nq); });
}

// ModUp basis conversion: grid (N/512 (N/256 when MAXS > 16), rows = digits), two adjacent coefficients per thread
// (one for digits of more than 16 towers), all converted rows of one digit.  MAXS bounds the digit size the
// instance compiles (8, 10, 12, 16 or 32), so the common small digits do not pay for the registers of large ones.  The
// digit's 30-bit-sliced [Qhat_i]_{m_j} constants are staged in shared memory.
template <int MAXS>
__global__ void __launch_bounds__(kT, MAXS <= 10 ? 3 : 1) modup_conv_kernel(const __grid_constant__ KsBatch b, Ring r, CrtTables c,
                                                        const PrimeConst* __restrict__ pc) {
  pdl_prologue();
  extern __shared__ uint2 cs[];
  const int z = find_job(b.row_begin, b.njobs, (int)blockIdx.y);
  const KsJob& J = b.jobs[z];
  const int t = J.t, d = (int)blockIdx.y - b.row_begin[z];
  const int start = d * c.alpha;
  if (start >= t) return;
  const int s = min(c.alpha, t - start);
  const int nout = t - s + c.np;
  const int base = (d * c.alpha + (s - 1)) * c.alpha;
  for (int idx = threadIdx.x; idx < s * nout; idx += kT) {
    const int i = idx / nout, jj = idx - i * nout;
    const uint32_t* src = c.mu_qhat + ((size_t)(base + i) * c.ntow + conv_tower(jj, start, s, t, c.nq)) * 2;
    cs[idx] = make_uint2(src[0], src[1]);
  }
  __syncthreads();
  constexpr int NC = MAXS <= 16 ? 2 : 1;
#define FGB_MODUP_CASE(S_)                                              \
  case S_:                                                              \
    if constexpr (S_ <= MAXS) modup_body<S_, NC>(J, r, c, pc, d, start, t, nout, base, cs); \
    break;
  switch (s) {  // sizes above MAXS are not reached: launch_modup_conv picks the instance from alpha
    FGB_MODUP_CASE(1) FGB_MODUP_CASE(2) FGB_MODUP_CASE(3) FGB_MODUP_CASE(4) FGB_MODUP_CASE(5) FGB_MODUP_CASE(6)
    FGB_MODUP_CASE(7) FGB_MODUP_CASE(8) FGB_MODUP_CASE(9) FGB_MODUP_CASE(10) FGB_MODUP_CASE(11)
    FGB_MODUP_CASE(12) FGB_MODUP_CASE(13) FGB_MODUP_CASE(14) FGB_MODUP_CASE(15) FGB_MODUP_CASE(16)
    FGB_MODUP_CASE(20) FGB_MODUP_CASE(24) FGB_MODUP_CASE(28) FGB_MODUP_CASE(32)
    default:
      break;
  }
#undef FGB_MODUP_CASE
}

// Key inner product: grid (N / (512 iters), rows); a thread takes `iters` pairs of coefficients (16-byte loads),
// with its job, tower and row pointers worked out once.  Jobs are grouped by key; group g owns (tmax_g + np) * m_g
// rows, tmax_g its largest tower count and m_g its job count, ordered (tower row, job) with the job fastest, so the
// m_g blocks that read the same key values are scheduled back to back and a key shared by several ciphertexts (one
// rotation of a lock-step batch, the relinearisation key of a batch of products) is read from HBM about once, the
// other reads hitting L2.  When jobs of different groups share their digits (row_outer, set by the launcher) the
// rows are ordered (tower row, job) over the whole batch instead, (tmax + np) * njobs rows, so that both the digits
// and the keys of a row are read about once.  A block whose tower lies above its job's level exits.  Every digit's
// value and both key halves are loaded before any arithmetic; digits are split into 30-bit halves here and key
// values come split (launch_key_split), accumulated in one accumulator per half-key (Acc3 for four or more
// digits, Acc4 below: at most 8 terms); MAXB bounds beta at compile time.  Outputs are left in [0, 4p): the
// ModDown INTT takes them as they are and both epilogues reduce.
template <int MAXB>
__global__ void __launch_bounds__(kT, MAXB <= 3 ? 3 : 2)
    ks_inner_kernel(const __grid_constant__ KsBatch b, Ring r, CrtTables c, const PrimeConst* __restrict__ pc,
                    int iters) {
  pdl_prologue();
  int q, rr, tmax;
  if (b.row_outer) {  // block row y = rr * njobs + q
    q = (int)blockIdx.y % b.njobs;
    rr = (int)blockIdx.y / b.njobs;
    tmax = b.jobs[q].t;
    if (rr >= tmax + c.np) return;  // beyond this job's rows
  } else {
    const int G = find_job(b.row_begin, b.ngroups, (int)blockIdx.y);
    const int m = b.grp_begin[G + 1] - b.grp_begin[G];
    const int local = (int)blockIdx.y - b.row_begin[G];
    rr = local / m;
    tmax = (b.row_begin[G + 1] - b.row_begin[G]) / m - c.np;
    q = b.grp_begin[G] + (local - rr * m);
  }
  const KsJob& J = b.jobs[q];
  const int t = J.t;
  const int tower = rr < tmax ? rr : c.nq + (rr - tmax);
  if (tower < c.nq && tower >= t) return;  // a Q tower above this job's level
  const int ext = t + c.np, j = tower < c.nq ? tower : t + (tower - c.nq);
  const size_t N = r.N;
  const int beta = (t + c.alpha - 1) / c.alpha;
  const size_t khalf = (size_t)c.dnum * c.ntow * N, kstep = (size_t)c.ntow * N;
  // Digit d's row j is the input's own tower (row j of a) inside the digit, else row jj of its converted block.
  // For three digits (three CTAs per SM, 80 registers) the rows are kept as 32-bit indices (negative: row -1-r of
  // a) and turned into pointers per iteration, so no 64-bit pointers stay live across the products: that instance
  // then has no register spills (68 bytes of spill stores with the pointers held).  The other instances spill less
  // with the pointers worked out once, so they keep that form (ptxas -v).
  constexpr bool kRowIndex = MAXB == 3;
  // Four or more digits (the bootstrap's dnum 5, whose inner products are bound by their multiply-add stream)
  // accumulate in the three-product form.  Three digits (dnum 3, three CTAs per SM at 80 registers) keep the
  // four-product form: there the three-product form's extra live sums spill (68 bytes, ptxas -v), and with fewer
  // digits the inner product is bound by its key reads; one or two digits keep it too.
  constexpr bool kKaratsuba = MAXB >= 4;
  static_assert(MAXB <= kAcc3Terms, "one accumulator chunk per half-key");
  const u64* src[MAXB];
  int srow[MAXB];
#pragma unroll
  for (int d = 0; d < MAXB; d++) {
    if (d >= beta) break;
    const int start = d * c.alpha;
    const int s = min(c.alpha, t - start);
    srow[d] = (j >= start && j < start + s) ? -1 - j : d * ext + (j < start ? j : j - s);
    if constexpr (!kRowIndex) src[d] = srow[d] < 0 ? J.a + (size_t)j * N : J.conv + (size_t)srow[d] * N;
  }
  const PrimeConst& P = pc[tower];
  const u64 p4 = 4 * P.p;
  const u64* key0 = J.key + (size_t)tower * N;
#pragma unroll 1
  for (int it = 0; it < iters; it++) {
    const int n = (((int)blockIdx.x * iters + it) * kT + (int)threadIdx.x) * 2;
    ulonglong2 D[MAXB], KA[MAXB], KB[MAXB];
    const u64* key = key0 + n;
#pragma unroll
    for (int d = 0; d < MAXB; d++) {
      if (d >= beta) break;
      const u64* sp;
      if constexpr (kRowIndex)
        sp = srow[d] < 0 ? J.a + (size_t)(-1 - srow[d]) * N : J.conv + (size_t)srow[d] * N;
      else
        sp = src[d];
      D[d] = *reinterpret_cast<const ulonglong2*>(sp + n);
      KA[d] = *reinterpret_cast<const ulonglong2*>(key + d * kstep);
      KB[d] = *reinterpret_cast<const ulonglong2*>(key + d * kstep + khalf);
    }
    u64 v0[2], v1[2];
#pragma unroll
    for (int e = 0; e < 2; e++) {
      u64 h0 = 0, l0 = 0, h1 = 0, l1 = 0;
      if constexpr (kKaratsuba) {
        Acc3 A0{0, 0, 0}, A1{0, 0, 0};
#pragma unroll
        for (int d = 0; d < MAXB; d++) {
          if (d >= beta) break;
          const u64 Dv = e ? D[d].y : D[d].x, ka = e ? KA[d].y : KA[d].x, kb = e ? KB[d].y : KB[d].x;
          const uint32_t dl = (uint32_t)(Dv & kMask30), dh = (uint32_t)(Dv >> 30);
          acc3_mac(A0, dl, dh, dl + dh, (uint32_t)kb, (uint32_t)(kb >> 32));
          acc3_mac(A1, dl, dh, dl + dh, (uint32_t)ka, (uint32_t)(ka >> 32));
        }
        acc3_fold(A0, h0, l0);
        acc3_fold(A1, h1, l1);
      } else {
        Acc4 A0{0, 0, 0, 0}, A1{0, 0, 0, 0};
#pragma unroll
        for (int d = 0; d < MAXB; d++) {
          if (d >= beta) break;
          const u64 Dv = e ? D[d].y : D[d].x, ka = e ? KA[d].y : KA[d].x, kb = e ? KB[d].y : KB[d].x;
          const uint32_t dl = (uint32_t)(Dv & kMask30), dh = (uint32_t)(Dv >> 30);
          acc4_mac(A0, dl, dh, (uint32_t)kb, (uint32_t)(kb >> 32));
          acc4_mac(A1, dl, dh, (uint32_t)ka, (uint32_t)(ka >> 32));
        }
        acc4_fold(A0, h0, l0);
        acc4_fold(A1, h1, l1);
      }
      v0[e] = csub(reduce128_lazy8(h0, l0, P), p4);
      v1[e] = csub(reduce128_lazy8(h1, l1, P), p4);
    }
    *reinterpret_cast<ulonglong2*>(J.inner + (size_t)j * N + n) = make_ulonglong2(v0[0], v0[1]);
    *reinterpret_cast<ulonglong2*>(J.inner + ((size_t)ext + j) * N + n) = make_ulonglong2(v1[0], v1[1]);
  }
}

// Keys in the form the inner product reads: residue k (< 2^60) stored as (k mod 2^30) | (floor(k / 2^30) << 32).
__global__ void __launch_bounds__(kT) key_split_kernel(u64* __restrict__ k, size_t n) {
  for (size_t i = (size_t)blockIdx.x * kT + threadIdx.x; i < n; i += (size_t)gridDim.x * kT) {
    const u64 v = k[i];
    k[i] = (v & kMask30) | ((v >> 30) << 32);
  }
}

// ModDown basis conversion P -> Q_t: grid (N/512 (N/256 for more than 16 special primes), polys per job), two
// adjacent coefficients per thread (one above 16 special primes); reads the (coefficient-form) P rows of inner.
// Up to 11 special primes the instance is held to 80 registers, three CTAs per SM (ten primes: 90 -> 80 registers
// with 4 bytes of spills; the 64-rotation step 7,670 -> 7,687 ops/s).
template <int K>
__global__ void __launch_bounds__(kT, K <= 11 ? 3 : 1) moddown_conv_kernel(const __grid_constant__ KsBatch b, Ring r, CrtTables c,
                                                          const PrimeConst* __restrict__ pc) {
  pdl_prologue();
  extern __shared__ uint2 cs[];  // [K][t]
  const int z = find_job(b.row_begin, b.njobs, (int)blockIdx.y);
  const KsJob& J = b.jobs[z];
  const int t = J.t, ext = t + K;
  for (int idx = threadIdx.x; idx < K * t; idx += kT) {
    const int kk = idx / t, j = idx - kk * t;
    const uint32_t* src = c.md_phat + ((size_t)kk * c.nq + j) * 2;
    cs[idx] = make_uint2(src[0], src[1]);
  }
  __syncthreads();
  const int poly = (int)blockIdx.y - b.row_begin[z];
  constexpr int NC = K <= 16 ? 2 : 1;
  const int n = (blockIdx.x * kT + threadIdx.x) * NC;
  const u64* x = J.inner + ((size_t)poly * ext + t) * r.N + n;
  uint32_t yl[NC][K], yh[NC][K];
#pragma unroll
  for (int i = 0; i < K; i++) {
    uint32_t lo[NC], hi[NC];
    load_split<NC>(x + (size_t)i * r.N, c.md_phinv[i], pc[c.nq + i].p, lo, hi);
#pragma unroll
    for (int k = 0; k < NC; k++) {
      yl[k][i] = lo[k];
      yh[k][i] = hi[k];
    }
  }
  conv_rows<K, NC>(yl, yh, cs, t, J.md + (size_t)poly * t * r.N + n, (size_t)r.N, pc, [](int j) { return j; });
}

// out = automorph((inner_Q - NTT(conv)) * P^-1 + add): grid (N/512, rows); inner_Q and NTT(conv) arrive in [0, 4p)
// (both left lazy by their producers), so x + 4p - y is in (0, 8p) and the Shoup product by P^-1 reduces it.
__global__ void __launch_bounds__(kT) moddown_epilogue_kernel(const __grid_constant__ KsBatch b, Ring r,
                                                              CrtTables c, const PrimeConst* __restrict__ pc) {
  pdl_prologue();
  const int z = find_job(b.row_begin, b.njobs, (int)blockIdx.y);
  const KsJob& J = b.jobs[z];
  const int t = J.t, row = (int)blockIdx.y - b.row_begin[z];
  const int poly = row >= t ? 1 : 0, j = row - poly * t;
  const int n = (blockIdx.x * kT + threadIdx.x) * 2;  // two coefficients per thread, 16-byte loads
  const size_t N = r.N;
  const u64 q = pc[j].p;
  const ulonglong2 w = c.md_pinv[j];
  const ulonglong2 x = *reinterpret_cast<const ulonglong2*>(J.inner + ((size_t)poly * (t + c.np) + j) * N + n);
  const ulonglong2 y = *reinterpret_cast<const ulonglong2*>(J.md + ((size_t)poly * t + j) * N + n);
  const u64 q4 = 4 * q;
  const u64* add = poly == 0 ? J.add0 : J.add1;
  const ulonglong2 a = add ? *reinterpret_cast<const ulonglong2*>(add + (size_t)j * N + n) : make_ulonglong2(0, 0);
  u64* out = J.out + ((size_t)poly * t + j) * N;
#pragma unroll
  for (int e = 0; e < 2; e++) {
    u64 v = shoup((e ? x.y : x.x) + q4 - (e ? y.y : y.x), w.x, w.y, q);
    if (add) v = add_mod(v, e ? a.y : a.x, q);
    uint32_t pos = n + e;
    if (J.galois_inv != 1) {
      const uint32_t idx = brev_n(n + e, r.logN);
      const uint32_t jj = (uint32_t)((((2ull * idx + 1) * J.galois_inv) & (2ull * N - 1)) >> 1);
      pos = brev_n(jj, r.logN);
    }
    out[pos] = v;
  }
}

// Extended-basis key-switch output (double hoisting, no ModDown): rows 2 (t + np) per job over Q_t ∪ P,
// out[p][j] = automorph(inner[p][j] + a_p[j]) with a_0 = P * add0 on the Q rows (ext_mode 1) or add0 in the
// extended layout (ext_mode 2), a_1 = P * add1 on the Q rows (ext_mode 1); inner may be null (zero), which lifts
// a Q-basis ciphertext into the extended basis.
__global__ void __launch_bounds__(kT) ext_epilogue_kernel(const __grid_constant__ KsBatch b, Ring r, CrtTables c,
                                                          const PrimeConst* __restrict__ pc) {
  pdl_prologue();
  const int z = find_job(b.row_begin, b.njobs, (int)blockIdx.y);
  const KsJob& J = b.jobs[z];
  const int t = J.t, ext = t + c.np, row = (int)blockIdx.y - b.row_begin[z];
  const int poly = row >= ext ? 1 : 0, j = row - poly * ext;
  const int tower = j < t ? j : c.nq + (j - t);
  const u64 q = pc[tower].p;
  const int n = (blockIdx.x * kT + threadIdx.x) * 2;
  const size_t N = r.N;
  ulonglong2 v = J.inner ? *reinterpret_cast<const ulonglong2*>(J.inner + ((size_t)poly * ext + j) * N + n)
                         : make_ulonglong2(0, 0);
  v = make_ulonglong2(csub(csub(v.x, 2 * q), q), csub(csub(v.y, 2 * q), q));  // inner products are in [0, 4p)
  const u64* add = poly == 0 ? J.add0 : J.add1;
  if (add && J.ext_mode == 2) {
    const ulonglong2 a = *reinterpret_cast<const ulonglong2*>(add + (size_t)j * N + n);
    v = make_ulonglong2(add_mod(v.x, a.x, q), add_mod(v.y, a.y, q));
  } else if (add && j < t) {
    const ulonglong2 a = *reinterpret_cast<const ulonglong2*>(add + (size_t)j * N + n);
    const ulonglong2 w = c.md_pmodq[j];
    v = make_ulonglong2(add_mod(v.x, shoup(a.x, w.x, w.y, q), q), add_mod(v.y, shoup(a.y, w.x, w.y, q), q));
  }
  u64* out = J.out + ((size_t)poly * ext + j) * N;
#pragma unroll
  for (int e = 0; e < 2; e++) {
    uint32_t pos = n + e;
    if (J.galois_inv != 1) {
      const uint32_t idx = brev_n(n + e, r.logN);
      const uint32_t jj = (uint32_t)((((2ull * idx + 1) * J.galois_inv) & (2ull * N - 1)) >> 1);
      pos = brev_n(jj, r.logN);
    }
    out[pos] = e ? v.y : v.x;
  }
}

// Element-wise kernels move two coefficients per thread (16-byte accesses); grid.x = N / (2 kT).
__device__ __forceinline__ ulonglong2 ld2(const u64* p) { return *reinterpret_cast<const ulonglong2*>(p); }
__device__ __forceinline__ void st2(u64* p, ulonglong2 v) { *reinterpret_cast<ulonglong2*>(p) = v; }

__global__ void __launch_bounds__(kT) tensor_kernel(const __grid_constant__ TensorBatch b, Ring r,
                                                    const PrimeConst* __restrict__ pc) {
  pdl_prologue();
  const int z = find_job(b.row_begin, b.njobs, (int)blockIdx.y);
  const TensorJob& J = b.jobs[z];
  const int j = (int)blockIdx.y - b.row_begin[z];
  const size_t o = (size_t)j * r.N + ((size_t)blockIdx.x * kT + threadIdx.x) * 2;
  const size_t P = (size_t)J.t * r.N;
  const PrimeConst& c = pc[j];
  const ulonglong2 x0 = ld2(J.x + o), x1 = ld2(J.x + P + o), y0 = ld2(J.y + o), y1 = ld2(J.y + P + o);
  st2(J.d + o, make_ulonglong2(mul_mod(x0.x, y0.x, c), mul_mod(x0.y, y0.y, c)));
  st2(J.d + P + o, make_ulonglong2(add_mod(mul_mod(x0.x, y1.x, c), mul_mod(x1.x, y0.x, c), c.p),
                                   add_mod(mul_mod(x0.y, y1.y, c), mul_mod(x1.y, y0.y, c), c.p)));
  st2(J.d + 2 * P + o, make_ulonglong2(mul_mod(x1.x, y1.x, c), mul_mod(x1.y, y1.y, c)));
}

__global__ void __launch_bounds__(kT) addsub_kernel(const __grid_constant__ AddBatch b, Ring r,
                                                    const PrimeConst* __restrict__ pc) {
  pdl_prologue();
  const int z = find_job(b.row_begin, b.njobs, (int)blockIdx.y);
  const AddJob& J = b.jobs[z];
  const int j = (int)blockIdx.y - b.row_begin[z];
  const u64 p = pc[j].p;
  const size_t n = ((size_t)blockIdx.x * kT + threadIdx.x) * 2;
#pragma unroll
  for (int poly = 0; poly < 2; poly++) {
    const size_t o = ((size_t)poly * J.t + j) * r.N + n;
    const ulonglong2 x = ld2(J.x + o), y = ld2(J.y + o);
    st2(J.out + o, J.sub ? make_ulonglong2(sub_mod(x.x, y.x, p), sub_mod(x.y, y.y, p))
                         : make_ulonglong2(add_mod(x.x, y.x, p), add_mod(x.y, y.y, p)));
  }
}

// OpenFHE NativeVector::SwitchModulus: values above om/2 are lifted to v - om before reduction mod nm.
__global__ void __launch_bounds__(kT) ptop_kernel(const __grid_constant__ PtBatch b, Ring r,
                                                  const PrimeConst* __restrict__ pc) {
  pdl_prologue();
  const int z = find_job(b.row_begin, b.njobs, (int)blockIdx.y);
  const PtJob& J = b.jobs[z];
  const int j = (int)blockIdx.y - b.row_begin[z];
  const size_t n = ((size_t)blockIdx.x * kT + threadIdx.x) * 2;
  const size_t o0 = (size_t)j * r.N + n, o1 = ((size_t)J.t + j) * r.N + n;
  const PrimeConst& c = pc[j];
  const ulonglong2 w = ld2(J.pt + (size_t)j * r.N + n);
  const ulonglong2 x0 = ld2(J.ct + o0), x1 = ld2(J.ct + o1);
  if (J.mode == 0) {
    st2(J.out + o0, make_ulonglong2(mul_mod(x0.x, w.x, c), mul_mod(x0.y, w.y, c)));
    st2(J.out + o1, make_ulonglong2(mul_mod(x1.x, w.x, c), mul_mod(x1.y, w.y, c)));
  } else {
    st2(J.out + o0, J.mode == 1 ? make_ulonglong2(add_mod(x0.x, w.x, c.p), add_mod(x0.y, w.y, c.p))
                                : make_ulonglong2(sub_mod(x0.x, w.x, c.p), sub_mod(x0.y, w.y, c.p)));
    st2(J.out + o1, x1);
  }
}

__global__ void __launch_bounds__(kT) scalar_kernel(const __grid_constant__ ScalarBatch b, Ring r,
                                                    const PrimeConst* __restrict__ pc) {
  pdl_prologue();
  const int z = find_job(b.row_begin, b.njobs, (int)blockIdx.y);
  const ScalarJob& J = b.jobs[z];
  const ScalarSet& S = b.sets[J.set];
  const int j = (int)blockIdx.y - b.row_begin[z];
  const size_t n = ((size_t)blockIdx.x * kT + threadIdx.x) * 2;
  const u64 q = pc[j].p, w = S.mul[j], wsh = S.mul_sh[j], a = S.add[j];
  const size_t o0 = (size_t)j * r.N + n, o1 = ((size_t)J.t + j) * r.N + n;
  const ulonglong2 x0 = ld2(J.ct + o0), x1 = ld2(J.ct + o1);
  st2(J.out + o0, make_ulonglong2(add_mod(shoup(x0.x, w, wsh, q), a, q), add_mod(shoup(x0.y, w, wsh, q), a, q)));
  st2(J.out + o1, make_ulonglong2(shoup(x1.x, w, wsh, q), shoup(x1.y, w, wsh, q)));
}

// grid (N/512, 2 t per job): two coefficients of one row per thread; every term's values are loaded before the
// products, each product reduced (Shoup) and summed mod q.
__global__ void __launch_bounds__(kT) wsum_kernel(const __grid_constant__ WsumBatch b, Ring r,
                                                  const PrimeConst* __restrict__ pc) {
  pdl_prologue();
  const int z = find_job(b.row_begin, b.njobs, (int)blockIdx.y);
  const WsumJob& J = b.jobs[z];
  const int row = (int)blockIdx.y - b.row_begin[z];
  const int poly = row >= J.t ? 1 : 0, j = row - poly * J.t;
  const size_t n = ((size_t)blockIdx.x * kT + threadIdx.x) * 2;
  const u64 q = pc[j].p;
  ulonglong2 x[kMaxWsumTerms];
#pragma unroll
  for (int k = 0; k < kMaxWsumTerms; k++)
    if (k < b.nterms) x[k] = ld2(J.term[k] + ((size_t)poly * J.term_t[k] + j) * r.N + n);
  u64* o = J.out + ((size_t)poly * J.t + j) * r.N + n;
  ulonglong2 acc = b.accumulate ? ld2(o) : make_ulonglong2(0, 0);
#pragma unroll
  for (int k = 0; k < kMaxWsumTerms; k++)
    if (k < b.nterms) {
      const u64 w = b.set.mul[k][j], wsh = b.set.mul_sh[k][j];
      acc.x = add_mod(acc.x, shoup(x[k].x, w, wsh, q), q);
      acc.y = add_mod(acc.y, shoup(x[k].y, w, wsh, q), q);
    }
  st2(o, acc);
}

// grid rows per job: 2*t (poly-major).  X^k at point psi^(2 brev(i) + 1) is psi^e, e = (2 brev(i) + 1) k mod 2N;
// psi^e = tw[brev(e)] for e < N and -tw[brev(e - N)] otherwise (psi^N = -1).
__global__ void __launch_bounds__(kT) monomial_kernel(const __grid_constant__ MonoBatch b, Ring r,
                                                      const PrimeConst* __restrict__ pc,
                                                      const ulonglong2* __restrict__ tw) {
  pdl_prologue();
  const int z = find_job(b.row_begin, b.njobs, (int)blockIdx.y);
  const MonoJob& J = b.jobs[z];
  const int row = (int)blockIdx.y - b.row_begin[z];
  const int j = row >= J.t ? row - J.t : row;
  const uint32_t i = blockIdx.x * kT + threadIdx.x;
  const uint32_t two_n_mask = 2u * r.N - 1;
  const uint32_t e = (uint32_t)(((2ull * brev_n(i, r.logN) + 1) * J.k) & two_n_mask);
  const uint32_t eh = e & (r.N - 1);
  const ulonglong2 w = tw[(size_t)j * r.N + brev_n(eh, r.logN)];
  const u64 q = pc[j].p;
  const size_t o = (size_t)row * r.N + i;
  u64 v = shoup(J.ct[o], w.x, w.y, q);
  if (e >= (uint32_t)r.N && v) v = q - v;
  J.out[o] = v;
}

// Inner sums: grid (N/256, (t+np) njobs), ordered (row, job) with the job fastest, so that the blocks reading the
// same plaintext rows (every input of a batch) run back to back and share them through L2.  A thread takes one
// coefficient of both polys for up to kDotG giant steps, in rounds of four baby steps: each round's baby-step
// values (both polys) and plaintext values (24 words) are copied to shared memory with cp.async (zero-filled where
// a diagonal is absent) one round ahead of the products, so two rounds of loads are in flight per thread without
// holding them in registers, and each plaintext value is read once for both polys.  Each thread only reads back
// the words it copied itself, so completion (cp.async.wait_group) needs no block barrier.  One Acc4 per (giant
// step, poly) holds at most 16 products (bs <= 16), folded and reduced once at the end.
constexpr int kDotWords = 8 + 4 * kDotG;  // per thread and round: 4 x 2 baby-step values, 4 x kDotG plaintexts

__device__ __forceinline__ void cp_async8(u64* dst, const u64* src, bool on) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(src), "r"(on ? 8 : 0) : "memory");
}

__global__ void __launch_bounds__(kT) ptdot_kernel(const __grid_constant__ DotBatch b, Ring r,
                                                   const PrimeConst* __restrict__ pc) {
  pdl_prologue();
  extern __shared__ __align__(16) u64 stage[];  // [2 rounds][kDotWords][kT]
  const int y = (int)blockIdx.y, job = y % b.njobs, j = y / b.njobs;
  const DotJob& J = b.jobs[job];
  const int t = b.t, rows = t + b.np;
  const int tower = j < t ? j : b.nq + (j - t), prow = j < t ? j : b.pt_prow + (j - t);
  const int tid = threadIdx.x;
  const size_t n = (size_t)blockIdx.x * kT + tid;
  const size_t c0 = (size_t)j * r.N + n, c1 = ((size_t)rows + j) * r.N + n, po = (size_t)prow * r.N + n;
  const unsigned long long pm = J.pmask;
  const int rounds = (b.bs + 3) / 4;
  auto issue = [&](int round) {
    u64* buf = stage + (size_t)(round & 1) * kDotWords * kT + tid;
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const int bb = round * 4 + u;
      bool any = false;
#pragma unroll
      for (int g = 0; g < kDotG; g++) {
        const bool on = bb < b.bs && ((pm >> (g * 16 + (bb & 15))) & 1ull);
        any = any || on;
        const u64* src = on ? b.pt_base + (size_t)((J.g + g) * b.bs + bb) * b.pt_stride + po : b.pt_base;
        cp_async8(buf + (8 + u * kDotG + g) * kT, src, on);
      }
      const u64* ct = !any ? J.rot0 : bb == 0 ? J.rot0 : J.rot_base + (size_t)(bb - 1) * b.rot_stride;
      cp_async8(buf + (2 * u) * kT, any ? ct + c0 : ct, any);
      cp_async8(buf + (2 * u + 1) * kT, any ? ct + c1 : ct, any);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  };
  Acc4 A[kDotG][2];
#pragma unroll
  for (int g = 0; g < kDotG; g++) A[g][0] = A[g][1] = Acc4{0, 0, 0, 0};
  issue(0);
#pragma unroll 1
  for (int round = 0; round < rounds; round++) {
    if (round + 1 < rounds) {
      issue(round + 1);
      asm volatile("cp.async.wait_group 1;" ::: "memory");
    } else {
      asm volatile("cp.async.wait_group 0;" ::: "memory");
    }
    const u64* buf = stage + (size_t)(round & 1) * kDotWords * kT + tid;
#pragma unroll
    for (int u = 0; u < 4; u++) {
      const u64 x0 = buf[(2 * u) * kT], x1 = buf[(2 * u + 1) * kT];
      const uint32_t l0 = (uint32_t)(x0 & kMask30), h0 = (uint32_t)(x0 >> 30);
      const uint32_t l1 = (uint32_t)(x1 & kMask30), h1 = (uint32_t)(x1 >> 30);
#pragma unroll
      for (int g = 0; g < kDotG; g++) {
        const u64 w = buf[(8 + u * kDotG + g) * kT];
        const uint32_t wl = (uint32_t)(w & kMask30), wh = (uint32_t)(w >> 30);
        acc4_mac(A[g][0], l0, h0, wl, wh);
        acc4_mac(A[g][1], l1, h1, wl, wh);
      }
    }
  }
  const PrimeConst& P = pc[tower];
#pragma unroll
  for (int g = 0; g < kDotG; g++) {
    if (g >= J.ng) break;
    u64 hi = 0, lo = 0;
    acc4_fold(A[g][0], hi, lo);
    J.out[(size_t)g * b.out_stride + c0] = reduce128_fast(hi, lo, P);
    hi = lo = 0;
    acc4_fold(A[g][1], hi, lo);
    J.out[(size_t)g * b.out_stride + c1] = reduce128_fast(hi, lo, P);
  }
}

__global__ void __launch_bounds__(kT) sum_kernel(const __grid_constant__ SumBatch b, Ring r,
                                                 const PrimeConst* __restrict__ pc) {
  pdl_prologue();
  const int z = find_job(b.row_begin, b.njobs, (int)blockIdx.y);
  const SumJob& J = b.jobs[z];
  const int row = (int)blockIdx.y - b.row_begin[z];
  const int t = J.t, rows = t + J.np, poly = row >= rows ? 1 : 0, j = row - poly * rows;
  const size_t o = ((size_t)poly * rows + j) * r.N + (size_t)blockIdx.x * kT + threadIdx.x;
  const u64 q = pc[j < t ? j : b.nq + (j - t)].p;
  u64 acc = J.first ? J.first[o] : 0;
#pragma unroll 4
  for (int k = 0; k < J.n; k++) acc = add_mod(acc, J.base[(size_t)k * J.stride + o], q);
  J.out[o] = acc;
}

// Centred lift of tower 0 into towers 0..T-1 (OpenFHE SwitchModulus semantics, as in Rescale).
__global__ void __launch_bounds__(kT) raise_switch_kernel(const __grid_constant__ RaiseBatch b, Ring r,
                                                          const PrimeConst* __restrict__ pc) {
  pdl_prologue();
  const int z = find_job(b.row_begin, b.njobs, (int)blockIdx.y);
  const RaiseJob& J = b.jobs[z];
  const int row = (int)blockIdx.y - b.row_begin[z];
  const int poly = row >= J.T ? 1 : 0, i = row - poly * J.T;
  const int n = blockIdx.x * kT + threadIdx.x;
  const PrimeConst& om = pc[0];
  const PrimeConst& nm = pc[i];
  const u64 om_mod_nm = shoup(om.p, 1ull, nm.one_sh, nm.p);
  const u64 diff = nm.p - om_mod_nm;
  u64 v = J.top[(size_t)poly * r.N + n];
  if (v > (om.p >> 1)) v += diff;
  J.tmp[((size_t)poly * J.T + i) * r.N + n] = shoup(v, 1ull, nm.one_sh, nm.p);
}

template <class B>
int max_t(const B& b) {
  int m = 0;
  for (int i = 0; i < b.njobs; i++) m = b.jobs[i].t > m ? b.jobs[i].t : m;
  return m;
}

// Copy of a batch with row_begin filled for `rows(job)` rows per job; returns the total row count.
template <class B, class F>
int with_rows(const B& in, B& out, F rows) {
  out = in;
  out.row_begin[0] = 0;
  for (int i = 0; i < in.njobs; i++) out.row_begin[i + 1] = out.row_begin[i] + rows(in.jobs[i]);
  return out.row_begin[in.njobs];
}

}  // namespace

cudaError_t launch_modup_conv(const KsBatch& b, const Ring& r, const CrtTables& c, const PrimeConst* pc,
                              cudaStream_t s) {
  if (b.njobs <= 0) return cudaSuccess;
  if (c.alpha > 16 && c.alpha != 20 && c.alpha != 24 && c.alpha != 28 && c.alpha != 32) return cudaErrorInvalidValue;
  for (int i = 0; i < b.njobs; i++) {  // partial last digits must have a compiled size
    const int tt = b.jobs[i].t, last = tt - ((tt - 1) / c.alpha) * c.alpha;
    if (last > 16 && last != 20 && last != 24 && last != 28 && last != 32) return cudaErrorInvalidValue;
  }
  const int mt = max_t(b);
  const size_t smem = sizeof(uint2) * c.alpha * (mt + c.np);
  KsBatch bb;
  const int alpha = c.alpha;
  const int rows = with_rows(b, bb, [alpha](const KsJob& j) { return (j.t + alpha - 1) / alpha; });
  dim3 grid(r.N / (c.alpha <= 16 ? 2 * kT : kT), rows, 1);
  if (c.alpha <= 8)
    launch_pdl(modup_conv_kernel<8>, grid, dim3(kT), smem, s, bb, r, c, pc);
  else if (c.alpha <= 10)
    launch_pdl(modup_conv_kernel<10>, grid, dim3(kT), smem, s, bb, r, c, pc);
  else if (c.alpha <= 12)
    launch_pdl(modup_conv_kernel<12>, grid, dim3(kT), smem, s, bb, r, c, pc);
  else if (c.alpha <= 16)
    launch_pdl(modup_conv_kernel<16>, grid, dim3(kT), smem, s, bb, r, c, pc);
  else
    launch_pdl(modup_conv_kernel<32>, grid, dim3(kT), smem, s, bb, r, c, pc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_ks_inner(const KsBatch& b, const Ring& r, const CrtTables& c, const PrimeConst* pc,
                            cudaStream_t s) {
  if (b.njobs <= 0) return cudaSuccess;
  // jobs reordered so that those with the same key are adjacent (first-appearance order of the keys)
  KsBatch bb = b;
  bool used[kMaxJobs] = {};
  int k = 0, rows = 0;
  bb.ngroups = 0;
  bb.row_begin[0] = 0;
  for (int i = 0; i < b.njobs; i++) {
    if (used[i]) continue;
    bb.grp_begin[bb.ngroups] = k;
    int tmax = 0;
    for (int q = i; q < b.njobs; q++)
      if (!used[q] && b.jobs[q].key == b.jobs[i].key) {
        used[q] = true;
        bb.jobs[k++] = b.jobs[q];
        tmax = std::max(tmax, b.jobs[q].t);
      }
    rows += (tmax + c.np) * (k - bb.grp_begin[bb.ngroups]);
    bb.row_begin[++bb.ngroups] = rows;
  }
  bb.grp_begin[bb.ngroups] = k;
  // Jobs of different key groups that read the same digits (the rotations of one hoisted ModUp: baby steps of a
  // linear transform, RotateHoisted) would re-read those digits once per group when the groups run one after the
  // other.  Then the blocks are ordered by tower row first, so every job's blocks of one row run together and the
  // row's digits and key values are read from HBM about once, the other reads hitting L2.
  bb.row_outer = 0;
  for (int i = 0; i < bb.ngroups && !bb.row_outer; i++)
    for (int x = bb.grp_begin[i]; x < bb.grp_begin[i + 1] && !bb.row_outer; x++)
      for (int y = bb.grp_begin[i + 1]; y < k; y++)
        if (bb.jobs[x].a == bb.jobs[y].a && bb.jobs[x].conv == bb.jobs[y].conv) {
          bb.row_outer = 1;
          break;
        }
  if (bb.row_outer) {
    int tmax = 0;
    for (int i = 0; i < k; i++) tmax = std::max(tmax, bb.jobs[i].t);
    rows = (tmax + c.np) * k;
  }
  const int iters = std::min(c.ks_iters > 0 ? c.ks_iters : 4, r.N / (2 * kT));  // N / 512 is a power of two >= 2
  dim3 grid(r.N / (2 * kT * iters), rows, 1);
  switch (c.dnum) {  // beta <= dnum: size the register arrays exactly (fewer registers, more resident warps)
#define FGB_KSI_CASE(B_)                                          \
  case B_:                                                        \
    launch_pdl(ks_inner_kernel<B_>, grid, dim3(kT), 0, s, bb, r, c, pc, iters); \
    break;
    FGB_KSI_CASE(1) FGB_KSI_CASE(2) FGB_KSI_CASE(3) FGB_KSI_CASE(4) FGB_KSI_CASE(5) FGB_KSI_CASE(6)
    FGB_KSI_CASE(7) FGB_KSI_CASE(8)
#undef FGB_KSI_CASE
    default:
      return cudaErrorInvalidValue;
  }
  count_launch();
  return cudaGetLastError();
}

// Input validation (opt-in, fides_ctx_set_input_check): sets *bad when a residue is not below its prime.  Row r of
// x holds tower j = r % period, whose prime is j for j < tq and nq + (j - tq) past it (the special rows of an
// extended layout).
__global__ void range_check_kernel(const u64* __restrict__ x, long long rows, int logN, int period, int tq, int nq,
                                   const PrimeConst* __restrict__ pc, int* bad) {
  const long long n = rows << logN;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int j = (int)((i >> logN) % period);
    if (x[i] >= pc[j < tq ? j : nq + (j - tq)].p) {
      *bad = 1;
      return;
    }
  }
}

cudaError_t launch_range_check(const u64* x, long long rows, int logN, int period, int tq, int nq,
                               const PrimeConst* pc, int* bad, cudaStream_t s) {
  if (rows <= 0) return cudaSuccess;
  range_check_kernel<<<1024, kT, 0, s>>>(x, rows, logN, period, tq, nq, pc, bad);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_key_split(u64* key, size_t n, cudaStream_t s) {
  key_split_kernel<<<1024, kT, 0, s>>>(key, n);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_moddown_conv(const KsBatch& b, const Ring& r, const CrtTables& c, const PrimeConst* pc,
                                cudaStream_t s) {
  if (b.njobs <= 0) return cudaSuccess;
  const size_t smem = sizeof(uint2) * c.np * max_t(b);
  KsBatch bb;
  const int rows = with_rows(b, bb, [](const KsJob& j) { return j.polys ? j.polys : 2; });
  dim3 grid(r.N / (c.np <= 16 ? 2 * kT : kT), rows, 1);
  switch (c.np) {
#define FGB_MD_CASE(K_)                                                    \
  case K_:                                                                 \
    launch_pdl(moddown_conv_kernel<K_>, grid, dim3(kT), smem, s, bb, r, c, pc);          \
    break;
    FGB_MD_CASE(1) FGB_MD_CASE(2) FGB_MD_CASE(3) FGB_MD_CASE(4) FGB_MD_CASE(5) FGB_MD_CASE(6) FGB_MD_CASE(7)
    FGB_MD_CASE(8) FGB_MD_CASE(9) FGB_MD_CASE(10) FGB_MD_CASE(11) FGB_MD_CASE(12) FGB_MD_CASE(13)
    FGB_MD_CASE(14) FGB_MD_CASE(15) FGB_MD_CASE(16) FGB_MD_CASE(20) FGB_MD_CASE(24) FGB_MD_CASE(32)
#undef FGB_MD_CASE
    default:
      return cudaErrorInvalidValue;
  }
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_moddown_epilogue(const KsBatch& b, const Ring& r, const CrtTables& c, const PrimeConst* pc,
                                    cudaStream_t s) {
  if (b.njobs <= 0) return cudaSuccess;
  KsBatch bb;
  const int rows = with_rows(b, bb, [](const KsJob& j) { return (j.polys ? j.polys : 2) * j.t; });
  dim3 grid(r.N / (2 * kT), rows, 1);
  launch_pdl(moddown_epilogue_kernel, grid, dim3(kT), 0, s, bb, r, c, pc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_ext_epilogue(const KsBatch& b, const Ring& r, const CrtTables& c, const PrimeConst* pc,
                                cudaStream_t s) {
  if (b.njobs <= 0) return cudaSuccess;
  KsBatch bb;
  const int np = c.np;
  const int rows = with_rows(b, bb, [np](const KsJob& j) { return 2 * (j.t + np); });
  dim3 grid(r.N / (2 * kT), rows, 1);
  launch_pdl(ext_epilogue_kernel, grid, dim3(kT), 0, s, bb, r, c, pc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_tensor(const TensorBatch& b, const Ring& r, int nq, const PrimeConst* pc, cudaStream_t s) {
  if (b.njobs <= 0) return cudaSuccess;
  TensorBatch bb;
  const int rows = with_rows(b, bb, [](const TensorJob& j) { return j.t; });
  dim3 grid(r.N / (2 * kT), rows, 1);
  launch_pdl(tensor_kernel, grid, dim3(kT), 0, s, bb, r, pc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_addsub(const AddBatch& b, const Ring& r, int nq, const PrimeConst* pc, cudaStream_t s) {
  if (b.njobs <= 0) return cudaSuccess;
  AddBatch bb;
  const int rows = with_rows(b, bb, [](const AddJob& j) { return j.t; });
  dim3 grid(r.N / (2 * kT), rows, 1);
  launch_pdl(addsub_kernel, grid, dim3(kT), 0, s, bb, r, pc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_ptop(const PtBatch& b, const Ring& r, const PrimeConst* pc, cudaStream_t s) {
  if (b.njobs <= 0) return cudaSuccess;
  PtBatch bb;
  const int rows = with_rows(b, bb, [](const PtJob& j) { return j.t; });
  launch_pdl(ptop_kernel, dim3(r.N / (2 * kT), rows, 1), dim3(kT), 0, s, bb, r, pc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_scalar(const ScalarBatch& b, const Ring& r, const PrimeConst* pc, cudaStream_t s) {
  if (b.njobs <= 0) return cudaSuccess;
  ScalarBatch bb;
  const int rows = with_rows(b, bb, [](const ScalarJob& j) { return j.t; });
  launch_pdl(scalar_kernel, dim3(r.N / (2 * kT), rows, 1), dim3(kT), 0, s, bb, r, pc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_wsum(const WsumBatch& b, const Ring& r, const PrimeConst* pc, cudaStream_t s) {
  if (b.njobs <= 0) return cudaSuccess;
  if (b.nterms < 1 || b.nterms > kMaxWsumTerms) return cudaErrorInvalidValue;
  WsumBatch bb;
  const int rows = with_rows(b, bb, [](const WsumJob& j) { return 2 * j.t; });
  launch_pdl(wsum_kernel, dim3(r.N / (2 * kT), rows, 1), dim3(kT), 0, s, bb, r, pc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_monomial(const MonoBatch& b, const Ring& r, const PrimeConst* pc, const ulonglong2* tw_fwd,
                            cudaStream_t s) {
  if (b.njobs <= 0) return cudaSuccess;
  MonoBatch bb;
  const int rows = with_rows(b, bb, [](const MonoJob& j) { return 2 * j.t; });
  launch_pdl(monomial_kernel, dim3(r.N / kT, rows, 1), dim3(kT), 0, s, bb, r, pc, tw_fwd);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_ptdot(const DotBatch& b, const Ring& r, const PrimeConst* pc, cudaStream_t s) {
  if (b.njobs <= 0) return cudaSuccess;
  if (b.bs > 16) return cudaErrorInvalidValue;
  DotBatch bb = b;
  for (int i = 0; i < b.njobs; i++) {
    DotJob& J = bb.jobs[i];
    if (J.ng < 1 || J.ng > kDotG) return cudaErrorInvalidValue;
    J.pmask = 0;
    for (int g = 0; g < J.ng; g++)
      for (int k = 0; k < b.bs; k++)
        if (b.present[(J.g + g) * b.bs + k]) J.pmask |= 1ull << (g * 16 + k);
  }
  const size_t smem = sizeof(u64) * 2 * kDotWords * kT;
  static std::atomic<unsigned long long> attr_done{0};
  const cudaError_t ea = once_per_device(attr_done, [&] {
    return cudaFuncSetAttribute(ptdot_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  });
  if (ea != cudaSuccess) return ea;
  launch_pdl(ptdot_kernel, dim3(r.N / kT, (b.t + b.np) * b.njobs, 1), dim3(kT), smem, s, bb, r, pc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_sum(const SumBatch& b, const Ring& r, const PrimeConst* pc, cudaStream_t s) {
  if (b.njobs <= 0) return cudaSuccess;
  SumBatch bb;
  const int rows = with_rows(b, bb, [](const SumJob& j) { return 2 * (j.t + j.np); });
  launch_pdl(sum_kernel, dim3(r.N / kT, rows, 1), dim3(kT), 0, s, bb, r, pc);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_raise_switch(const RaiseBatch& b, const Ring& r, const PrimeConst* pc, cudaStream_t s) {
  if (b.njobs <= 0) return cudaSuccess;
  RaiseBatch bb;
  const int rows = with_rows(b, bb, [](const RaiseJob& j) { return 2 * j.T; });
  launch_pdl(raise_switch_kernel, dim3(r.N / kT, rows, 1), dim3(kT), 0, s, bb, r, pc);
  count_launch();
  return cudaGetLastError();
}

}  // namespace fgb
