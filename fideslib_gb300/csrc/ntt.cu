// Batched 64-bit negacyclic NTT / INTT, one HBM read and one HBM write per limb.
//
// Reference counterpart: src/NTT.cu:331-769 (NTT_/INTT_, a two-kernel four-step transform with 10 KiB of
// shared memory per 128-thread CTA, i.e. two HBM round trips per limb).  Here one limb of N = 2^16 residues
// (512 KiB) is held by a thread-block cluster of C = N/8192 CTAs, 64 KiB of shared memory each:
//   forward (Cooley–Tukey, natural -> bit-reversed, twiddle table index m+i as in OpenFHE's
//   ForwardTransformToBitReverse, test/cpuNTT_nega.cpp:38-85):
//     phase X : the log2(C) stages that pair residues held by different CTAs.  CTA c loads the columns
//               l in [c*E/C, (c+1)*E/C) of all C blocks, runs a radix-C butterfly on them and writes each
//               result into the shared memory of the CTA that owns its block (distributed shared memory);
//     pass A  : stages on bits [LOGE-1 .. 8]   (32 residues per thread, stride 256),
//     pass B  : stages on bits [7 .. 4]        (16 residues per thread, stride 16),
//     pass C  : stages on bits [3 .. 0]        (16 contiguous residues), then the store to HBM.
//   inverse (Gentleman–Sande, bit-reversed -> natural, N^-1 applied on the way out) runs the passes in the
//   reverse order.
// For N = 2^13 .. 2^16 the forward transform uses a radix-16 variant of the same cluster layout (ntt16_fwd_kernel
// below: four radix-16 passes, 16 residues per thread, three CTAs per SM).
// Butterflies are Harvey-lazy with a cheaper quotient estimate (shoup_lazy4, products in [0, 4p)): forward
// values live in [0, 16p) (the compare-and-subtract on every other stage), inverse values below 16p with a
// compile-time bound per position (GsPlan); outputs are reduced to [0, p).  Needs p < 2^60.  Shared memory is
// XOR-swizzled on bits 1..3 (word l stored at l ^ (((l >> 4) & 7) << 1)): the passes that hold 16 residues at a
// stride (X, A, B) access 64-bit words of distinct banks in every half-warp, and the last pass, whose thread holds
// 16 contiguous residues, moves them as eight 16-byte pairs (the swizzle keeps pairs adjacent and aligned) with
// distinct banks in every quarter-warp.  Against a swizzle on bits 0..3 with 64-bit accesses in the last pass this
// took the 640-limb forward from 0.457 to 0.445 ms and the inverse from 0.543 to 0.534 ms.
#include <cooperative_groups.h>

#include <atomic>

#include "kernels.cuh"
#include "ntt.cuh"

namespace cg = cooperative_groups;

namespace fgb {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int swz(int l) { return l ^ (((l >> 4) & 7) << 1); }

// Distributed shared memory through 32-bit shared::cluster addresses: element `local` of this CTA's shared memory as
// it appears in the cluster window at CTA `rank` (one register per address instead of a 64-bit generic pointer, which
// keeps the cross-CTA phases of the radix-16 kernels free of register spills).
__device__ __forceinline__ uint32_t peer_smem(const u64* local, int rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"((uint32_t)__cvta_generic_to_shared(local)), "r"(rank));
  return r;
}
__device__ __forceinline__ u64 ld_peer(uint32_t addr) {
  u64 v;
  asm volatile("ld.shared::cluster.u64 %0, [%1];" : "=l"(v) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ void st_peer(uint32_t addr, u64 v) {
  asm volatile("st.shared::cluster.u64 [%0], %1;" ::"r"(addr), "l"(v) : "memory");
}

// Forward (CT): x + wY, x - wY + 4p with wY from shoup_lazy4 in [0, 4p).  Values stay below 16p (< 2^64 for
// p < 2^60): a stage with the correction maps X in [0, 16p) to x in [0, 8p) (X - 8p when X >= 8p) and outputs
// [0, 12p); a stage without it takes X in [0, 12p) and outputs [0, 16p).  Stages alternate (correction on even global
// stages), so half the butterflies skip the compare-and-subtract.
template <bool CORR>
__device__ __forceinline__ void ct_bfly(u64& X, u64& Y, const ulonglong2& w, u64 negp, u64 p4) {
  const u64 x = CORR ? (X >= 2 * p4 ? X - 2 * p4 : X) : X;
  const u64 t = shoup_lazy4(Y, w.x, w.y, negp);
  X = x + t;
  Y = x - t + p4;
}

// Inverse (GS): X, Y -> X + Y, (X - Y + b_Y p) w, where b_Y p bounds Y.  The product is in [0, 4p) whatever its
// input, so only the sums grow.  Every residue of a pass carries a bound b p (b a power of two) that its position
// fixes at compile time (GsPlan): a compare-and-subtract (b p -> b p / 2) is spent only where a sum could reach 16p
// (< 2^64 for p < 2^60) and where the pass hands its residues on (bound 8p between passes; the transform's input is
// below 4p).  That is about 0.53 compare-and-subtracts per butterfly instead of one.
template <int R>
struct GsPlan {
  unsigned char bx[R][1 << R], by[R][1 << R];  // bounds of X (at k) and Y (at k + 2^kb) before stage kb's butterfly
  unsigned char hx[R][1 << R], hy[R][1 << R];  // halvings applied to each before it
  unsigned char bend[1 << R], hend[1 << R];    // bound at the end of the pass and the halvings that meet ENDB
  bool ok;                                     // every halving count within gs_reduce's three
};

// FINAL: the pass ends the transform; its last stage is the N^-1-scaled one (both outputs are products, < 4p).
// lim: the largest sum allowed (16p; 8p keeps every offset and subtrahend at 4p, one 64-bit constant fewer for a
// pass whose registers are at the limit).
template <int R>
__host__ __device__ constexpr GsPlan<R> gs_plan(int b0, int endb, bool final_pass, int lim = 16) {
  GsPlan<R> P{};
  P.ok = true;
  int b[1 << R] = {};
  for (int k = 0; k < (1 << R); k++) b[k] = b0;
  for (int kb = 0; kb < R; kb++)
    for (int k = 0; k < (1 << R); k++) {
      if (k & (1 << kb)) continue;
      const int j = k + (1 << kb);
      P.bx[kb][k] = (unsigned char)b[k];
      P.by[kb][k] = (unsigned char)b[j];
      int hx = 0, hy = 0;
      while (b[k] + b[j] > lim) {
        if (b[k] >= b[j]) {
          b[k] /= 2;
          hx++;
        } else {
          b[j] /= 2;
          hy++;
        }
      }
      P.hx[kb][k] = (unsigned char)hx;
      P.hy[kb][k] = (unsigned char)hy;
      P.ok = P.ok && hx <= 3 && hy <= 3;
      b[k] = (final_pass && kb == R - 1) ? 4 : b[k] + b[j];
      b[j] = 4;
    }
  for (int k = 0; k < (1 << R); k++) {
    P.bend[k] = (unsigned char)b[k];
    int h = 0;
    while (endb > 0 && b[k] > endb) {
      b[k] /= 2;
      h++;
    }
    P.hend[k] = (unsigned char)h;
    P.ok = P.ok && h <= 3;
  }
  return P;
}

// v < b p -> the same residue below (b >> h) p, by h compare-and-subtracts (b, h compile-time after unrolling).
__device__ __forceinline__ u64 gs_reduce(u64 v, int b, int h, u64 p) {
#pragma unroll
  for (int i = 0; i < 3; i++)
    if (i < h) {
      b >>= 1;
      v = csub(v, p * (u64)b);
    }
  return v;
}

// The inverse's last stage (s = 0, one twiddle w1 = psi^-brev(1)) with N^-1 folded in: (X + Y) N^-1,
// (X - Y + b_Y p) w1 N^-1, both in [0, 4p).  Saves the separate scaling of every output by N^-1.
struct LastStage {
  u64 ninv, ninv_sh, w1ninv, w1ninv_sh;
};

// Butterfly of pair (k, k + 2^kb) at stage kb of a pass planned by P; last != null: the N^-1-scaled final stage.
template <int R>
__device__ __forceinline__ void gs_bfly(u64 (&x)[1 << R], const GsPlan<R>& P, int kb, int k, const ulonglong2& w,
                                        u64 p, u64 negp, const LastStage* last = nullptr) {
  const int j = k + (1 << kb);
  const u64 X = gs_reduce(x[k], P.bx[kb][k], P.hx[kb][k], p);
  const u64 Y = gs_reduce(x[j], P.by[kb][k], P.hy[kb][k], p);
  const u64 d = X - Y + p * (u64)(P.by[kb][k] >> P.hy[kb][k]);
  if (last) {
    x[k] = shoup_lazy4(X + Y, last->ninv, last->ninv_sh, negp);
    x[j] = shoup_lazy4(d, last->w1ninv, last->w1ninv_sh, negp);
  } else {
    x[k] = X + Y;
    x[j] = shoup_lazy4(d, w.x, w.y, negp);
  }
}

template <int R>
__device__ __forceinline__ void gs_end(u64 (&x)[1 << R], const GsPlan<R>& P, u64 p) {
#pragma unroll
  for (int k = 0; k < (1 << R); k++) x[k] = gs_reduce(x[k], P.bend[k], P.hend[k], p);
}

// Radix-2^LOGR stages over x[k] = a[G*2^(LOGS+LOGR) + k*2^LOGS + low] (low < 2^LOGS).  At the sub-stage on
// bit kb of k the pair distance is 2^(LOGS+kb), the global stage is s = LOGN-1-(LOGS+kb) and the twiddle of
// the pair whose lower member is k has table index 2^s + G*2^(LOGR-1-kb) + j, j = k >> (kb+1).  The last four
// stages (LOGS = 0, LOGR = 4: one 16-residue group per thread, consecutive groups in a warp) read the transposed
// copy of the table, index 2^s + j*(N/16) + G (DeviceTables), so a warp's loads are contiguous.
template <int LOGR, int LOGS, int LOGN>
__device__ __forceinline__ const ulonglong2* tw_entry(const ulonglong2* __restrict__ tw, int s, int kb, int G, int j) {
  if constexpr (LOGS == 0) {
    static_assert(LOGR == 4, "the transposed twiddle layout covers radix-16 groups");
    return tw + (1 << s) + j * (1 << (LOGN - 4)) + G;
  } else {
    return tw + (1 << s) + G * (1 << (LOGR - 1 - kb)) + j;
  }
}

template <int LOGR, int LOGS, int LOGN>
__device__ __forceinline__ void fwd_radix(u64 (&x)[1 << LOGR], int G, const ulonglong2* __restrict__ tw, u64 negp,
                                          u64 p4) {
#pragma unroll
  for (int kb = LOGR - 1; kb >= 0; kb--) {
    const int s = LOGN - 1 - (LOGS + kb);
#pragma unroll
    for (int k = 0; k < (1 << LOGR); k++) {
      if (k & (1 << kb)) continue;
      const ulonglong2 w = __ldg(tw_entry<LOGR, LOGS, LOGN>(tw, s, kb, G, k >> (kb + 1)));
      if ((s & 1) == 0)
        ct_bfly<true>(x[k], x[k + (1 << kb)], w, negp, p4);
      else
        ct_bfly<false>(x[k], x[k + (1 << kb)], w, negp, p4);
    }
  }
}

// Inverse stages of a pass (LOGS = 0: the transform's first pass, input below 4p; otherwise below 8p).  A pass whose
// stages reach s = 0 ends the transform and takes last (N^-1, LastStage); its outputs are below 4p, every other
// pass's below 8p.  LIM: gs_plan's lim.
template <int LOGR, int LOGS, int LOGN, int LIM = 16>
__device__ __forceinline__ void inv_radix(u64 (&x)[1 << LOGR], int G, const ulonglong2* __restrict__ tw, u64 negp,
                                          u64 p, const LastStage* last = nullptr) {
  constexpr bool kFinal = LOGS + LOGR == LOGN;
  constexpr GsPlan<LOGR> P = gs_plan<LOGR>(LOGS == 0 ? 4 : 8, kFinal ? 0 : 8, kFinal, LIM);
  static_assert(P.ok, "a residue needs more halvings than gs_reduce applies");
  if constexpr (LOGS == 0) {
    // The inverse's first pass (16 contiguous residues per thread, each thread's 15 twiddles its own and read from
    // L2): all 15 twiddle loads are issued before the first butterfly, so their latencies overlap instead of
    // adding up stage by stage (640-limb inverse 0.5325 -> 0.5192 ms; the same in the forward's last pass, whose
    // inputs come from shared memory, measured 0.4465 -> 0.4526 ms and is not done).  s >= LOGN - 4 > 0 here, so
    // the last-stage scaling never applies.
    static_assert(LOGR == 4 && !kFinal, "the first pass of the inverse works on 16-residue groups");
    ulonglong2 wv[15];  // stage kb's twiddles start at 16 - (16 >> kb): 8, 4, 2 and 1 of them
#pragma unroll
    for (int kb = 0, q = 0; kb < LOGR; kb++)
#pragma unroll
      for (int j = 0; j < (8 >> kb); j++, q++) wv[q] = __ldg(tw_entry<LOGR, LOGS, LOGN>(tw, LOGN - 1 - kb, kb, G, j));
#pragma unroll
    for (int kb = 0; kb < LOGR; kb++) {
#pragma unroll
      for (int k = 0; k < (1 << LOGR); k++) {
        if (k & (1 << kb)) continue;
        gs_bfly<LOGR>(x, P, kb, k, wv[16 - (16 >> kb) + (k >> (kb + 1))], p, negp);
      }
    }
    gs_end<LOGR>(x, P, p);
  } else {
#pragma unroll
    for (int kb = 0; kb < LOGR; kb++) {
      const int s = LOGN - 1 - (LOGS + kb);
#pragma unroll
      for (int k = 0; k < (1 << LOGR); k++) {
        if (k & (1 << kb)) continue;
        if (s == 0) {
          gs_bfly<LOGR>(x, P, kb, k, ulonglong2{}, p, negp, last);
        } else {
          const ulonglong2 w = __ldg(tw_entry<LOGR, LOGS, LOGN>(tw, s, kb, G, k >> (kb + 1)));
          gs_bfly<LOGR>(x, P, kb, k, w, p, negp);
        }
      }
    }
    if constexpr (!kFinal) gs_end<LOGR>(x, P, p);
  }
}

struct LimbRef {
  const u64* src;
  u64* dst;
  int prime;
  bool valid;
  int job, poly, row;
};

// Flattened limb blockIdx.y -> (job, limb of job); uniform over a cluster.
__device__ __forceinline__ LimbRef locate(const NttBatch& b, int N) {
  const int z = find_job(b.limb_begin, b.njobs, (int)blockIdx.y);
  const NttJob& J = b.jobs[z];
  const int q = (int)blockIdx.y - b.limb_begin[z];
  LimbRef r{nullptr, nullptr, 0, false, z, 0, 0};
  if (q < J.limbs * J.npolys) {
    const int poly = q / J.limbs, j = q - poly * J.limbs;
    r.src = J.src + poly * J.src_stride + (long long)j * N;
    r.dst = J.dst + poly * J.dst_stride + (long long)j * N;
    r.prime = J.prime_of[j];
    r.valid = true;
    r.poly = poly;
    r.row = j;
  }
  return r;
}

template <int LOGN>
struct Shape {
  static constexpr int N = 1 << LOGN;
  static constexpr int LOGE = LOGN < 13 ? LOGN : 13;
  static constexpr int E = 1 << LOGE;
  static constexpr int LOGC = LOGN - LOGE;
  static constexpr int C = 1 << LOGC;
  static constexpr int LOGRA = LOGE - 8;  // pass A radix
  static constexpr int NB = E / 256;      // pass-B groups per CTA (their twiddles are staged in shared memory)
  static constexpr size_t SMEM = sizeof(u64) * E + sizeof(ulonglong2) * 15 * NB;
};

// Twiddles of the middle passes in shared memory (NA = 0 for the radix-32/16 kernels, whose radix-32 pass A has
// one group per CTA and reads its 31 twiddles through L1).  A CTA's pass A (LOGS = 8) and pass B (LOGS = 4) use the
// groups G0 + gl, gl < n (n = NA or NB, G0 = h * n), whose stage-kb twiddles are the contiguous table entries
// 2^s + G0 * 2^(3-kb) + [0, n * 2^(3-kb)).  They are copied once per CTA (cp.async, 16 bytes each, during phase X or
// pass C^-1) into blocks: pass A's four stage blocks (kb = 3 .. 0, n * 2^(3-kb) entries each) then pass B's, so
// stage kb's block starts at n * (2^(3-kb) - 1) within its pass and entry gl * 2^(3-kb) + j is twiddle j of group
// gl.  Without the copy these loads went to L2 whenever the last pass's streaming twiddles had evicted them from
// L1.
template <int LOGN, int NA, int NB>
__device__ __forceinline__ void stage_mid_twiddles(ulonglong2* tws, const ulonglong2* __restrict__ tw, int h) {
  for (int e = threadIdx.x; e < 15 * (NA + NB); e += (int)blockDim.x) {
    const bool passA = e < 15 * NA;
    const int n = passA ? NA : NB, logs = passA ? 8 : 4;
    int local = passA ? e : e - 15 * NA, kb = 3;
    while (local >= (n << (3 - kb))) {
      local -= n << (3 - kb);
      kb--;
    }
    const int st = LOGN - 1 - (logs + kb);
    const ulonglong2* src = tw + (1 << st) + (h * n << (3 - kb)) + local;
    const unsigned dst = (unsigned)__cvta_generic_to_shared(tws + e);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
  }
  asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void wait_staged() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// fwd_radix / inv_radix for a radix-16 pass whose twiddles are staged (stage_mid_twiddles): tws is the pass's
// first block, n its group count, gl the local group.
template <int LOGS, int LOGN>
__device__ __forceinline__ void fwd_radix16_staged(u64 (&x)[16], int gl, const ulonglong2* tws, int n, u64 negp,
                                                   u64 p4) {
#pragma unroll
  for (int kb = 3; kb >= 0; kb--) {
    const int s = LOGN - 1 - (LOGS + kb);
    const ulonglong2* blk = tws + n * ((8 >> kb) - 1) + gl * (8 >> kb);
#pragma unroll
    for (int k = 0; k < 16; k++) {
      if (k & (1 << kb)) continue;
      const ulonglong2 w = blk[k >> (kb + 1)];
      if ((s & 1) == 0)
        ct_bfly<true>(x[k], x[k + (1 << kb)], w, negp, p4);
      else
        ct_bfly<false>(x[k], x[k + (1 << kb)], w, negp, p4);
    }
  }
}
template <int LOGS, int LOGN>
__device__ __forceinline__ void inv_radix16_staged(u64 (&x)[16], int gl, const ulonglong2* tws, int n, u64 negp,
                                                   u64 p) {
  static_assert(LOGS > 0 && LOGS + 4 < LOGN, "a staged pass neither starts nor ends the inverse");
  constexpr GsPlan<4> P = gs_plan<4>(8, 8, false);
  static_assert(P.ok, "a residue needs more halvings than gs_reduce applies");
#pragma unroll
  for (int kb = 0; kb < 4; kb++) {
    const ulonglong2* blk = tws + n * ((8 >> kb) - 1) + gl * (8 >> kb);
#pragma unroll
    for (int k = 0; k < 16; k++) {
      if (k & (1 << kb)) continue;
      gs_bfly<4>(x, P, kb, k, blk[k >> (kb + 1)], p, negp);
    }
  }
  gs_end<4>(x, P, p);
}


// Input side of the fused rescale: the job's one row per poly (coefficients of prime switch_top) switched into
// this limb's prime on load.
// The switched value x (+ diff) is below q_top + p; the transform takes inputs below 16p, so the reduction into
// [0, p) is skipped unless q_top >= 15p (prime sets of very different sizes): the dropped tower's prime is then
// within 15 times the others', which the moduli of a CKKS chain always are.
struct SwitchIn {
  u64 diff = 0, half = 0, one_sh = 0, p = 0;
  bool reduce = true;
  __device__ __forceinline__ u64 operator()(u64 x) const {
    const u64 v = x > half ? x + diff : x;
    return reduce ? shoup(v, 1ull, one_sh, p) : v;
  }
};

__device__ __forceinline__ SwitchIn switch_in(const NttBatch& b, const DeviceTables& T, const NttEpi* e,
                                              const LimbRef& L, const u64*& src) {
  SwitchIn sw;
  const u64 om = T.pc[e->jobs[L.job].switch_top].p;
  src = b.jobs[L.job].src + L.poly * b.jobs[L.job].src_stride;
  sw.p = T.pc[L.prime].p;
  sw.one_sh = T.pc[L.prime].one_sh;
  sw.diff = sw.p - shoup(om, 1ull, sw.one_sh, sw.p);
  sw.half = om >> 1;
  sw.reduce = om >= 15 * sw.p;  // 15p < 2^64 for p < 2^60
  return sw;
}

// Output side of the fused rescale for a thread's 16 contiguous residues x (in [0, 16p)) at n0 .. n0 + 15: out =
// (x_tower - NTT) * q_l^-1 mod p, fully reduced.
template <int LOGN>
__device__ __forceinline__ void epi_store16(const NttEpi* e, const LimbRef& L, int n0, const u64 (&x)[16], u64 p) {
  constexpr int N = 1 << LOGN;
  const u64 p4 = 4 * p;
  const NttEpiJob& E = e->jobs[L.job];
  const ulonglong2 w = E.w[L.row];
  const u64* xr = E.x + ((size_t)L.poly * E.x_ps + L.row) * N + n0;
  ulonglong2* orow = reinterpret_cast<ulonglong2*>(E.out + ((size_t)L.poly * E.out_ps + L.row) * N + n0);
#pragma unroll
  for (int k = 0; k < 16; k += 2) {
    // y in [0, 4p) after two compare-and-subtracts, x in [0, p): x + 4p - y in (0, 5p), reduced by the Shoup product
    const ulonglong2 xv = *reinterpret_cast<const ulonglong2*>(xr + k);
    const u64 y0 = csub(csub(x[k], 2 * p4), p4);
    const u64 y1 = csub(csub(x[k + 1], 2 * p4), p4);
    orow[k / 2] = make_ulonglong2(shoup(xv.x + p4 - y0, w.x, w.y, p), shoup(xv.y + p4 - y1, w.x, w.y, p));
  }
}

// EPI: the fused rescale of NttEpi (null for the plain transform).
// LAZY (plain transform only): outputs left in [0, 4p) (NttBatch::lazy_out) instead of [0, p).
template <int LOGN, bool EPI, bool LAZY = false>
__device__ __forceinline__ void ntt_fwd_body(const NttBatch& b, const DeviceTables& T, const NttEpi* e) {
  using S = Shape<LOGN>;
  extern __shared__ __align__(16) u64 sm[];
  const int tid = threadIdx.x;
  const LimbRef L = locate(b, S::N);
  if (!L.valid) return;
  const u64 p = T.pc[L.prime].p, p2 = 2 * p, p4 = 4 * p, negp = T.pc[L.prime].negp;
  const ulonglong2* __restrict__ tw = T.tw_fwd + (size_t)L.prime * S::N;
  int h = 0;
  if constexpr (S::C > 1) h = (int)cg::this_cluster().block_rank();
  ulonglong2* const tws = reinterpret_cast<ulonglong2*>(sm + S::E);
  stage_mid_twiddles<LOGN, 0, S::NB>(tws, tw, h);
  const u64* src = L.src;
  SwitchIn sw;
  if constexpr (EPI) sw = switch_in(b, T, e, L, src);

  if constexpr (S::C > 1) {
    cg::cluster_group cl = cg::this_cluster();
    const int c = h;
    // "every CTA of the cluster is running" is all the first barrier has to establish (no data is exchanged
    // yet), so it is a relaxed arrive here and a wait just before the distributed-shared-memory stores,
    // overlapping the barrier with the loads and the first butterflies.
    asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");
    constexpr int LPC = S::E / S::C;
    constexpr int IT = LPC / kThreads;
    u64 x[IT][S::C];
#pragma unroll
    for (int it = 0; it < IT; it++) {
      const int l = c * LPC + it * kThreads + tid;
#pragma unroll
      for (int hh = 0; hh < S::C; hh++) x[it][hh] = __ldg(src + hh * S::E + l);
      if constexpr (EPI) {
#pragma unroll
        for (int hh = 0; hh < S::C; hh++) x[it][hh] = sw(x[it][hh]);
      }
    }
#pragma unroll
    for (int it = 0; it < IT; it++) fwd_radix<S::LOGC, S::LOGE, LOGN>(x[it], 0, tw, negp, p4);
    asm volatile("barrier.cluster.wait.aligned;" ::: "memory");
#pragma unroll
    for (int it = 0; it < IT; it++) {
      const int l = c * LPC + it * kThreads + tid;
#pragma unroll
      for (int hh = 0; hh < S::C; hh++) st_peer(peer_smem(sm + swz(l), hh), x[it][hh]);
    }
    cl.sync();
  }

  {  // pass A
    constexpr int R = 1 << S::LOGRA;
    u64 x[R];
#pragma unroll
    for (int k = 0; k < R; k++) {
      const int l = k * 256 + tid;
      if constexpr (S::C > 1)
        x[k] = sm[swz(l)];
      else
        x[k] = (l < S::E) ? (EPI ? sw(__ldg(src + l)) : __ldg(src + l)) : 0ull;
    }
    fwd_radix<S::LOGRA, 8, LOGN>(x, h, tw, negp, p4);
#pragma unroll
    for (int k = 0; k < R; k++) sm[swz(k * 256 + tid)] = x[k];
  }
  wait_staged();
  __syncthreads();

#pragma unroll 1
  for (int g = tid; g < S::E / 16; g += kThreads) {  // pass B
    const int low = g & 15, high = g >> 4;
    u64 x[16];
#pragma unroll
    for (int k = 0; k < 16; k++) x[k] = sm[swz(high * 256 + k * 16 + low)];
    fwd_radix16_staged<4, LOGN>(x, high, tws, S::NB, negp, p4);
#pragma unroll
    for (int k = 0; k < 16; k++) sm[swz(high * 256 + k * 16 + low)] = x[k];
  }
  __syncthreads();

#pragma unroll 1
  for (int g = tid; g < S::E / 16; g += kThreads) {  // pass C
    u64 x[16];
#pragma unroll
    for (int k = 0; k < 16; k += 2) {
      const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(sm + swz(g * 16 + k));
      x[k] = v.x;
      x[k + 1] = v.y;
    }
    fwd_radix<4, 0, LOGN>(x, h * (S::E / 16) + g, tw, negp, p4);
    if constexpr (EPI) {
      epi_store16<LOGN>(e, L, h * S::E + g * 16, x, p);
    } else {
      ulonglong2* out = reinterpret_cast<ulonglong2*>(L.dst + h * S::E + g * 16);
#pragma unroll
      for (int k = 0; k < 16; k += 2) {
        ulonglong2 v;
        if constexpr (LAZY) {
          v.x = csub(csub(x[k], 2 * p4), p4);
          v.y = csub(csub(x[k + 1], 2 * p4), p4);
        } else {
          v.x = csub(csub(csub(csub(x[k], 2 * p4), p4), p2), p);
          v.y = csub(csub(csub(csub(x[k + 1], 2 * p4), p4), p2), p);
        }
        out[k / 2] = v;
      }
    }
  }
}

template <int LOGN, bool LAZY>
__global__ void __launch_bounds__(kThreads, 2) ntt_fwd_kernel(const __grid_constant__ NttBatch b,
                                                           const __grid_constant__ DeviceTables T) {
  pdl_prologue();
  ntt_fwd_body<LOGN, false, LAZY>(b, T, nullptr);
}

template <int LOGN>
__global__ void __launch_bounds__(kThreads, 2) ntt_fwd_epi_kernel(const __grid_constant__ NttBatch b,
                                                               const __grid_constant__ DeviceTables T,
                                                               const __grid_constant__ NttEpi e) {
  pdl_prologue();
  ntt_fwd_body<LOGN, true>(b, T, &e);
}

// LAZY: outputs left in [0, 4p) (NttBatch::lazy_out), a compile-time choice so the exact path pays no branch.
template <int LOGN, bool LAZY>
__global__ void __launch_bounds__(kThreads, 2) ntt_inv_kernel(const __grid_constant__ NttBatch b,
                                                           const __grid_constant__ DeviceTables T) {
  pdl_prologue();
  using S = Shape<LOGN>;
  extern __shared__ __align__(16) u64 sm[];
  const int tid = threadIdx.x;
  const LimbRef L = locate(b, S::N);
  if (!L.valid) return;
  const PrimeConst& pc = T.pc[L.prime];
  const u64 p = pc.p, p2 = 2 * p, negp = pc.negp;
  const ulonglong2* __restrict__ tw = T.tw_inv + (size_t)L.prime * S::N;
  int h = 0;
  if constexpr (S::C > 1) h = (int)cg::this_cluster().block_rank();
  ulonglong2* const tws = reinterpret_cast<ulonglong2*>(sm + S::E);
  stage_mid_twiddles<LOGN, 0, S::NB>(tws, tw, h);

#pragma unroll 1
  for (int g = tid; g < S::E / 16; g += kThreads) {  // pass C^-1
    u64 x[16];
    const ulonglong2* in = reinterpret_cast<const ulonglong2*>(L.src + h * S::E + g * 16);
#pragma unroll
    for (int k = 0; k < 16; k += 2) {
      const ulonglong2 v = __ldg(in + k / 2);
      x[k] = v.x;
      x[k + 1] = v.y;
    }
    inv_radix<4, 0, LOGN>(x, h * (S::E / 16) + g, tw, negp, p);
#pragma unroll
    for (int k = 0; k < 16; k += 2) *reinterpret_cast<ulonglong2*>(sm + swz(g * 16 + k)) = make_ulonglong2(x[k], x[k + 1]);
  }
  wait_staged();
  __syncthreads();

#pragma unroll 1
  for (int g = tid; g < S::E / 16; g += kThreads) {  // pass B^-1
    const int low = g & 15, high = g >> 4;
    u64 x[16];
#pragma unroll
    for (int k = 0; k < 16; k++) x[k] = sm[swz(high * 256 + k * 16 + low)];
    inv_radix16_staged<4, LOGN>(x, high, tws, S::NB, negp, p);
#pragma unroll
    for (int k = 0; k < 16; k++) sm[swz(high * 256 + k * 16 + low)] = x[k];
  }
  __syncthreads();

  {  // pass A^-1
    constexpr int R = 1 << S::LOGRA;
    // gs_plan's lim for this radix-32 pass: 8 keeps one 64-bit constant out of the registers (128 a thread, 20 bytes
    // of spills with 16); 640 limbs at N = 2^16 take 0.494 ms against 0.507-0.522 ms with 16.
    constexpr int kLim = 8;
    u64 x[R];
#pragma unroll
    for (int k = 0; k < R; k++) {
      const int l = k * 256 + tid;
      x[k] = (l < S::E) ? sm[swz(l)] : 0ull;
    }
    if constexpr (S::C == 1) {  // this pass ends the transform
      const LastStage last{pc.ninv, pc.ninv_sh, pc.w1ninv, pc.w1ninv_sh};
      inv_radix<S::LOGRA, 8, LOGN, kLim>(x, h, tw, negp, p, &last);
#pragma unroll
      for (int k = 0; k < R; k++) {
        const int l = k * 256 + tid;
        if (l < S::E) L.dst[l] = LAZY ? x[k] : csub(csub(x[k], p2), p);
      }
      return;
    } else {
      inv_radix<S::LOGRA, 8, LOGN, kLim>(x, h, tw, negp, p);
#pragma unroll
      for (int k = 0; k < R; k++) sm[swz(k * 256 + tid)] = x[k];
    }
  }

  if constexpr (S::C > 1) {  // phase X^-1 across the cluster
    cg::cluster_group cl = cg::this_cluster();
    cl.sync();
    const int c = h;
    constexpr int LPC = S::E / S::C;
    constexpr int IT = LPC / kThreads;
#pragma unroll
    for (int it = 0; it < IT; it++) {
      const int l = c * LPC + it * kThreads + tid;
      u64 x[S::C];
#pragma unroll
      for (int hh = 0; hh < S::C; hh++) x[hh] = ld_peer(peer_smem(sm + swz(l), hh));
      const LastStage last{pc.ninv, pc.ninv_sh, pc.w1ninv, pc.w1ninv_sh};
      inv_radix<S::LOGC, S::LOGE, LOGN>(x, 0, tw, negp, p, &last);
#pragma unroll
      for (int hh = 0; hh < S::C; hh++) L.dst[hh * S::E + l] = LAZY ? x[hh] : csub(csub(x[hh], p2), p);
    }
    cl.sync();  // peers may still be reading this CTA's shared memory
  }
}

// ---- forward, N = 2^13 .. 2^16: radix-16 passes, 16 residues per thread ----
//
// Same cluster layout as above with a per-CTA share of E = 2^LOGE residues (LOGE = 13: C = N/8192 CTAs with 64 KiB
// of shared memory each; LOGE = 12: twice the CTAs per limb with 32 KiB each, for small batches whose launch
// latency matters more than throughput).  Every pass works on 16-residue groups, so a thread holds 16 residues
// at a time: 256 threads per CTA each take E/4096 groups per pass, and with 80 registers a thread three CTAs
// share an SM (24 warps; 8-CTA clusters then also pack a 19-SM GPC almost fully).  Passes:
//   X : bits [LOGN-1 .. 12] (LOGX = LOGN - 12 bits; the top LOGC of them cross CTAs via distributed shared
//       memory, the rest (bit 12 when LOGE = 13) inside the CTA) on columns l' in [0, 4096) of CTA c's share;
//   A : bits [11 .. 8]   (16 residues at stride 256),
//   B : bits [7 .. 4]    (16 residues at stride 16),
//   C : bits [3 .. 0]    (16 contiguous residues), then the store to HBM.
// The profile of this kernel shows the ALU pipe (64-bit compares, selects and adds of the lazy reductions) as the
// busiest unit; occupancy (16, 24 or 32 warps per SM) barely moves its time.
constexpr int kThreads16 = 256;

template <int LOGN, int LOGE>
struct Shape16 {
  static constexpr int N = 1 << LOGN;
  static constexpr int E = 1 << LOGE;
  static constexpr int LOGC = LOGN - LOGE;
  static constexpr int C = 1 << LOGC;
  static constexpr int LOGX = LOGN - 12;
  static constexpr int LOCAL = LOGE - 12;                  // phase-X bits inside the CTA (0 or 1)
  static constexpr int COLS = 4096 / C;                    // phase-X columns per CTA
  static constexpr int GX = COLS / kThreads16;             // phase-X groups per thread
  static constexpr int GROUPS = E / 16;                    // 16-residue groups per pass
  static constexpr int NA = E / 4096;                      // pass-A groups (G values) per CTA
  static constexpr int NB = E / 256;                       // pass-B groups per CTA
  static constexpr int TWS = 15 * (NA + NB);               // twiddles of passes A and B staged in shared memory
  static constexpr size_t SMEM = sizeof(u64) * E + sizeof(ulonglong2) * TWS;
};

// EPI: the fused rescale of NttEpi (null for the plain transform).
template <int LOGN, int LOGE, bool EPI, bool LAZY = false>
__device__ __forceinline__ void ntt16_fwd_body(const NttBatch& b, const DeviceTables& T, const NttEpi* e) {
  using S = Shape16<LOGN, LOGE>;
  extern __shared__ __align__(16) u64 sm[];
  const int tid = threadIdx.x;
  const LimbRef L = locate(b, S::N);
  if (!L.valid) return;
  const u64 p = T.pc[L.prime].p, p2 = 2 * p, p4 = 4 * p, negp = T.pc[L.prime].negp;
  const ulonglong2* __restrict__ tw = T.tw_fwd + (size_t)L.prime * S::N;
  int h = 0;
  if constexpr (S::C > 1) {
    asm volatile("barrier.cluster.arrive.relaxed.aligned;" ::: "memory");
    h = (int)cg::this_cluster().block_rank();
  }
  ulonglong2* const tws = reinterpret_cast<ulonglong2*>(sm + S::E);
  stage_mid_twiddles<LOGN, S::NA, S::NB>(tws, tw, h);
  const u64* src = L.src;
  SwitchIn sw;
  if constexpr (EPI) sw = switch_in(b, T, e, L, src);
  {  // phase X: residue k*4096 + col lives in CTA k >> LOCAL at (k & local mask) * 4096 + col
    constexpr int R = 1 << S::LOGX;
#pragma unroll 1
    for (int q = 0; q < S::GX; q++) {
      const int col = h * S::COLS + q * kThreads16 + tid;
      u64 x[R];
#pragma unroll
      for (int k = 0; k < R; k++) x[k] = __ldg(src + k * 4096 + col);
      if constexpr (EPI) {
#pragma unroll
        for (int k = 0; k < R; k++) x[k] = sw(x[k]);
      }
      fwd_radix<S::LOGX, 12, LOGN>(x, 0, tw, negp, p4);
      if constexpr (S::C > 1) {
        if (q == 0) asm volatile("barrier.cluster.wait.aligned;" ::: "memory");
#pragma unroll
        for (int k = 0; k < R; k++)
          st_peer(peer_smem(sm + swz((k & ((1 << S::LOCAL) - 1)) * 4096 + col), k >> S::LOCAL), x[k]);
      } else {
#pragma unroll
        for (int k = 0; k < R; k++) sm[swz(k * 4096 + col)] = x[k];
      }
    }
    wait_staged();
    if constexpr (S::C > 1)
      cg::this_cluster().sync();
    else
      __syncthreads();
  }
#pragma unroll 1
  for (int g = tid; g < S::GROUPS; g += kThreads16) {  // pass A
    const int hi = g >> 8, low = g & 255;
    u64 x[16];
#pragma unroll
    for (int k = 0; k < 16; k++) x[k] = sm[swz(hi * 4096 + k * 256 + low)];
    fwd_radix16_staged<8, LOGN>(x, hi, tws, S::NA, negp, p4);
#pragma unroll
    for (int k = 0; k < 16; k++) sm[swz(hi * 4096 + k * 256 + low)] = x[k];
  }
  __syncthreads();
#pragma unroll 1
  for (int g = tid; g < S::GROUPS; g += kThreads16) {  // pass B
    const int low = g & 15, high = g >> 4;
    u64 x[16];
#pragma unroll
    for (int k = 0; k < 16; k++) x[k] = sm[swz(high * 256 + k * 16 + low)];
    fwd_radix16_staged<4, LOGN>(x, high, tws + 15 * S::NA, S::NB, negp, p4);
#pragma unroll
    for (int k = 0; k < 16; k++) sm[swz(high * 256 + k * 16 + low)] = x[k];
  }
  __syncthreads();
#pragma unroll 1
  for (int g = tid; g < S::GROUPS; g += kThreads16) {  // pass C
    u64 x[16];
#pragma unroll
    for (int k = 0; k < 16; k += 2) {
      const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(sm + swz(g * 16 + k));
      x[k] = v.x;
      x[k + 1] = v.y;
    }
    fwd_radix<4, 0, LOGN>(x, h * S::GROUPS + g, tw, negp, p4);
    if constexpr (EPI) {
      epi_store16<LOGN>(e, L, h * S::E + g * 16, x, p);
    } else {
      ulonglong2* out = reinterpret_cast<ulonglong2*>(L.dst + h * S::E + g * 16);
#pragma unroll
      for (int k = 0; k < 16; k += 2) {
        ulonglong2 v;
        if constexpr (LAZY) {
          v.x = csub(csub(x[k], 2 * p4), p4);
          v.y = csub(csub(x[k + 1], 2 * p4), p4);
        } else {
          v.x = csub(csub(csub(csub(x[k], 2 * p4), p4), p2), p);
          v.y = csub(csub(csub(csub(x[k + 1], 2 * p4), p4), p2), p);
        }
        out[k / 2] = v;
      }
    }
  }
}

template <int LOGN, int LOGE, bool LAZY>
__global__ void __launch_bounds__(kThreads16, 3) ntt16_fwd_kernel(const __grid_constant__ NttBatch b,
                                                                 const __grid_constant__ DeviceTables T) {
  pdl_prologue();
  ntt16_fwd_body<LOGN, LOGE, false, LAZY>(b, T, nullptr);
}

// The forward transform with the fused rescale (NttEpi).
template <int LOGN, int LOGE>
__global__ void __launch_bounds__(kThreads16, 3) ntt16_fwd_epi_kernel(const __grid_constant__ NttBatch b,
                                                                     const __grid_constant__ DeviceTables T,
                                                                     const __grid_constant__ NttEpi e) {
  pdl_prologue();
  ntt16_fwd_body<LOGN, LOGE, true>(b, T, &e);
}

// Inverse of the same shape (Gentleman–Sande, passes C^-1, B^-1, A^-1, then the cross-CTA phase X^-1 reading
// the peers' shared memory; N^-1 applied on the way out), with LOGE = 12 or 13 (autotuned); LAZY as for
// ntt_inv_kernel.
template <int LOGN, int LOGE, bool LAZY>
__global__ void __launch_bounds__(kThreads16, 3) ntt16_inv_kernel(const __grid_constant__ NttBatch b,
                                                                 const __grid_constant__ DeviceTables T) {
  pdl_prologue();
  using S = Shape16<LOGN, LOGE>;
  extern __shared__ __align__(16) u64 sm[];
  const int tid = threadIdx.x;
  const LimbRef L = locate(b, S::N);
  if (!L.valid) return;
  const PrimeConst& pc = T.pc[L.prime];
  const u64 p = pc.p, p2 = 2 * p, negp = pc.negp;
  const ulonglong2* __restrict__ tw = T.tw_inv + (size_t)L.prime * S::N;
  int h = 0;
  if constexpr (S::C > 1) h = (int)cg::this_cluster().block_rank();
  ulonglong2* const tws = reinterpret_cast<ulonglong2*>(sm + S::E);
  stage_mid_twiddles<LOGN, S::NA, S::NB>(tws, tw, h);
#pragma unroll 1
  for (int g = tid; g < S::GROUPS; g += kThreads16) {  // pass C^-1
    u64 x[16];
    const ulonglong2* in = reinterpret_cast<const ulonglong2*>(L.src + h * S::E + g * 16);
#pragma unroll
    for (int k = 0; k < 16; k += 2) {
      const ulonglong2 v = __ldg(in + k / 2);
      x[k] = v.x;
      x[k + 1] = v.y;
    }
    inv_radix<4, 0, LOGN>(x, h * S::GROUPS + g, tw, negp, p);
#pragma unroll
    for (int k = 0; k < 16; k += 2) *reinterpret_cast<ulonglong2*>(sm + swz(g * 16 + k)) = make_ulonglong2(x[k], x[k + 1]);
  }
  wait_staged();
  __syncthreads();
#pragma unroll 1
  for (int g = tid; g < S::GROUPS; g += kThreads16) {  // pass B^-1
    const int low = g & 15, high = g >> 4;
    u64 x[16];
#pragma unroll
    for (int k = 0; k < 16; k++) x[k] = sm[swz(high * 256 + k * 16 + low)];
    inv_radix16_staged<4, LOGN>(x, high, tws + 15 * S::NA, S::NB, negp, p);
#pragma unroll
    for (int k = 0; k < 16; k++) sm[swz(high * 256 + k * 16 + low)] = x[k];
  }
  __syncthreads();
#pragma unroll 1
  for (int g = tid; g < S::GROUPS; g += kThreads16) {  // pass A^-1
    const int hi = g >> 8, low = g & 255;
    u64 x[16];
#pragma unroll
    for (int k = 0; k < 16; k++) x[k] = sm[swz(hi * 4096 + k * 256 + low)];
    inv_radix16_staged<8, LOGN>(x, hi, tws, S::NA, negp, p);
#pragma unroll
    for (int k = 0; k < 16; k++) sm[swz(hi * 4096 + k * 256 + low)] = x[k];
  }
  {  // phase X^-1
    constexpr int R = 1 << S::LOGX;
    if constexpr (S::C > 1)
      cg::this_cluster().sync();
    else
      __syncthreads();
#pragma unroll 1
    for (int q = 0; q < S::GX; q++) {
      const int col = h * S::COLS + q * kThreads16 + tid;
      u64 x[R];
      if constexpr (S::C > 1) {
#pragma unroll
        for (int k = 0; k < R; k++)
          x[k] = ld_peer(peer_smem(sm + swz((k & ((1 << S::LOCAL) - 1)) * 4096 + col), k >> S::LOCAL));
      } else {
#pragma unroll
        for (int k = 0; k < R; k++) x[k] = sm[swz(k * 4096 + col)];
      }
      const LastStage last{pc.ninv, pc.ninv_sh, pc.w1ninv, pc.w1ninv_sh};
      inv_radix<S::LOGX, 12, LOGN>(x, 0, tw, negp, p, &last);
#pragma unroll
      for (int k = 0; k < R; k++) L.dst[k * 4096 + col] = LAZY ? x[k] : csub(csub(x[k], p2), p);
    }
    if constexpr (S::C > 1) cg::this_cluster().sync();  // peers may still be reading this CTA's shared memory
  }
}

template <int LOGN, int LOGE>
cudaError_t launch16(const NttBatch& b, const DeviceTables& t, bool inverse, cudaStream_t s) {
  using S = Shape16<LOGN, LOGE>;
  const int which = (inverse ? 2 : 0) + (b.lazy_out ? 1 : 0);
  auto kern = which == 3   ? ntt16_inv_kernel<LOGN, LOGE, true>
              : which == 2 ? ntt16_inv_kernel<LOGN, LOGE, false>
              : which == 1 ? ntt16_fwd_kernel<LOGN, LOGE, true>
                           : ntt16_fwd_kernel<LOGN, LOGE, false>;
  static std::atomic<unsigned long long> attr_done[4];
  const size_t smem = S::SMEM;
  const cudaError_t ea = once_per_device(attr_done[which], [&] {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess && S::C > 8) e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return e;
  });
  if (ea != cudaSuccess) return ea;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(S::C, b.limb_begin[b.njobs], 1);
  cfg.blockDim = dim3(kThreads16, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  attr[1].id = cudaLaunchAttributeClusterDimension;
  attr[1].val.clusterDim.x = S::C;
  attr[1].val.clusterDim.y = 1;
  attr[1].val.clusterDim.z = 1;
  // the programmatic-serialization attribute for a grid of fewer CTAs than SMs (see launch_pdl), the cluster shape
  cfg.attrs = pdl_for((long long)cfg.gridDim.x * cfg.gridDim.y) ? attr : attr + 1;
  cfg.numAttrs = (cfg.attrs == attr ? 1 : 0) + (S::C > 1 ? 1 : 0);
  cudaError_t e = cudaLaunchKernelEx(&cfg, kern, b, t);
  if (e != cudaSuccess) return e;
  count_launch();
  return cudaSuccess;
}

template <int LOGN, int LOGE>
cudaError_t launch16_epi(const NttBatch& b, const NttEpi& e, const DeviceTables& t, cudaStream_t s) {
  using S = Shape16<LOGN, LOGE>;
  auto kern = ntt16_fwd_epi_kernel<LOGN, LOGE>;
  static std::atomic<unsigned long long> attr_done;
  const size_t smem = S::SMEM;
  const cudaError_t ea = once_per_device(attr_done, [&] {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess && S::C > 8) e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return e;
  });
  if (ea != cudaSuccess) return ea;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(S::C, b.limb_begin[b.njobs], 1);
  cfg.blockDim = dim3(kThreads16, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  attr[1].id = cudaLaunchAttributeClusterDimension;
  attr[1].val.clusterDim.x = S::C;
  attr[1].val.clusterDim.y = 1;
  attr[1].val.clusterDim.z = 1;
  // the programmatic-serialization attribute for a grid of fewer CTAs than SMs (see launch_pdl), the cluster shape
  cfg.attrs = pdl_for((long long)cfg.gridDim.x * cfg.gridDim.y) ? attr : attr + 1;
  cfg.numAttrs = (cfg.attrs == attr ? 1 : 0) + (S::C > 1 ? 1 : 0);
  cudaError_t err = cudaLaunchKernelEx(&cfg, kern, b, t, e);
  if (err != cudaSuccess) return err;
  count_launch();
  return cudaSuccess;
}

template <int LOGN>
cudaError_t launch_t_epi(const NttBatch& b, const NttEpi& e, const DeviceTables& t, cudaStream_t s) {
  using S = Shape<LOGN>;
  auto kern = ntt_fwd_epi_kernel<LOGN>;
  static std::atomic<unsigned long long> attr_done;
  const size_t smem = S::SMEM;
  const cudaError_t ea = once_per_device(attr_done, [&] {
    return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  });
  if (ea != cudaSuccess) return ea;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(S::C, b.limb_begin[b.njobs], 1);
  cfg.blockDim = dim3(kThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  attr[1].id = cudaLaunchAttributeClusterDimension;
  attr[1].val.clusterDim.x = S::C;
  attr[1].val.clusterDim.y = 1;
  attr[1].val.clusterDim.z = 1;
  // the programmatic-serialization attribute for a grid of fewer CTAs than SMs (see launch_pdl), the cluster shape
  cfg.attrs = pdl_for((long long)cfg.gridDim.x * cfg.gridDim.y) ? attr : attr + 1;
  cfg.numAttrs = (cfg.attrs == attr ? 1 : 0) + (S::C > 1 ? 1 : 0);
  cudaError_t err = cudaLaunchKernelEx(&cfg, kern, b, t, e);
  if (err != cudaSuccess) return err;
  count_launch();
  return cudaSuccess;
}

template <int LOGN>
cudaError_t launch_t(const NttBatch& b, const DeviceTables& t, bool inverse, cudaStream_t s) {
  using S = Shape<LOGN>;
  const int which = (inverse ? 2 : 0) + (b.lazy_out ? 1 : 0);
  auto kern = which == 3   ? ntt_inv_kernel<LOGN, true>
              : which == 2 ? ntt_inv_kernel<LOGN, false>
              : which == 1 ? ntt_fwd_kernel<LOGN, true>
                           : ntt_fwd_kernel<LOGN, false>;
  static std::atomic<unsigned long long> attr_done[4];
  const size_t smem = S::SMEM;
  const cudaError_t ea = once_per_device(attr_done[which], [&] {
    return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  });
  if (ea != cudaSuccess) return ea;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(S::C, b.limb_begin[b.njobs], 1);
  cfg.blockDim = dim3(kThreads, 1, 1);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  attr[1].id = cudaLaunchAttributeClusterDimension;
  attr[1].val.clusterDim.x = S::C;
  attr[1].val.clusterDim.y = 1;
  attr[1].val.clusterDim.z = 1;
  // the programmatic-serialization attribute for a grid of fewer CTAs than SMs (see launch_pdl), the cluster shape
  cfg.attrs = pdl_for((long long)cfg.gridDim.x * cfg.gridDim.y) ? attr : attr + 1;
  cfg.numAttrs = (cfg.attrs == attr ? 1 : 0) + (S::C > 1 ? 1 : 0);
  cudaError_t e = cudaLaunchKernelEx(&cfg, kern, b, t);
  if (e != cudaSuccess) return e;
  count_launch();
  return cudaSuccess;
}

}  // namespace

cudaError_t launch_ntt(const NttBatch& b, const DeviceTables& t, bool inverse, cudaStream_t s) {
  if (b.njobs <= 0 || b.limb_begin[b.njobs] <= 0) return cudaSuccess;
  if (b.njobs > kMaxNttJobs || b.limb_begin[b.njobs] > 65535) return cudaErrorInvalidValue;
  const long long work = (long long)b.limb_begin[b.njobs] << t.logN;
  const int cls = work <= kTinyNttWork ? 0 : work <= kSmallNttWork ? 1 : 2;
  const int v = inverse ? (cls == 0   ? t.inv_variant_tiny
                           : cls == 1 ? t.inv_variant_small
                           : b.lazy_out ? t.inv_variant_ks
                                        : t.inv_variant)
                        : (cls == 0 ? t.fwd_variant_tiny : cls == 1 ? t.fwd_variant_small : t.fwd_variant);
  switch (t.logN) {
    case 10: return launch_t<10>(b, t, inverse, s);
    case 11: return launch_t<11>(b, t, inverse, s);
    case 12: return launch_t<12>(b, t, inverse, s);
    // the variants tune_ntt picked for this direction and batch size (forward: 0 = radix-16 / 8192 per CTA,
    // 1 = radix-32/16, 2 = radix-16 / 4096 per CTA; inverse: 0 = radix-32/16, 1 = radix-16 / 4096 per CTA,
    // 2 = radix-16 / 8192 per CTA)
    case 13:
      if (inverse) return v == 0 ? launch_t<13>(b, t, true, s) : v == 1 ? launch16<13, 12>(b, t, true, s)
                                                         : launch16<13, 13>(b, t, true, s);
      return v == 1 ? launch_t<13>(b, t, false, s) : v == 0 ? launch16<13, 13>(b, t, false, s)
                                                           : launch16<13, 12>(b, t, false, s);
    case 14:
      if (inverse) return v == 0 ? launch_t<14>(b, t, true, s) : v == 1 ? launch16<14, 12>(b, t, true, s)
                                                         : launch16<14, 13>(b, t, true, s);
      return v == 1 ? launch_t<14>(b, t, false, s) : v == 0 ? launch16<14, 13>(b, t, false, s)
                                                           : launch16<14, 12>(b, t, false, s);
    case 15:
      if (inverse) return v == 0 ? launch_t<15>(b, t, true, s) : v == 1 ? launch16<15, 12>(b, t, true, s)
                                                         : launch16<15, 13>(b, t, true, s);
      return v == 1 ? launch_t<15>(b, t, false, s) : v == 0 ? launch16<15, 13>(b, t, false, s)
                                                           : launch16<15, 12>(b, t, false, s);
    case 16:
      if (inverse) return v == 0 ? launch_t<16>(b, t, true, s) : v == 1 ? launch16<16, 12>(b, t, true, s)
                                                         : launch16<16, 13>(b, t, true, s);
      return v == 1 ? launch_t<16>(b, t, false, s) : v == 0 ? launch16<16, 13>(b, t, false, s)
                                                           : launch16<16, 12>(b, t, false, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_ntt_epi(const NttBatch& b, const NttEpi& e, const DeviceTables& t, cudaStream_t s) {
  if (b.njobs <= 0 || b.limb_begin[b.njobs] <= 0) return cudaSuccess;
  if (b.njobs > kMaxNttJobs || b.limb_begin[b.njobs] > 65535) return cudaErrorInvalidValue;
  // the forward variant the autotuner picked for this batch size (as launch_ntt)
  const long long work = (long long)b.limb_begin[b.njobs] << t.logN;
  const int cls = work <= kTinyNttWork ? 0 : work <= kSmallNttWork ? 1 : 2;
  const int v = cls == 0 ? t.fwd_variant_tiny : cls == 1 ? t.fwd_variant_small : t.fwd_variant;
  switch (t.logN) {
    case 10: return launch_t_epi<10>(b, e, t, s);
    case 11: return launch_t_epi<11>(b, e, t, s);
    case 12: return launch_t_epi<12>(b, e, t, s);
    case 13: return v == 1 ? launch_t_epi<13>(b, e, t, s) : v == 2 ? launch16_epi<13, 12>(b, e, t, s)
                                                                   : launch16_epi<13, 13>(b, e, t, s);
    case 14: return v == 1 ? launch_t_epi<14>(b, e, t, s) : v == 2 ? launch16_epi<14, 12>(b, e, t, s)
                                                                   : launch16_epi<14, 13>(b, e, t, s);
    case 15: return v == 1 ? launch_t_epi<15>(b, e, t, s) : v == 2 ? launch16_epi<15, 12>(b, e, t, s)
                                                                   : launch16_epi<15, 13>(b, e, t, s);
    case 16: return v == 1 ? launch_t_epi<16>(b, e, t, s) : v == 2 ? launch16_epi<16, 12>(b, e, t, s)
                                                                   : launch16_epi<16, 13>(b, e, t, s);
    default: return cudaErrorNotSupported;
  }
}

cudaError_t tune_ntt(DeviceTables& t, cudaStream_t s, float* ms) {
  constexpr int kSlots = kNttSizeClasses * (kNttFwdVariants + kNttInvVariants);
  if (ms)
    for (int i = 0; i < kSlots; i++) ms[i] = -1.f;
  if (t.logN < 13) return cudaSuccess;  // one kernel per direction below 2^13
  const size_t n = (size_t)1 << t.logN;
  const int sizes[kNttSizeClasses] = {(int)((8ll << 16) >> t.logN), (int)((32ll << 16) >> t.logN),
                                      (int)((640ll << 16) >> t.logN)};
  const int large = sizes[kNttSizeClasses - 1];
  u64* buf = nullptr;
  cudaError_t e = cudaMallocAsync(&buf, (size_t)large * n * sizeof(u64), s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(buf, 0, (size_t)large * n * sizeof(u64), s);  // zeros are valid residues of every prime
  cudaEvent_t ev[2];
  cudaEventCreate(&ev[0]);
  cudaEventCreate(&ev[1]);
  int slot = 0;  // ms layout: forward tiny, small, large, then inverse tiny, small, large
  for (int inverse = 0; inverse < 2 && e == cudaSuccess; inverse++) {
    const int nv = inverse ? kNttInvVariants : kNttFwdVariants;
    for (int size = 0; size < kNttSizeClasses && e == cudaSuccess; size++) {
      NttBatch b{};
      uint8_t pm[1] = {0};
      ntt_add_job(b, buf, buf, (long long)n, (long long)n, 1, sizes[size], pm);
      float best = 0, el_v[kNttInvVariants > kNttFwdVariants ? kNttInvVariants : kNttFwdVariants] = {};
      int pick = 0;
      for (int v = 0; v < nv && e == cudaSuccess; v++, slot++) {
        DeviceTables tv = t;
        tv.fwd_variant = tv.fwd_variant_small = tv.fwd_variant_tiny = v;
        tv.inv_variant = tv.inv_variant_small = tv.inv_variant_tiny = v;
        e = launch_ntt(b, tv, inverse, s);  // warm-up
        if (e == cudaSuccess) e = cudaEventRecord(ev[0], s);
        for (int r = 0; r < 3 && e == cudaSuccess; r++) e = launch_ntt(b, tv, inverse, s);
        if (e == cudaSuccess) e = cudaEventRecord(ev[1], s);
        if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
        float el = 0;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&el, ev[0], ev[1]);
        el /= 3;
        el_v[v] = el;
        if (ms) ms[slot] = el;
        if (v == 0 || el < best) {
          best = el;
          pick = v;
        }
      }
      if (e == cudaSuccess) {
        int* dst[2][kNttSizeClasses] = {{&t.fwd_variant_tiny, &t.fwd_variant_small, &t.fwd_variant},
                                        {&t.inv_variant_tiny, &t.inv_variant_small, &t.inv_variant}};
        *dst[inverse][size] = pick;
        if (inverse && size == kNttSizeClasses - 1)  // the faster radix-16 variant (3 CTAs per SM)
          t.inv_variant_ks = el_v[1] <= el_v[2] ? 1 : 2;
      }
    }
  }
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  cudaFreeAsync(buf, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e;
}

}  // namespace fgb
