// Batched 64-bit negacyclic NTT / INTT for sm_103a.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "arith.cuh"

namespace fgb {

// One job = `npolys` polynomials of `limbs` towers.  Tower j of poly k is read from
// src + k*src_stride + j*N and written to dst + k*dst_stride + j*N (src == dst: in place), modulo prime
// index prime_of[j].  A launch carries up to kMaxNttJobs jobs in kernel-parameter space; every limb of
// every job is one thread-block cluster.
struct NttJob {
  const u64* src;
  u64* dst;
  long long src_stride;
  long long dst_stride;
  int limbs;
  int npolys;
  uint8_t prime_of[64];
};

constexpr int kMaxNttJobs = 64;

struct NttBatch {
  int njobs;
  int lazy_out;  // outputs left in [0, 4p) instead of [0, p), for readers that reduce them (see NttQueue)
  int limb_begin[kMaxNttJobs + 1];  // prefix sums of limbs * npolys: grid.y covers exactly the real limbs
  NttJob jobs[kMaxNttJobs];
};

// Rescale fused into the forward transform, as the reference's NTT_RESCALE fusion folds its epilogue into the NTT
// (src/NTTfusions.cuh:214-235).  NTT job z reads one row per poly k (coefficients of prime switch_top, the INTT of
// the dropped tower, at src + k * src_stride), switches each value into q_j on load with the centred rule
// (x > q_top / 2: x + q_j - [q_top]_{q_j}), transforms it, and instead of storing the transform writes
//   out[k * out_ps + j][n] = (x[k * x_ps + j][n] - NTT(switched row)[n]) * w[j]  mod q_j      (x in [0, q_j))
// for limbs j < limbs of the job.  (A ModDown fused the same way measured slower on single operations and no faster
// on batches than its separate epilogue kernel, so ModDown keeps that kernel.)
struct NttEpiJob {
  const u64* x;
  u64* out;
  const ulonglong2* w;  // [j] = {w_j, shoup(w_j)}
  int x_ps;             // poly stride of x in limbs
  int out_ps;           // poly stride of out in limbs
  int switch_top;
};

struct NttEpi {
  NttEpiJob jobs[kMaxNttJobs];
};

struct DeviceTables {
  const PrimeConst* pc;      // [ntowers]
  // [ntowers][N] {psi^brev(i), shoup} / {psi^-brev(i), shoup}, with the entries of the last four stages transposed:
  // entry m + G*nw + j of stage s >= logN - 4 (m = 2^s, nw = m*16/N twiddles per 16-residue group G) is stored at
  // m + j*(N/16) + G
  const ulonglong2* tw_fwd;
  const ulonglong2* tw_inv;
  int logN;
  // forward kernel for N >= 2^13 (0 = radix-16 with 8192 residues per CTA; 1 = radix-32/16; 2 = radix-16 with 4096
  // residues per CTA, twice the CTAs per limb), chosen by tune_ntt separately for launches of at most
  // kTinyNttWork residues (one op: latency-bound), at most kSmallNttWork and larger ones (throughput-bound)
  int fwd_variant = 0;
  int fwd_variant_small = 0;
  int fwd_variant_tiny = 0;
  int inv_variant = 0;  // inverse: 0 = radix-32/16, 1 = radix-16 with 4096, 2 = with 8192 residues per CTA
  int inv_variant_small = 0;
  int inv_variant_tiny = 0;
  // The key switch's large inverse launches (lazy outputs), whose two halves run on two streams beside the other
  // half's conversions and inner products: the faster of the radix-16 variants (1, 2; 80 registers a thread, three
  // CTAs per SM), which share the SMs better than the radix-32/16 kernel (128 registers, two CTAs per SM).  At
  // N = 2^16, 64 batched rotations run 1.1% faster with it although the radix-32/16 kernel is 1.6% faster alone.
  int inv_variant_ks = 0;
};
constexpr int kNttFwdVariants = 3;
constexpr int kNttInvVariants = 3;
constexpr int kNttSizeClasses = 3;                // tiny, small, large
constexpr long long kTinyNttWork = 16ll << 16;    // residues per launch (16 limbs at N = 2^16)
constexpr long long kSmallNttWork = 128ll << 16;  // 128 limbs at N = 2^16

// Forward (inverse=false: coefficient -> evaluation, bit-reversed) or inverse transform of every job.
cudaError_t launch_ntt(const NttBatch& b, const DeviceTables& t, bool inverse, cudaStream_t s);

// Forward transform of every job with the fused rescale `e`, on the kernel variant launch_ntt would pick
// (N = 2^10 .. 2^16).
cudaError_t launch_ntt_epi(const NttBatch& b, const NttEpi& e, const DeviceTables& t, cudaStream_t s);

// Autotuner: times every kernel variant of both directions on scratch batches of this ring (device memory from the
// stream-ordered pool, synchronising `s`) of 8, 32 and 640 limbs' worth of residues at N = 2^16 (tiny, small,
// large) and stores the fastest variant of each class in t.*_variant_tiny / *_small / *_variant.  The times in ms
// (forward tiny v0..v2, small v0..v2, large v0..v2, then the same for the inverse) are written to
// ms[0..2*3*3-1] when ms is non-null (-1 where a single kernel applies).
cudaError_t tune_ntt(DeviceTables& t, cudaStream_t s, float* ms);

// Job owning flattened row `row` of a prefix-sum table begin[0..njobs] (uniform per block / cluster).
__device__ __forceinline__ int find_job(const int* begin, int njobs, int row) {
  int lo = 0, hi = njobs;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (begin[mid] <= row) lo = mid; else hi = mid;
  }
  return lo;
}

// Convenience: appends a job; returns false when the batch is full.
inline bool ntt_add_job(NttBatch& b, const u64* src, u64* dst, long long src_stride, long long dst_stride, int limbs,
                        int npolys, const uint8_t* prime_of) {
  if (b.njobs >= kMaxNttJobs || limbs <= 0 || npolys <= 0) return limbs <= 0 || npolys <= 0;
  if (b.njobs == 0) b.limb_begin[0] = 0;
  b.limb_begin[b.njobs + 1] = b.limb_begin[b.njobs] + limbs * npolys;
  NttJob& j = b.jobs[b.njobs++];
  j.src = src;
  j.dst = dst;
  j.src_stride = src_stride;
  j.dst_stride = dst_stride;
  j.limbs = limbs;
  j.npolys = npolys;
  for (int k = 0; k < limbs; k++) j.prime_of[k] = prime_of[k];
  return true;
}

}  // namespace fgb
