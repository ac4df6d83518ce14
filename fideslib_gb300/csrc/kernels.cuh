// Job-batched kernels of the CKKS evaluation pipeline (launchers).  Every launch carries up to kMaxJobs
// ciphertext jobs in kernel-parameter space, so a batch of ciphertexts at different levels is one launch per
// pipeline stage; rows beyond a job's tower count exit immediately.
#pragma once
#include <cuda_runtime.h>

#include <atomic>

#include "arith.cuh"

namespace fgb {

constexpr int kMaxJobs = 64;

// Programmatic dependent launch for latency-bound launches.  A pipeline kernel whose grid is smaller than the
// GPU's SM count is launched with the programmatic-serialization attribute (launch_pdl), so its CTAs are scheduled
// while the previous kernel of the same stream is still running instead of after it.  Every pipeline kernel
// starts with pdl_prologue(): griddepcontrol.wait blocks until the previous kernel has completed and its writes
// are visible (a no-op for a kernel launched without the attribute), then griddepcontrol.launch_dependents lets
// the next kernel be scheduled the same way.  Nothing is read or written before the wait, so the stream order of
// every memory access is unchanged.  Larger grids launch as before: with the attribute on every launch, one
// HMult + relinearise + Rescale at N = 2^13 went 0.115 -> 0.092 ms, but 64 of them batched lost 6%, hoisted
// rotations 4% and the bootstrap batch 3%.
__device__ __forceinline__ void pdl_prologue() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
// Whether a launch of `ctas` CTAs takes the programmatic-serialization attribute (fewer CTAs than the current
// device has SMs).
bool pdl_for(long long ctas);
template <typename... P, typename... A>
inline cudaError_t launch_pdl(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl_for((long long)grid.x * grid.y * grid.z) ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<A&&>(args)...);
}

// Runs `set` (a kernel attribute such as its dynamic shared-memory limit, which applies per device) once per device
// of the process; safe to call from several host threads.
template <class F>
inline cudaError_t once_per_device(std::atomic<unsigned long long>& done, F set) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const unsigned long long bit = 1ull << (dev & 63);
  if (done.load(std::memory_order_acquire) & bit) return cudaSuccess;
  e = set();
  if (e == cudaSuccess) done.fetch_or(bit, std::memory_order_acq_rel);
  return e;
}

// CRT tables resident on the device (built once per context, Context::build).
struct CrtTables {
  int nq, np, alpha, dnum, ntow;
  int ks_iters;  // coefficient pairs per thread of the key inner product (power of two; 0 = 4), picked by tune_ks
  // ModUp, digit d with s towers: base b = (d*alpha + s-1)*alpha
  const ulonglong2* mu_qhinv;  // [b + i] = {[Qhat_i^-1]_{q_i}, shoup}
  const uint32_t* mu_qhat;     // [((b + i)*ntow + tower)*2 + {0,1}] = 30-bit slices (lo, hi) of [Qhat_i]_{m_tower}
  // ModDown
  const ulonglong2* md_phinv;  // [k] = {[Phat_k^-1]_{p_k}, shoup}
  const uint32_t* md_phat;     // [(k*nq + j)*2 + {0,1}] = 30-bit slices of [Phat_k]_{q_j}
  const ulonglong2* md_pinv;   // [j] = {[P^-1]_{q_j}, shoup}
  const ulonglong2* md_pmodq;  // [j] = {[P]_{q_j}, shoup} (lifting Q-basis values into the extended basis)
  // Rescale: top tower l, target i < l
  const ulonglong2* rs_qinv;   // [l*nq + i] = {[q_l^-1]_{q_i}, shoup}
};

struct Ring {
  int N, logN;
};

// One key switch: ModUp(a) (shared by jobs with the same input), inner product with `key`, ModDown of both
// halves, + add0/add1, automorphism scatter by galois_inv (1 = none) into out.
// ext_mode 1 / 2 (double hoisting) skips the ModDown: out = automorph(inner + add) stays in the extended basis
// Q_t ∪ P ([2][t+np][N]); mode 1 adds P*add0 (and P*add1) on the Q rows (add0 / add1 in Q_t layout), mode 2 adds
// add0 given in the extended layout to poly 0.  A ModDown-only job (moddown_batch) has polys = 1 or 2.
struct KsJob {
  const u64* a;      // [t][N] evaluation form (the digit's own towers are read from here)
  const u64* add0;   // [t][N] or null
  const u64* add1;   // [t][N] or null
  const u64* key;    // [2][dnum][ntow][N] (0 = a vectors, 1 = b vectors), split form (launch_key_split)
  const u64* coeff;  // [t][N] coefficient form of a (ModUp input)
  u64* conv;         // digit d: conv + d*(t+np)*N, rows = the t - s_d + np converted towers
  u64* inner;        // [2][t+np][N]
  u64* md;           // [2][t][N]
  u64* out;          // [2][t][N]
  int t;
  uint32_t galois_inv;
  int polys;     // polys the ModDown kernels process (0 means 2)
  int ext_mode;  // 0: ModDown output; 1, 2: extended output (see above)
};

struct KsBatch {
  int njobs;
  int row_begin[kMaxJobs + 1];  // filled by each launcher: prefix sums of that kernel's rows per job (per key
                                // group for the key inner product)
  int ngroups;                  // key inner product: jobs grp_begin[g] .. grp_begin[g+1]-1 share one key
  int grp_begin[kMaxJobs + 1];
  int row_outer;                // key inner product: block rows ordered (tower row, job) instead of (group, row, job)
  KsJob jobs[kMaxJobs];
};

// x, y: [2][t][N] -> d: [3][t][N] = (x0y0, x0y1 + x1y0, x1y1)
struct TensorJob {
  const u64* x;
  const u64* y;
  u64* d;
  int t;
};
struct TensorBatch {
  int njobs;
  int row_begin[kMaxJobs + 1];  // filled by each launcher: prefix sums of that kernel's rows per job
  TensorJob jobs[kMaxJobs];
};

// out = x +/- y over [2][t][N]
struct AddJob {
  const u64* x;
  const u64* y;
  u64* out;
  int t;
  int sub;
};
struct AddBatch {
  int njobs;
  int row_begin[kMaxJobs + 1];  // filled by each launcher: prefix sums of that kernel's rows per job
  AddJob jobs[kMaxJobs];
};

// Plaintext op on [2][t][N]: mode 0 = multiply both polys by pt, 1 = c0 + pt, 2 = c0 - pt (c1 copied).
struct PtJob {
  const u64* ct;
  const u64* pt;  // [t][N]
  u64* out;
  int t;
  int mode;
};
struct PtBatch {
  int njobs;
  int row_begin[kMaxJobs + 1];
  PtJob jobs[kMaxJobs];
};

// out[p][j] = ct[p][j] * mul[j] (+ add[j] on poly 0) with the per-tower constants of the job's set; several
// jobs may share one set (the many-to-one form: one scalar applied to a group of ciphertexts).
constexpr int kMaxScalarSets = 8;
struct ScalarSet {
  u64 mul[64];
  u64 mul_sh[64];
  u64 add[64];
};
struct ScalarJob {
  const u64* ct;
  u64* out;
  int t;
  int set;
};
struct ScalarBatch {
  int njobs;
  int row_begin[kMaxJobs + 1];
  ScalarJob jobs[kMaxJobs];
  ScalarSet sets[kMaxScalarSets];
};

// Weighted sums out = sum_k mul[k][j] * term_k over [2][t][N] (term k laid out [2][term_t[k]][N], rows j < t read),
// one constant set shared by every job of the launch; accumulate != 0 adds the sum to what out holds.
constexpr int kMaxWsumTerms = 8;
struct WsumSet {
  u64 mul[kMaxWsumTerms][64];
  u64 mul_sh[kMaxWsumTerms][64];
};
struct WsumJob {
  const u64* term[kMaxWsumTerms];
  int term_t[kMaxWsumTerms];
  u64* out;
  int t;
};
struct WsumBatch {
  int njobs;
  int nterms;
  int accumulate;
  int row_begin[kMaxJobs + 1];
  WsumJob jobs[kMaxJobs];
  WsumSet set;
};

// Baby-step/giant-step inner sums: job (x, g, ng) writes, for the giant steps g .. g+ng-1,
// out + k*out_stride ([2][rows][N]) = sum_{b<bs, present} rot[b] (.) pt[(g+k)*bs+b] with rot[0] = rot0 (the input
// itself), rot[b] = rot_base + (b-1)*rot_stride ([2][rows][N] each) and pt[i] = pt_base + i*pt_stride.  One thread
// reads each rot[b] value once for all ng giant steps (ng <= kDotG, bs <= 16); rows = t (+ np).  pmask bit
// k*16 + b marks diagonal (g+k)*bs + b present (filled by launch_ptdot from `present`).
constexpr int kDotG = 4;
struct DotJob {
  u64* out;
  const u64* rot0;
  const u64* rot_base;
  int g;
  int ng;
  unsigned long long pmask;
};
struct DotBatch {
  int njobs;
  int row_begin[kMaxJobs + 1];
  long long rot_stride;
  long long out_stride;
  const u64* pt_base;
  long long pt_stride;
  const uint8_t* present;  // host [gs*bs] (read by launch_ptdot)
  int bs, t;
  // extended basis (np > 0): ciphertexts are [2][t+np][N], row t+k is special prime nq+k and reads plaintext
  // row pt_prow+k
  int np, nq, pt_prow;
  DotJob jobs[kMaxJobs];
};

// out = sum_k in[k] over [2][t][N] (in[k] = base + k*stride), k < n.
struct SumJob {
  const u64* base;
  long long stride;
  int n;
  const u64* first;  // added too when non-null
  u64* out;
  int t;
  int np;  // rows t..t+np-1 are the special primes (extended-basis sums), else 0
};
struct SumBatch {
  int nq;
  int njobs;
  int row_begin[kMaxJobs + 1];
  SumJob jobs[kMaxJobs];
};

// ModRaise: top [2][N] = coefficient form of tower 0 (mod q_0); tmp [2][T][N] <- centred lift into towers 0..T-1.
struct RaiseJob {
  const u64* top;
  u64* tmp;
  int T;
};
struct RaiseBatch {
  int njobs;
  int row_begin[kMaxJobs + 1];
  RaiseJob jobs[kMaxJobs];
};

// out[p][j][i] = ct[p][j][i] * X^k evaluated at the i-th evaluation point psi^(2 brev(i) + 1): multiplication by
// the monomial X^k, 0 <= k < 2N, done pointwise in the evaluation domain (twiddles {psi^brev(e), shoup}).
struct MonoJob {
  const u64* ct;
  u64* out;
  int t;
  unsigned k;
};
struct MonoBatch {
  int njobs;
  int row_begin[kMaxJobs + 1];
  MonoJob jobs[kMaxJobs];
};

cudaError_t launch_ptop(const PtBatch& b, const Ring& r, const PrimeConst* pc, cudaStream_t s);
cudaError_t launch_scalar(const ScalarBatch& b, const Ring& r, const PrimeConst* pc, cudaStream_t s);
cudaError_t launch_ptdot(const DotBatch& b, const Ring& r, const PrimeConst* pc, cudaStream_t s);
cudaError_t launch_wsum(const WsumBatch& b, const Ring& r, const PrimeConst* pc, cudaStream_t s);
cudaError_t launch_sum(const SumBatch& b, const Ring& r, const PrimeConst* pc, cudaStream_t s);
cudaError_t launch_raise_switch(const RaiseBatch& b, const Ring& r, const PrimeConst* pc, cudaStream_t s);
cudaError_t launch_monomial(const MonoBatch& b, const Ring& r, const PrimeConst* pc, const ulonglong2* tw_fwd,
                            cudaStream_t s);

cudaError_t launch_modup_conv(const KsBatch& b, const Ring& r, const CrtTables& c, const PrimeConst* pc,
                              cudaStream_t s);
cudaError_t launch_ks_inner(const KsBatch& b, const Ring& r, const CrtTables& c, const PrimeConst* pc,
                            cudaStream_t s);
cudaError_t launch_moddown_conv(const KsBatch& b, const Ring& r, const CrtTables& c, const PrimeConst* pc,
                                cudaStream_t s);
cudaError_t launch_moddown_epilogue(const KsBatch& b, const Ring& r, const CrtTables& c, const PrimeConst* pc,
                                    cudaStream_t s);
cudaError_t launch_ext_epilogue(const KsBatch& b, const Ring& r, const CrtTables& c, const PrimeConst* pc,
                                cudaStream_t s);
// Sets *bad (device int) when a residue of x ([rows][N]) is not below its prime: row r is tower j = r % period,
// prime j for j < tq, else nq + (j - tq).
cudaError_t launch_range_check(const u64* x, long long rows, int logN, int period, int tq, int nq,
                               const PrimeConst* pc, int* bad, cudaStream_t s);
// In place: every key residue k becomes (k mod 2^30) | (floor(k / 2^30) << 32), the form ks_inner_kernel reads.
cudaError_t launch_key_split(u64* key, size_t n, cudaStream_t s);
cudaError_t launch_tensor(const TensorBatch& b, const Ring& r, int nq, const PrimeConst* pc, cudaStream_t s);
cudaError_t launch_addsub(const AddBatch& b, const Ring& r, int nq, const PrimeConst* pc, cudaStream_t s);

}  // namespace fgb
