// Host-side CKKS evaluation engine: context tables, device-resident ciphertexts and keys, op pipelines.
//
// Reference counterparts: FIDESlib::CKKS::ContextData (src/CKKS/Context.cuh:47-184), SetupConstants
// (src/ConstantsGPU.cu:125-697), Ciphertext::mult/rotate/rotate_hoisted/rescale (src/CKKS/Ciphertext.cpp)
// and LimbPartition::modup_ksk_moddown_mgpu (src/CKKS/LimbPartitionMGPU.cu:588-1870, single-GPU branch).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "arith.cuh"
#include "kernels.cuh"
#include "ntt.cuh"

namespace fgb {

struct DevCt {
  u64* data = nullptr;  // [2][t][N]
  int t = 0;            // active Q towers
  double scale = 0.0;   // scaling factor (RawCipherText::Noise)
  int noise_deg = 1;    // RawCipherText::NoiseLevel
  int slots = 0;
};

// Precomputed ModUp of a ciphertext's c1 (EvalFastRotationPrecompute): a copy of c1 (its own-digit towers are
// read from it) and the extended digits.
struct DevModUp {
  u64* c1 = nullptr;      // [t][N] evaluation form
  u64* digits = nullptr;  // [beta][t+np][N], modup()'s layout
  int t = 0;
};

struct DevPt {
  u64* data = nullptr;  // [t + prows][N] evaluation form
  int t = 0;
  double scale = 1.0;
  int prows = 0;  // special-prime rows after the t Q rows (np for an extended-basis plaintext, else 0)
};

// Baby-step / giant-step linear transform over the diagonals at slot offsets base + k*stride, k = g*bs + b:
//   out = sum_g rot_{base + g*bs*stride}( sum_b D[g*bs + b] (.) rot_{b*stride}(x) ).
// Diagonals are laid out contiguously [gs*bs][t][N]; D[g*bs + b] is the diagonal of offset base + k*stride
// already rotated by -(base + g*bs*stride) (the layout the reference's LT precomputation produces).
struct DevLT {
  u64* diags = nullptr;
  uint8_t* present_dev = nullptr;
  std::vector<uint8_t> present;
  int bs = 0, gs = 0, t = 0;
  int stride = 1, base = 0;
  bool ext = false;  // diagonals hold t + np rows (Q towers, then the special primes): double-hoisted evaluation
  int rows = 0;      // rows per diagonal: t, or t + np when ext
  double scale = 1.0;
  // slot-rotation indices the transform needs keys for (nonzero modulo N/2)
  std::vector<int32_t> baby_rotations(int N) const;
  std::vector<int32_t> giant_rotations(int N) const;
};

class Context {
 public:
  ~Context();
  // Creates tables on the current device.  `roots` may be null (generated as g^((p-1)/2N), smallest
  // generator g).  Returns an error string on failure.
  static Context* create(int logN, int nq, int np, int dnum, const u64* moduli, const u64* roots, std::string* err);

  int N = 0, logN = 0, nq = 0, np = 0, dnum = 0, alpha = 0, ntow = 0;
  int device = 0;  // the CUDA device current at creation; every call on the context runs on it
  std::vector<u64> mod, psi;
  cudaStream_t stream = nullptr;      // stream all work is ordered on
  cudaStream_t own_stream = nullptr;  // the context's own stream
  cudaStream_t copy_in = nullptr, copy_out = nullptr;  // copy streams of the pipelined host batch (lazily made)
  cudaStream_t chunk_alt = nullptr;  // compute stream of the pipelined host batch's odd chunks (lazily made)
  cudaStream_t side = nullptr;                         // second stream of split key-switch batches (lazily made)
  cudaEvent_t side_ev[2] = {nullptr, nullptr};

  DeviceTables tabs{};
  float ntt_tune_ms[kNttSizeClasses * (kNttFwdVariants + kNttInvVariants)] = {};  // tune_ntt timings
  // Key inner product tile (coefficient pairs per thread: 1, 2, 4, 8 or 16), tuned on the context's first
  // key-switch launch of at least kKsTuneJobs jobs; until then (and where a tile does not apply) ks_tune_ms holds -1.
  static constexpr int kKsTileVariants = 5;
  static constexpr int kKsTuneJobs = 16;
  float ks_tune_ms[kKsTileVariants] = {-1.f, -1.f, -1.f, -1.f, -1.f};
  bool ks_tuned = false;  // also set by fides_ctx_ks_tuning_set
  CrtTables crt{};
  PrimeConst* d_pc = nullptr;
  const ulonglong2* psi_brev = nullptr;  // [ntow][N] {psi^brev(i), shoup} in natural order (monomial products)

  // --- primitives on device memory ---
  cudaError_t ntt(const u64* src, u64* dst, int npolys, int limbs, int first_prime, long long poly_stride,
                  bool inverse, cudaStream_t s);

  // One key switch of `a` (evaluation form, t towers) with `key` ([2][dnum][ntow][N]).  Results
  // (ModDown(sum D b) + add0, ModDown(sum D a) + add1), permuted by the automorphism whose inverse Galois
  // element is galois_inv (1 = none), go to out [2][t][N]; out must not alias a, add0 or add1.
  struct KsReq {
    const u64* a;
    int t;
    const u64* key;
    const u64* add0;
    const u64* add1;
    u64* out;
    uint32_t galois_inv;
    const u64* digits = nullptr;  // precomputed ModUp of `a` (modup()'s conv layout); skips the ModUp
    // 1, 2: no ModDown; out ([2][t+np][N], extended basis Q_t ∪ P) = automorph(inner + lift), where the lift is
    // (P*add0, P*add1) on the Q rows (mode 1, add0 / add1 in Q_t layout) or add0 in the extended layout added to
    // poly 0 (mode 2, add1 unused).  Double hoisting (the linear transforms of bootstrapping).
    int ext_mode = 0;
  };
  // All requests in one pipeline: requests with the same (a, t) share one ModUp (hoisting).  Batches of at least
  // kKsSplit ordinary requests run as two halves on `s` and a side stream (64 rotations at ragged levels: +0.9%; 64
  // products at N=2^13: +4.6%), the requests ordered by key first so that each key's inner products fall in one
  // half and read the key once.
  cudaError_t keyswitch_batch(const KsReq* reqs, int n, cudaStream_t s);
  static constexpr int kKsSplit = 32;
  // ModDown of `polys` polys of x ([polys][t+np][N], extended basis, evaluation form) into out ([polys][t][N]).
  // x's special rows are left in coefficient form (used as scratch).
  struct MdReq {
    u64* x;
    int t;
    int polys;
    u64* out;
  };
  cudaError_t moddown_batch(const MdReq* reqs, int n, cudaStream_t s);
  // ModUp of ng inputs a[g] (t[g] towers, evaluation form): coeff[g] (t limbs) is scratch, conv[g] receives the
  // beta (t + np) limbs of extended digits (digit d at conv + d (t+np) N; its own towers are not written).
  cudaError_t modup(const u64* const* a, const int* ts, u64* const* coeff, u64* const* conv, int ng, cudaStream_t s);

  struct MultReq {
    const u64* x;
    const u64* y;
    int t;
    u64* out;
  };
  cudaError_t mult_batch(const MultReq* reqs, int n, const u64* rlk, cudaStream_t s);

  struct RescaleReq {
    const u64* x;
    int t;
    u64* out;
  };
  cudaError_t rescale_batch(const RescaleReq* reqs, int n, cudaStream_t s);

  struct AddReq {
    const u64* x;
    const u64* y;
    int t;
    u64* out;
    bool sub;
  };
  cudaError_t add_batch(const AddReq* reqs, int n, cudaStream_t s);

  // y = sum_g rot_{g*bs}( sum_b lt.diag[g*bs+b] (.) rot_b(x) ): baby-step rotations share one ModUp, the inner
  // sums are one pt-dot launch, the giant-step rotations one key-switch batch, the final sum one launch.
  cudaError_t linear_transform(const u64* x, int t, const DevLT& lt, u64* out, cudaStream_t s);
  // The same transform of n ciphertexts with t towers each, every stage batched over all of them.
  cudaError_t linear_transform_batch(const u64* const* xs, int n, int t, const DevLT& lt, u64* const* outs,
                                     cudaStream_t s);
  // The double-hoisted form for transforms whose diagonals carry the special primes (lt.ext): baby steps stay in
  // the extended basis Q_t ∪ P (no ModDown), the inner sums run there, each giant-step sum is ModDowned in c1
  // only before its rotation (which again skips the ModDown), and one ModDown of the total ends the transform.
  cudaError_t linear_transform_ext_batch(const u64* const* xs, int n, int t, const DevLT& lt, u64* const* outs,
                                         cudaStream_t s);
  cudaError_t mult_monomial(const u64* x, int t, unsigned k, u64* out, cudaStream_t s);
  // Raise a ciphertext's tower 0 to T towers (centred lift) — the first step of bootstrapping.
  cudaError_t mod_raise(const u64* x, int t_in, int T, u64* out, cudaStream_t s);

  // --- object registry (handles as in api/CryptoContext.hpp:233-246) ---
  std::mutex mu;
  std::unordered_map<uint32_t, DevCt> cts;
  std::unordered_map<uint32_t, DevCt> ext_cts;  // extended basis Q_t ∪ P: data [2][t+np][N]
  uint32_t next_handle = 1;
  std::map<uint32_t, u64*> rot_keys;  // Galois element -> key
  std::unordered_map<uint32_t, DevPt> pts;
  std::unordered_map<uint32_t, DevModUp> modups;
  std::unordered_map<uint32_t, DevLT> lts;
  u64* relin_key = nullptr;

  // Stream-ordered allocations of ciphertexts and workspaces from the context's own memory pool (created on its
  // device at build time, so the device's default pool and every other user of it keep their settings), counted
  // against mem_limit (0 = none).
  cudaMemPool_t pool = nullptr;
  // Opt-in validation of loaded residues (fides_ctx_set_input_check); d_bad is its device flag.
  bool input_check = false;
  int* d_bad = nullptr;
  // 0 when every residue of x ([rows][N], row r = tower r % period, see launch_range_check) is below its prime,
  // 1 when one is not, -1 on a CUDA error.  Synchronises the context stream.
  int residues_out_of_range(const u64* x, long long rows, int period, int tq);
  u64* alloc_limbs(size_t nlimbs, cudaStream_t s);
  void free_limbs(u64* p, cudaStream_t s);
  size_t mem_limit = 0, mem_in_use = 0;

  // Scaling technique (FIDES_FIXEDMANUAL .. FIDES_FLEXIBLEAUTOEXT) and its per-level tables, indexed by
  // towers - 1 (RawParams::ScalingFactorReal / ScalingFactorRealBig / ModReduceFactor, RawCiphertext.cuh:50-86).
  int technique = 0;
  std::vector<double> sf, big, mrf;
  // Sets the technique and its tables (null tables: computed as OpenFHE does for the technique); FIDES_OK or
  // FIDES_EINVAL with *err set.
  int set_scaling(int technique, const double* sf, const double* big, const double* mrf, double default_scale,
                  std::string* err);
  // Residues (towers 0..t-1) of the constant `operand` encoded at sf[t - 1] (ContextData::ElemForEvalMult).
  void eval_mult_constants(int t, double operand, u64* out) const;

  uint32_t galois_inverse(uint32_t g) const;
  static uint32_t galois_for_index(int N, int32_t index);
  // Galois element of the key a rotation by `index` of a ciphertext packing `slots` values uses, or 0 when no such
  // key is loaded (Ciphertext::normalyzeIndex + ContextData::GetRotationKey(index, keyID, slots, actual_index),
  // src/CKKS/Context.cu:591-619,1118-1125): with a sparse packing (0 < slots < N/2) the index is taken modulo slots
  // (the upper half as negative rotations) and, when no key exists for it, the first loaded key of an index
  // congruent to it modulo slots is used, as a rotation by any of them moves the packed values alike.  slots 0
  // (unknown) or N/2: the index modulo N/2.
  uint32_t rotation_key_galois(int32_t index, int slots) const;

 private:
  std::mutex mem_mu_;
  std::unordered_map<const void*, size_t> mem_sizes_;
  Context() = default;
  bool build(const u64* roots, std::string* err);
  // Key inner product tile: runs the inner products of kb once per tile (identical results), timed on s with CUDA
  // events, and sets crt.ks_iters to the fastest (ks_tune_ms holds the timings).  Synchronises with s once.
  cudaError_t tune_ks(const KsBatch& kb, cudaStream_t s);
  std::vector<void*> owned_;  // device allocations freed at destruction
  void* dmalloc(size_t bytes);
  // INTT of the special rows, ModDown conversion, NTT and epilogue for the jobs of kb (inner, md, out, t, polys,
  // add0 / add1, galois_inv set).
  cudaError_t moddown_jobs(const KsBatch& kb, cudaStream_t s);
  cudaError_t keyswitch_run(const KsReq* reqs, int n, cudaStream_t s);

  Ring ring_{};
};

}  // namespace fgb
