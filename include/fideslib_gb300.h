/*
 * fideslib_gb300 — C ABI of the GB300 CKKS evaluation engine.
 *
 * Plain pointers, sizes and integer status codes; no C++ types, no exceptions and no process exit cross
 * this boundary.  Every function returns FIDES_OK (0) or a negative FIDES_E* code; fides_last_error()
 * gives the message of the calling thread's last failure.
 *
 * Data contract (the one FIDESlib's OpenFHE interop extracts, src/CKKS/openfhe-interface/RawCiphertext.cuh:
 * 19-93):
 *   - residues are uint64 in [0, q), evaluation (NTT, bit-reversed) format, exactly the layout of
 *     RawCipherText::sub_0 / sub_1 (RawCiphertext.cu:55-64);
 *   - a ciphertext with t active towers (OpenFHE level = nq - t) is host memory u64[2][t][N];
 *   - a key-switching key is u64[2][dnum][nq+np][N], index 0 = the "a" vectors, 1 = the "b" vectors, as in
 *     RawKeySwitchKey::r_key (RawCiphertext.cu:650-666);
 *   - moduli are the nq Q primes followed by the np special primes, each prime < 2^60 and == 1 mod 2N.
 * Ownership: the engine owns device memory behind opaque uint32 handles (0 is never a valid handle), the
 * caller owns every host buffer.  A context is used by one host thread at a time.
 */
#ifndef FIDESLIB_GB300_H
#define FIDESLIB_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  FIDES_OK = 0,
  FIDES_EINVAL = -1,    /* bad argument (sizes, handles, parameters) */
  FIDES_ENOKEY = -2,    /* no relinearisation / rotation key loaded for the request */
  FIDES_ENOMEM = -3,    /* device allocation failed */
  FIDES_ECUDA = -4,     /* CUDA runtime error */
  FIDES_ENODEV = -5     /* no usable CUDA device */
};

/* Scaling technique tags, same values as lbcrypto::ScalingTechnique used by Parameters::scalingTechnique
 * (src/CKKS/Parameters.cuh:27). */
enum { FIDES_FIXEDMANUAL = 0, FIDES_FIXEDAUTO = 1, FIDES_FLEXIBLEAUTO = 2, FIDES_FLEXIBLEAUTOEXT = 3 };

typedef struct fides_ctx fides_ctx;

/* Replaces RawParams + FIDESlib::CKKS::Parameters::adaptTo + GenCryptoContextGPU
 * (src/CKKS/openfhe-interface/RawCiphertext.cuh:50-86, src/CKKS/Parameters.cu:7-34, src/CKKS/Context.cu:36-86). */
typedef struct {
  uint32_t log_n;           /* ring dimension N = 2^log_n, 10 <= log_n <= 16 */
  uint32_t nq;              /* Q towers (OpenFHE L + 1) */
  uint32_t np;              /* special towers K */
  uint32_t dnum;            /* key-switching digits; towers per digit alpha = ceil(nq / dnum) */
  const uint64_t* moduli;   /* nq + np primes */
  const uint64_t* roots;    /* nq + np primitive 2N-th roots (RawParams::root_of_unity); NULL = generated */
  /* FIDES_FIXEDMANUAL: operands of an addition or multiplication at different tower counts are cut to the lower
   * count, nothing else is adjusted.  FIDES_FIXEDAUTO / FIDES_FLEXIBLEAUTO / FIDES_FLEXIBLEAUTOEXT: before
   * fides_eval_add / sub / mult / square (and their fides_eval_batch requests) the operands are rescaled, multiplied
   * by scale-correcting constants and cut down to one level and scale exactly as Ciphertext::adjustForAddOrSub /
   * adjustForMult do (src/CKKS/Ciphertext.cpp:1376-1518); a degree-2 operand of a square or of a plaintext
   * product is rescaled first (Ciphertext::square, multPt).  Scalar ops encode at the scale the caller passes. */
  int32_t scaling_technique;
  /* Per-level tables of RawParams (ScalingFactorReal, ScalingFactorRealBig, ModReduceFactor,
   * RawCiphertext.cuh:50-86), nq entries each, indexed by towers - 1.  NULL = computed for the technique:
   * FIXED*: every level default_scale (0 = 2^round(log2 q_{nq-1})); FLEXIBLEAUTO: sf[nq-1] = q_{nq-1},
   * sf[l] = sf[l+1]^2 / q_{l+1}; FLEXIBLEAUTOEXT: sf[nq-1] = sf[nq-2] = q_{nq-2}, then the same recursion;
   * big[l] = sf[l]^2 (FLEXIBLEAUTOEXT top level: sf[nq-1] sf[nq-2]); mod_reduce[l] = q_l. */
  const double* scaling_factor_real;
  const double* scaling_factor_real_big;
  const double* mod_reduce_factor;
  double default_scale;
} fides_params;

/* Ciphertext metadata (RawCipherText::Noise / NoiseLevel / slots, RawCiphertext.cuh:28-31). */
typedef struct {
  uint32_t towers;          /* active Q towers t */
  uint32_t noise_deg;       /* noise scale degree */
  uint32_t slots;
  uint32_t reserved;        /* fides_ct_meta_get: the special rows of an extended-basis ciphertext (else 0) */
  double scale;             /* scaling factor */
} fides_ct_meta;

const char* fides_last_error(void);
const char* fides_version(void);

/* Parameter helper (the role of OpenFHE's FirstPrime/PreviousPrime in GenCryptoContext): the `count` largest
 * primes below 2^bits that are == 1 mod two_n, skipping `exclude`.  Returns the number found. */
int fides_find_primes(uint32_t bits, uint32_t count, uint64_t two_n, const uint64_t* exclude, uint32_t nexclude,
                      uint64_t* out);

/* Context (LoadContext, api/CryptoContext.cpp:199-249).  The context lives on the CUDA device current when it is
 * created; make that device current in any other host thread that calls into it (fides_server_create records it
 * for its worker thread). */
int fides_ctx_create(const fides_params* params, fides_ctx** out);
int fides_ctx_destroy(fides_ctx* ctx);
/* The scaling technique and its per-level tables in use (nq entries each, indexed by towers - 1; NULL skips). */
int fides_ctx_scaling(const fides_ctx* ctx, int32_t* technique, double* scaling_factor_real,
                      double* scaling_factor_real_big, double* mod_reduce_factor);
/* The moduli and primitive 2N-th roots actually used (nq + np entries each). */
int fides_ctx_moduli(const fides_ctx* ctx, uint64_t* moduli, uint64_t* roots);
/* Galois element 5^index mod 2N (2N-1 for conjugation), FindAutomorphismIndex2nComplex semantics. */
uint32_t fides_galois_element(const fides_ctx* ctx, int32_t index);
/* Blocks until all queued device work of the context finished (CryptoContextImpl::Synchronize,
 * api/CryptoContext.hpp:201). */
int fides_synchronize(fides_ctx* ctx);
/* The cudaStream_t the context orders its work on, and a way to replace it with a caller's stream (NULL
 * restores the context's own).  FIDESlib exposes its per-limb streams the same way through
 * LimbPartition / Stream (src/CudaUtils.cuh:98-160). */
void* fides_ctx_stream(fides_ctx* ctx);
int fides_ctx_set_stream(fides_ctx* ctx, void* stream);
/* The NTT autotuner's choices for this ring (no counterpart in the reference, whose NTT kernels are fixed at build
 * time): at context creation every forward and inverse kernel variant is timed on a tiny, a small and a large
 * scratch batch (8, 32 and 640 limbs' worth of residues at N = 2^16) and the fastest one of each is used for
 * launches of at most 16 limbs' worth (one op: latency-bound), at most 128 limbs' worth and more (batches).
 * variant[0..5] = forward tiny, small, large, inverse tiny, small, large; forward variants: 0 = radix-16 passes
 * with 8192 residues per CTA, 1 = radix-32/16 passes, 2 = radix-16 passes with 4096 residues per CTA (twice the
 * CTAs per limb); inverse: 0 = radix-32/16, 1 = radix-16 with 4096 per CTA, 2 = radix-16 with 8192 per CTA.
 * ms[0..17] = forward tiny v0..v2, small v0..v2, large v0..v2, then the inverse the same way (-1 where a single
 * kernel applies, N < 2^13).  The key switch's inverse launches of the large class run beside the other half of
 * their batch on a second stream and use the faster of inverse variants 1 and 2 (ms[16], ms[17]), whose CTAs share
 * an SM three at a time; fides_ctx_ntt_tuning_set fixes them too. */
int fides_ctx_ntt_tuning(fides_ctx* ctx, int32_t* variant, float* ms);
/* Device-memory budget of the context (the reference's pool has a release threshold only, Context.cu:74-80):
 * ciphertexts and per-op workspaces come from the stream-ordered pool and are counted; an op whose allocation
 * would exceed `bytes` fails with FIDES_ENOMEM and leaves the context usable (0 = no limit; keys, plaintexts and
 * transforms are not counted).  fides_ctx_mem_in_use reports the bytes currently counted. */
int fides_ctx_set_mem_limit(fides_ctx* ctx, uint64_t bytes);
int fides_ctx_mem_in_use(fides_ctx* ctx, uint64_t* bytes);
/* Opt-in validation of loaded residues (no counterpart in the reference, which copies them unchecked): while
 * enabled, fides_ct_load*, fides_pt_load* and the key loaders check that every residue is below its tower's prime
 * and refuse the object with FIDES_EINVAL otherwise (a refused key is unloaded, also one previously loaded under the
 * same name).  The kernels' lazy-reduction bounds assume residues in [0, q); out-of-range input otherwise gives
 * wrong results silently.  Costs one extra read of the object and a synchronisation per load. */
int fides_ctx_set_input_check(fides_ctx* ctx, int enable);
/* Overrides the autotuner's choices for every batch size (all variants give identical residues). */
int fides_ctx_ntt_tuning_set(fides_ctx* ctx, int32_t fwd_variant, int32_t inv_variant);
/* The key inner product's tile (no counterpart in the reference, whose fusedDotKSK_2_ launch shape is fixed,
 * src/CKKS/LimbPartitionMGPU.cu:444): the coefficient pairs each thread takes (1, 2, 4, 8 or 16, at most N / 512).
 * The context's first key-switch launch of at least 16 ciphertexts runs its inner products once per tile, timed
 * with CUDA events (one synchronisation), and keeps the fastest.  iters = the tile in use (4 before that launch),
 * ms[0..4] = the timings of 1, 2, 4, 8 and 16 (-1 before the tuning or where a tile does not apply).
 * fides_ctx_ks_tuning_set sets the tile and turns the tuning off (every tile gives identical residues). */
int fides_ctx_ks_tuning(fides_ctx* ctx, int32_t* iters, float* ms);
int fides_ctx_ks_tuning_set(fides_ctx* ctx, int32_t iters);
/* Ring and basis shape of a context. */
typedef struct {
  uint32_t n, log_n, nq, np, dnum, alpha;
} fides_ctx_shape;
int fides_ctx_get_shape(const fides_ctx* ctx, fides_ctx_shape* shape);
/* Number of engine kernels launched by this process so far (all contexts). */
uint64_t fides_kernel_launches(void);
/* Diagnostic (no counterpart in the reference): throughput of the units that bound the engine's kernels, measured
 * on the current device with register-only kernels — 32-bit multiply-add and 32x32->64 multiply-add lanes per
 * clock per SM, forward NTT butterflies (the engine's Shoup product and lazy reductions) per clock per SM, the
 * legacy mma.sync INT8 tensor rate (tcgen05 has no INT8 form on sm_103a), and the spacing of back-to-back launches.
 * Per-clock figures use the device's peak SM clock. */
typedef struct {
  uint32_t sms;
  double clock_mhz;
  double imad32_per_clk_sm, imad_wide_per_clk_sm, butterflies_per_clk_sm;
  double int8_mma_tops;     /* tera int8 ops (2 per multiply-add) per second */
  double launch_spacing_us; /* back-to-back empty launches (64 CTAs), GPU time per launch */
} fides_probe_result;
int fides_probe_pipes(fides_probe_result* r);

/* Batched negacyclic NTT (inverse = 0: coefficient -> evaluation, bit-reversed) or INTT on `npolys`
 * polynomials of `limbs` towers each, tower j using prime first_prime + j.  Device memory, in place,
 * ordered on `stream` (a cudaStream_t; NULL = the context stream).  Replaces the batched NTT_/INTT_
 * launches of LimbPartition::NTT / INTT (src/CKKS/LimbPartition.cu:332-421).  `data` must be 16-byte aligned. */
int fides_ntt_batch_device(fides_ctx* ctx, uint64_t* data, uint32_t npolys, uint32_t limbs, uint32_t first_prime,
                           int inverse, void* stream);
/* Same from host memory: copies in, transforms, copies back, synchronises. */
int fides_ntt_batch_host(fides_ctx* ctx, uint64_t* data, uint32_t npolys, uint32_t limbs, uint32_t first_prime,
                         int inverse);

/* Keys (KeySwitchingKey::Initialize via GetEvalKeySwitchKey / GetRotationKeySwitchKey,
 * src/CKKS/KeySwitchingKey.cu:19-34, RawCiphertext.cu:672-760).  The rotation key is registered under its
 * Galois element. */
int fides_load_eval_mult_key(fides_ctx* ctx, const uint64_t* key);
int fides_load_eval_mult_key_device(fides_ctx* ctx, const uint64_t* dev_key);
int fides_load_rotation_key(fides_ctx* ctx, uint32_t galois, const uint64_t* key);
int fides_load_rotation_key_device(fides_ctx* ctx, uint32_t galois, const uint64_t* dev_key);
/* A key switching from one secret to another (same layout; key_id < 2^31 is the caller's name for it): the
 * secret-switching keys of sparse-secret encapsulation (GetSecretSwitchingKey, src/CKKS/Context.cu:1091, used by
 * src/CKKS/Bootstrap.cu:254-262 and 592-600). */
int fides_load_switch_key(fides_ctx* ctx, uint32_t key_id, const uint64_t* key);
int fides_load_switch_key_device(fides_ctx* ctx, uint32_t key_id, const uint64_t* dev_key);

/* Ciphertexts (LoadCiphertext / GetOpenFHECipherText, api/CryptoContext.cpp:270-289,
 * RawCiphertext.cu:47-129). */
int fides_ct_load(fides_ctx* ctx, const uint64_t* data, const fides_ct_meta* meta, uint32_t* handle);
int fides_ct_load_device(fides_ctx* ctx, const uint64_t* dev_data, const fides_ct_meta* meta, uint32_t* handle);
int fides_ct_store(fides_ctx* ctx, uint32_t handle, uint64_t* data, fides_ct_meta* meta);
int fides_ct_meta_get(fides_ctx* ctx, uint32_t handle, fides_ct_meta* meta);
int fides_ct_free(fides_ctx* ctx, uint32_t handle);

/* Evaluation (api/CryptoContext.cpp EvalAdd/EvalSub, EvalMult 1185-1210, EvalSquare, Rescale 1669-1712,
 * EvalRotate 1406-1430, EvalFastRotation 1451-1617).  Results are new handles. */
int fides_eval_add(fides_ctx* ctx, uint32_t a, uint32_t b, uint32_t* out);
int fides_eval_sub(fides_ctx* ctx, uint32_t a, uint32_t b, uint32_t* out);
int fides_eval_mult(fides_ctx* ctx, uint32_t a, uint32_t b, uint32_t* out);
int fides_eval_square(fides_ctx* ctx, uint32_t a, uint32_t* out);
int fides_rescale(fides_ctx* ctx, uint32_t a, uint32_t* out);
int fides_eval_rotate(fides_ctx* ctx, uint32_t a, int32_t index, uint32_t* out);
int fides_eval_automorphism(fides_ctx* ctx, uint32_t a, uint32_t galois, uint32_t* out);
/* Key switch with a key loaded by fides_load_switch_key (Ciphertext::keySwitch, src/CKKS/Ciphertext.cpp:1354). */
int fides_eval_key_switch(fides_ctx* ctx, uint32_t a, uint32_t key_id, uint32_t* out);
int fides_eval_fast_rotation(fides_ctx* ctx, uint32_t a, uint32_t n, const int32_t* indices, uint32_t* outs);
/* EvalFastRotationPrecompute (api/CryptoContext.hpp:169): the ModUp of a's c1, kept on the device under a handle
 * (a copy of c1 is kept with it, so `a` may change or be freed afterwards). */
int fides_fast_rotation_precompute(fides_ctx* ctx, uint32_t a, uint32_t* pre);
/* EvalFastRotation(ct, index, m, precomp) (api/CryptoContext.hpp:170): the rotation of `a` by `index` from the
 * precomputed digits; `a` must be the ciphertext the digits were computed from (same residues).  Same result as
 * fides_eval_rotate. */
int fides_eval_fast_rotation_precomputed(fides_ctx* ctx, uint32_t a, uint32_t pre, int32_t index, uint32_t* out);
int fides_precompute_free(fides_ctx* ctx, uint32_t pre);
/* Extended-basis ciphertexts, u64[2][t+np][N] over Q_t ∪ P (the key-switch output before its ModDown), for
 * hoisted linear maps with one ModDown at the end:
 *   EvalFastRotationExt (api/CryptoContext.cpp:1497-1526, 1575-1617; OpenFHE KeySwitchHYBRID::EvalFastRotationExt):
 *     per index, the inner product of the digits of c1 (`pre` from fides_fast_rotation_precompute, or 0 to ModUp
 *     here once for all indices) with the rotation key, plus P*c0 on the Q rows when add_first, then the
 *     automorphism; index 0 gives (add_first ? P*c0 : 0, P*c1).  Handles go to outs[n] (free with fides_ct_free).
 *   fides_ext_add: sum of two extended ciphertexts with the same towers.
 *   fides_pt_load_ext + fides_ext_mult_plain: product with a plaintext given at the towers Q rows and the np special
 *     rows (u64[towers+np][N], towers >= the ciphertext's), the extended plaintexts of OpenFHE's hoisted
 *     EvalLinearTransform; the scale is multiplied.
 *   fides_key_switch_down (OpenFHE KeySwitchDown): ModDown of both polys, a regular ciphertext again.
 *   fides_ext_store: u64[2][t+np][N] to host memory. */
int fides_eval_fast_rotation_ext(fides_ctx* ctx, uint32_t a, uint32_t pre, uint32_t n, const int32_t* indices,
                                 int32_t add_first, uint32_t* outs);
int fides_ext_add(fides_ctx* ctx, uint32_t a, uint32_t b, uint32_t* out);
int fides_pt_load_ext(fides_ctx* ctx, const uint64_t* data, uint32_t towers, double scale, uint32_t* handle);
int fides_ext_mult_plain(fides_ctx* ctx, uint32_t a, uint32_t pt, uint32_t* out);
int fides_key_switch_down(fides_ctx* ctx, uint32_t a, uint32_t* out);
int fides_ext_store(fides_ctx* ctx, uint32_t h, uint64_t* data, fides_ct_meta* meta);

/* Plaintexts (RawPlainText / LoadPlaintext, RawCiphertext.cuh:37-48, api/CryptoContext.cpp:250-269):
 * u64[towers][N] evaluation form at scaling factor `scale`. */
int fides_pt_load(fides_ctx* ctx, const uint64_t* data, uint32_t towers, double scale, uint32_t* handle);
int fides_pt_free(fides_ctx* ctx, uint32_t handle);
/* EvalMult / EvalAdd / EvalSub with a plaintext (multPt / addPt: LimbPartition.cu:654-691,
 * src/AddSub.cu); the product's scale is the product of scales. */
int fides_eval_mult_plain(fides_ctx* ctx, uint32_t a, uint32_t pt, uint32_t* out);
int fides_eval_add_plain(fides_ctx* ctx, uint32_t a, uint32_t pt, uint32_t* out);
int fides_eval_sub_plain(fides_ctx* ctx, uint32_t a, uint32_t pt, uint32_t* out);
/* Multiplication by an integer (multIntScalar, src/CKKS/ApproxModEval.cu:131-136): scale unchanged. */
int fides_eval_mult_int(fides_ctx* ctx, uint32_t a, int64_t k, uint32_t* out);
/* Multiplication by a real constant encoded as round(v * scale) (EvalMult(ct, double)): scale *= scale. */
int fides_eval_mult_scalar(fides_ctx* ctx, uint32_t a, double v, double scale, uint32_t* out);
/* Adds v in every slot: round(v * ct scale) added to c0 (EvalAdd(ct, double), src/AddSub.cu scalar_add_). */
int fides_eval_add_scalar(fides_ctx* ctx, uint32_t a, double v, uint32_t* out);
/* Batched many-to-one form of the element-wise ops (addBatchManyToOne, multPtBatchManyToOne,
 * addScalarBatchManyToOne, multScalarBatchManyToOne: src/CKKS/LimbPartitionBatch.cu:20-266,
 * src/CKKS/RNSPolyBatch.cpp:15-80): for i < nb and j < stride, ciphertext a[i*stride + j] is combined with
 * operand i, all nb*stride ciphertexts (each at its own level) in one launch per 64.  `op` and operand i:
 *   FIDES_OP_ADD / FIDES_OP_SUB               b[i], a ciphertext with the same towers as its group
 *   FIDES_OP_MULT_PLAIN / ADD_PLAIN / SUB_PLAIN   b[i], a plaintext with at least as many towers
 *   FIDES_OP_MULT_SCALAR  round(values[i] * scales[i]); the result's scale is multiplied by scales[i]
 *   FIDES_OP_ADD_SCALAR   values[i] in every slot (round(values[i] * ct scale) added to c0)
 *   FIDES_OP_MULT_INT     the integer values[i] (|values[i]| < 2^53); scale unchanged
 * outs (nb*stride handles) receives new ciphertexts; outs == NULL updates the a ciphertexts in place, as the
 * reference does (their handles stay valid, metadata updated; no handle may repeat in `a`). */
enum { FIDES_OP_MULT_SCALAR = 13, FIDES_OP_ADD_SCALAR = 14, FIDES_OP_MULT_INT = 15 };
int fides_eval_many_to_one(fides_ctx* ctx, int32_t op, uint32_t nb, uint32_t stride, const uint32_t* a,
                           const uint32_t* b, const double* values, const double* scales, uint32_t* outs);
/* Weighted sum of ciphertexts, m sums in lock step (Ciphertext::evalLinearWSumMutable, src/CKKS/Ciphertext.cpp:
 * 1171-1212, as the reference's Chebyshev evaluation uses it, src/CKKS/ApproxModEval.cu:213,255,328): for i < m,
 *   outs[i] = sum_{k < n_terms} round(weights[k] * scales[k*m + i]) * cts[k*m + i]
 * on the smallest tower count among element i's terms, in one launch per 64 sums (one kernel pass reading each term
 * once).  Every term must have noise degree 1; the result has noise degree 2 and the scale of its first term times
 * scales[i] (the caller chooses the scales so that all terms land on that scale).  n_terms <= 16. */
int fides_eval_linear_wsum(fides_ctx* ctx, uint32_t m, uint32_t n_terms, const uint32_t* cts, const double* weights,
                           const double* scales, uint32_t* outs);
/* Keeps the first `towers` towers (LevelReduce / SetLevel, api/CryptoContext.hpp:184). */
int fides_level_reduce(fides_ctx* ctx, uint32_t a, uint32_t towers, uint32_t* out);
/* ModRaise (src/CKKS/Bootstrap.cu:393-...): tower 0 of `a`, lifted (centred) to `towers` towers. */
int fides_mod_raise(fides_ctx* ctx, uint32_t a, uint32_t towers, uint32_t* out);
/* Baby-step/giant-step linear transform (EvalLinearTransform, src/CKKS/LinearTransform.cu:63-256):
 * diags = u64[gs*bs][towers][N] evaluation form, diagonal i = g*bs + b already rotated by -g*bs;
 * present[i] = 0 marks a zero diagonal; 1 <= bs <= 16, gs <= 64.  Needs rotation keys for 1..bs-1 and for g*bs.
 * `diags` may be host or device memory (copied into the transform). */
int fides_lt_create(fides_ctx* ctx, uint32_t bs, uint32_t gs, uint32_t towers, const uint64_t* diags,
                    const uint8_t* present, double scale, uint32_t* handle);
/* The same over the diagonals at slot offsets base + k*stride (k = g*bs + b), the form of one level of a
 * factored CoeffsToSlots / SlotsToCoeffs (LinearTransform(ct, rowSize, bStep, pts, stride, offset),
 * src/CKKS/LinearTransform.cu:63; EvalCoeffsToSlots level steps, src/CKKS/CoeffsToSlots.cu:98-150):
 *   out = sum_g rot_{base + g*bs*stride}( sum_b D[g*bs + b] (.) rot_{b*stride}(x) ),
 * diagonal g*bs + b supplied already rotated by -(base + g*bs*stride).  Rotation keys needed: b*stride
 * (0 < b < bs) and base + g*bs*stride for every giant step with a present diagonal (indices taken modulo N/2;
 * a zero rotation needs no key). */
int fides_lt_create_strided(fides_ctx* ctx, uint32_t bs, uint32_t gs, int32_t stride, int32_t base, uint32_t towers,
                            const uint64_t* diags, const uint8_t* present, double scale, uint32_t* handle);
/* The same with every diagonal also given at the special primes (plaintexts raised to the extended basis, the
 * reference's ModUp'd LT plaintexts, src/CKKS/LinearTransform.cu:93-99): diags = u64[gs*bs][towers + np][N], the
 * towers Q rows then the np special rows.  Such a transform is evaluated double-hoisted (LinearTransform's
 * MODDOWN_HOIST / ONLY_C1 path, src/CKKS/LinearTransform.cu:104-190): the baby-step rotations skip their ModDown
 * and the inner sums run in the extended basis Q_t ∪ P, each giant-step sum has only its c1 ModDowned before its
 * rotation (which again skips the ModDown), and one ModDown of the total ends the transform, so a transform does
 * one ModUp per baby-step input and per giant step and gs + 1 ModDowns instead of bs + gs - 1. */
int fides_lt_create_strided_ext(fides_ctx* ctx, uint32_t bs, uint32_t gs, int32_t stride, int32_t base,
                                uint32_t towers, const uint64_t* diags, const uint8_t* present, double scale,
                                uint32_t* handle);
int fides_lt_free(fides_ctx* ctx, uint32_t handle);
int fides_eval_linear_transform(fides_ctx* ctx, uint32_t a, uint32_t lt, uint32_t* out);
/* The same transform of n ciphertexts with equal tower counts, each stage (baby-step rotations, inner sums,
 * giant-step rotations, sums) run as one batch over all of them (the reference batches the inner sums of one
 * ciphertext: DotProductPtInternal, src/CKKS/LinearTransform.cu:21-60). */
int fides_eval_linear_transform_batch(fides_ctx* ctx, uint32_t n, const uint32_t* cts, uint32_t lt, uint32_t* outs);
/* Multiplication by the monomial X^k (0 <= k < 2N), pointwise in the evaluation domain; X^(N/2) multiplies
 * every slot by i (Ciphertext::multMonomial, used by the full-slot bootstrap, src/CKKS/Bootstrap.cu:262). */
int fides_eval_mult_monomial(fides_ctx* ctx, uint32_t a, uint32_t k, uint32_t* out);

/* CKKS encoding on the GPU (OpenFHE MakeCKKSPackedPlaintext, which the reference runs on the CPU before
 * LoadPlaintext, api/CryptoContext.cpp:488-535): slots = n values re[k] + i im[k] (host; im may be null), n a power
 * of two <= N/2, encoded at `scale` into `towers` towers (sparse packings replicate with period n).  FP64 special
 * FFT on the device; every |round(scale * coefficient)| must be < 2^62 (FIDES_EINVAL otherwise). */
int fides_pt_encode(fides_ctx* ctx, const double* re, const double* im, uint32_t slots, double scale, uint32_t towers,
                    uint32_t* handle);
/* Decoding of a plaintext's first n slots at its scale (CKKSPackedEncoding::Decode): coefficients are rebuilt from
 * towers 0 and 1, so |round(scale * coefficient)| must stay below q_0 q_1 / 2 (q_0 / 2 with one tower). */
int fides_pt_decode(fides_ctx* ctx, uint32_t pt, uint32_t slots, double* re, double* im);
/* Copies a plaintext's residues (u64[towers][N], evaluation form) to host memory. */
int fides_pt_store(fides_ctx* ctx, uint32_t pt, uint64_t* data);
/* fides_lt_create_strided with the diagonals given as slot vectors (re/im [bs*gs][slots], host) and encoded on
 * the GPU at `scale` into `towers` towers: the whole bootstrap precomputation stays on the device. */
int fides_lt_create_slots(fides_ctx* ctx, uint32_t bs, uint32_t gs, int32_t stride, int32_t base, uint32_t towers,
                          const double* re, const double* im, const uint8_t* present, uint32_t slots, double scale,
                          uint32_t* handle);
/* The same encoded at the special primes too: a double-hoisted transform (fides_lt_create_strided_ext). */
int fides_lt_create_slots_ext(fides_ctx* ctx, uint32_t bs, uint32_t gs, int32_t stride, int32_t base,
                              uint32_t towers, const double* re, const double* im, const uint8_t* present,
                              uint32_t slots, double scale, uint32_t* handle);

/* EvalChebyshevSeries (api/CryptoContext.hpp:154-156, src/CKKS/ApproxModEval.cu:138-370):
 * p(x) = sum_k coeffs[k] T_k((2x - lo - hi)/(hi - lo)), k < n, constants encoded at const_scale.  The exact op
 * recipe (doubling identities for T_k, level alignment by dropping towers) is documented in
 * fideslib_gb300/csrc/poly_eval.cu.  Depth: ceil(log2(n-1)) + 1, plus 1 when [lo, hi] != [-1, 1]. */
int fides_eval_chebyshev(fides_ctx* ctx, uint32_t a, const double* coeffs, uint32_t n, double lo, double hi,
                         double const_scale, uint32_t* out);
/* x <- 2x^2 - 1 applied `iterations` times (ApproxModEval.cu:724-739 double-angle iterations of EvalMod). */
int fides_eval_double_angle(fides_ctx* ctx, uint32_t a, uint32_t iterations, uint32_t* out);
/* The same two routines over m ciphertexts in lock step (one batched launch per step; the reference evaluates
 * one ciphertext per call).  Results equal the single-ciphertext calls'. */
int fides_eval_chebyshev_batch(fides_ctx* ctx, uint32_t m, const uint32_t* cts, const double* coeffs, uint32_t n,
                               double lo, double hi, double const_scale, uint32_t* outs);
int fides_eval_double_angle_batch(fides_ctx* ctx, uint32_t m, const uint32_t* cts, uint32_t iterations,
                                  uint32_t* outs);

/* Bootstrapping (EvalBootstrap, api/CryptoContext.cpp:1719-1768; src/CKKS/Bootstrap.cu:169-333) with the
 * caller's precomputation: the CoeffsToSlots / SlotsToCoeffs factors of the level budget (one
 * fides_lt_create_strided transform per factor), the EvalMod approximation and, for sparse-secret
 * encapsulation, two switch keys.  Steps and conventions are documented in fideslib_gb300/csrc/bootstrap.cu.
 * With n = slots: the CoeffsToSlots factors multiply (first applied rightmost) to Pi U_n^-1 / (N/n) and the
 * SlotsToCoeffs factors to U_n Pi^-1, where U_n[j][k] = xi^(5^j k), xi = exp(i pi / 2n), and Pi is any slot
 * permutation (the factored special FFT leaves bit-reversed order).  Keys needed: relinearisation,
 * conjugation (Galois 2N-1), rotations n, 2n, ..., N/4 (sparse-slot trace), the factors' baby/giant steps. */
typedef struct {
  uint32_t slots;          /* n, power of two <= N/2 */
  uint32_t raise_towers;   /* towers after ModRaise */
  uint32_t cts_count;      /* CoeffsToSlots factors, 1..4 (the level budget) */
  uint32_t lt_cts[4];      /* applied in this order, each followed by a rescale */
  uint32_t stc_count;      /* SlotsToCoeffs factors, 1..4 */
  uint32_t lt_stc[4];
  uint32_t sse;            /* 1: sparse-secret encapsulation around ModRaise */
  uint32_t sse_to_sparse;  /* switch-key ids (fides_load_switch_key): dense -> sparse at one tower, */
  uint32_t sse_to_dense;   /* sparse -> dense after ModRaise */
  const double* cheb_coeffs;  /* Chebyshev approximation of cos(2 pi (r/K - 1/4) / 2^double_angle) */
  uint32_t cheb_n;
  uint32_t double_angle;
  double cheb_lo, cheb_hi;    /* approximation interval in slot values r */
  double const_scale;         /* scale for the constants of EvalMod */
  double prescale;            /* 0: the input is prescaled (the reference's `prescaled`); else the input (>= 2
                                 towers) is first multiplied by this factor, encoded at its top prime, and
                                 rescaled (ModRaise's adjustment, src/CKKS/Bootstrap.cu:441-484) */
} fides_bootstrap_plan;
int fides_eval_bootstrap(fides_ctx* ctx, uint32_t ct, const fides_bootstrap_plan* plan, uint32_t* out);
/* m bootstraps in flight together: every step batched over all m ciphertexts (equal results to m single calls;
 * the reference bootstraps one ciphertext per call). */
int fides_eval_bootstrap_batch(fides_ctx* ctx, uint32_t m, const uint32_t* cts, const fides_bootstrap_plan* plan,
                               uint32_t* outs);

/* Batched evaluation: `n` independent requests (no request may consume another one's output) run together,
 * one launch per pipeline stage for all ciphertexts of an op family, at whatever level each ciphertext is.
 * Requests rotating the same input share its ModUp.  On success ops[i].out holds the result handle.
 * Generalises the reference's cross-ciphertext batching (src/CKKS/LimbPartitionBatch.cu:20-600,
 * RNSPolyBatch.cpp) to the whole key-switching pipeline. */
enum { FIDES_OP_ADD = 1, FIDES_OP_SUB = 2, FIDES_OP_MULT = 3, FIDES_OP_SQUARE = 4, FIDES_OP_RESCALE = 5,
       FIDES_OP_ROTATE = 6, FIDES_OP_AUTOMORPHISM = 7, FIDES_OP_KEY_SWITCH = 8,
       FIDES_OP_BOOTSTRAP = 9 /* request server only (fides_server_set_bootstrap_plan) */,
       FIDES_OP_MULT_PLAIN = 10, FIDES_OP_ADD_PLAIN = 11, FIDES_OP_SUB_PLAIN = 12 /* b = plaintext handle */ };
typedef struct {
  int32_t op;      /* FIDES_OP_* */
  uint32_t a;      /* first operand handle */
  uint32_t b;      /* second operand (ADD / SUB / MULT: ciphertext; *_PLAIN: plaintext) */
  int32_t index;   /* rotation index (ROTATE), Galois element (AUTOMORPHISM) or switch-key id (KEY_SWITCH) */
  uint32_t out;    /* result handle, written by the call */
} fides_op;
int fides_eval_batch(fides_ctx* ctx, fides_op* ops, uint32_t n);

/* The same from and to host memory, pipelined (no counterpart in the reference, whose API loads, evaluates and
 * stores one ciphertext per call, api/CryptoContext.cpp:270-289): requests run in chunks of `chunk` (0 = automatic:
 * chunks of 8 with a first and last chunk of 4, which shortens the pipeline's fill and drain; one chunk below 16
 * requests); chunk k's inputs are copied to the device while earlier chunks compute and chunk k-2's results are
 * copied back, on separate streams, and consecutive chunks compute on two streams that overlap on the device.  a (and b for ADD / SUB / MULT) are host u64[2][towers][N] with `meta`; out receives
 * u64[2][out towers][N] and out_meta its metadata.  Returns after every result is in host memory.  Use pinned
 * host buffers: pageable ones make the copies synchronous. */
typedef struct {
  int32_t op;               /* FIDES_OP_* except BOOTSTRAP */
  const uint64_t* a;
  const uint64_t* b;
  fides_ct_meta meta;       /* of a (and b) */
  int32_t index;            /* rotation index / Galois element / switch-key id */
  uint64_t* out;
  fides_ct_meta out_meta;   /* written */
} fides_host_op;
int fides_eval_batch_host(fides_ctx* ctx, fides_host_op* ops, uint32_t n, uint32_t chunk);

/* Allocation-free rotation (no counterpart in the reference).  For callers that cannot allocate device memory
 * on their request path — a process whose GPU memory is pre-reserved by its own allocator, or a
 * latency-critical caller that cannot pay for cudaMalloc's implicit synchronisation.  Same result as
 * fides_eval_automorphism on the ciphertext dev_in (device u64[2][towers][N], evaluation form) with the
 * context's rotation key for `galois`, written to dev_out (device u64[2][towers][N], must not overlap dev_in).
 * Its key-switch workspace is a fixed 32 MiB device array inside the library (held by every GPU that loads it),
 * so it rejects, with FIDES_EINVAL, rotations whose workspace (t + beta(t+np) + 2(t+np) + 2t limbs of 8N bytes)
 * exceeds 32 MiB, and it calls no cudaMalloc, cudaFree or other allocating routine.  All calls share that array
 * (it keeps the last call's contents; nothing needs it zeroed): calls whose GPU work overlaps race, so order
 * them on one stream.  The context's device must be the current device (FIDES_EINVAL otherwise).  The first call
 * on a device looks up the array's address with that device current; make it before any stream capture.
 * `stream` is a cudaStream_t (NULL = the context stream). */
int fides_eval_rotate_noalloc(fides_ctx* ctx, const uint64_t* dev_in, uint32_t towers, uint32_t galois,
                              uint64_t* dev_out, void* stream);  /* dev_in, dev_out 16-byte aligned */

/* Raw residue files (no counterpart file format in the reference: it moves the same content between OpenFHE and
 * the GPU in memory, as RawCipherText / RawPlainText / RawKeySwitchKey, src/CKKS/openfhe-interface/
 * RawCiphertext.cuh:19-93).  This library's own little-endian format — NOT OpenFHE's cereal serialisation, whose
 * schema is not in this tree: a 96-byte header (magic "FGBRAW01", the fields of fides_raw_info), the rows tower
 * moduli, the rows primitive 2N-th roots the residues were transformed with (0 = not recorded), the residues
 * u64[polys][rows][N] in evaluation form (bit-reversed, RawCipherText::sub_0 / sub_1 order), and an FNV-1a 64 hash
 * of all preceding bytes.  A key holds polys = 2 dnum (the a vectors of every digit, then the b vectors) over all
 * nq + np towers, the RawKeySwitchKey::r_key layout.  Readers refuse (FIDES_EINVAL) a bad magic or size, a hash
 * mismatch, a residue at or above its modulus and, when loading into a context, other moduli, roots or ring. */
enum { FIDES_RAW_CIPHERTEXT = 1, FIDES_RAW_PLAINTEXT = 2, FIDES_RAW_RELIN_KEY = 3, FIDES_RAW_ROTATION_KEY = 4,
       FIDES_RAW_SWITCH_KEY = 5 };
typedef struct {
  uint32_t kind;       /* FIDES_RAW_* */
  uint32_t log_n;
  uint32_t rows;       /* towers per polynomial */
  uint32_t polys;      /* 2 (ciphertext), 1 (plaintext), 2 dnum (key) */
  uint32_t noise_deg;  /* RawCipherText::NoiseLevel */
  uint32_t slots;
  uint32_t id;         /* rotation key: Galois element; switch key: its id; else 0 */
  uint32_t reserved;
  double scale;        /* RawCipherText::Noise (scaling factor) */
} fides_raw_info;
/* Host buffers <-> file (no context, no device needed).  moduli and roots hold `rows` entries; roots may be NULL
 * on write.  The file is written to path.tmp and renamed into place. */
int fides_raw_write(const char* path, const fides_raw_info* info, const uint64_t* moduli, const uint64_t* roots,
                    const uint64_t* data);
int fides_raw_read_info(const char* path, fides_raw_info* info);
/* Any of moduli / roots / data may be NULL (sizes from fides_raw_read_info). */
int fides_raw_read(const char* path, fides_raw_info* info, uint64_t* moduli, uint64_t* roots, uint64_t* data);
/* Context conveniences: a resident ciphertext to a file with its towers' moduli and roots, a file back into the
 * context (its moduli and roots must be the context's), and a key file loaded as the relinearisation, rotation
 * (under its Galois element) or switch key its kind names. */
int fides_ct_save(fides_ctx* ctx, uint32_t handle, const char* path);
int fides_ct_load_file(fides_ctx* ctx, const char* path, uint32_t* handle);
int fides_key_load_file(fides_ctx* ctx, const char* path);

/* Continuous-batching request server over one context (no counterpart in the reference, whose API runs one op
 * per call).  One worker thread owns the context: while a server runs, use the context only through it.
 * Clients on any thread submit independent requests (operands must be resident ciphertext handles); the worker
 * admits every pending request that fits `mem_budget_bytes` (output + key-switch workspace per request) up to
 * `max_batch`, runs them with fides_eval_batch, and keeps up to `max_inflight_batches` batches in flight, each on a
 * stream of its own, so arrivals during a batch join the next one, which runs beside it on the GPU.  Work queued
 * on the context before the server starts completes first.  Latency = submit to completion of the request's
 * batch. */
typedef struct fides_server fides_server;
typedef struct {
  uint32_t max_batch;
  uint32_t max_inflight_batches;
  uint64_t mem_budget_bytes;
} fides_server_config;
typedef struct {
  uint64_t completed, batches;
  double p50_ms, p99_ms, mean_ms, max_ms, ops_per_s, mean_batch;
} fides_server_stats;
int fides_server_create(fides_ctx* ctx, const fides_server_config* cfg, fides_server** out);
/* One server over n contexts (rings: e.g. N = 2^15 and N = 2^16 with their own keys), all created on the current
 * device: one worker, one admission queue in arrival order and one memory budget across the rings; each admitted
 * ring's requests run as one fides_eval_batch on that ring's stream, so the rings' batches overlap on the GPU.
 * fides_server_create(ctx, ...) is the one-ring case.  Bootstrap requests go to ring 0 (the plan's ring). */
int fides_server_create_multi(fides_ctx* const* ctxs, uint32_t n, const fides_server_config* cfg,
                              fides_server** out);
/* Bootstrap requests (FIDES_OP_BOOTSTRAP, operand a) use this plan (copied, with its coefficients); requests
 * admitted together run as one fides_eval_bootstrap_batch.  Set it before submitting. */
int fides_server_set_bootstrap_plan(fides_server* s, const fides_bootstrap_plan* plan);
int fides_server_submit(fides_server* s, const fides_op* op, uint64_t* ticket);
/* Submits to ring `ring` (index into the contexts of fides_server_create_multi); the handles in `op` are that
 * ring's.  fides_server_submit submits to ring 0. */
int fides_server_submit_to(fides_server* s, uint32_t ring, const fides_op* op, uint64_t* ticket);
/* Blocks until the request finished; returns its status and result handle. */
int fides_server_wait(fides_server* s, uint64_t ticket, uint32_t* out, double* latency_ms);
/* Frees the request's result ciphertext and forgets the ticket.  The worker frees it once no pending request and
 * no batch in flight reads it, so a result may be released right after submitting requests that take it as an
 * operand. */
int fides_server_release(fides_server* s, uint64_t ticket);
int fides_server_stats_get(fides_server* s, fides_server_stats* st);
int fides_server_reset_stats(fides_server* s);
/* Drains pending work and stops the worker; results not released stay in the context (caller-owned). */
int fides_server_destroy(fides_server* s);

#ifdef __cplusplus
}
#endif
#endif
