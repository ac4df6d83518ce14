/*
 * CPU oracle for the CKKS evaluation hot path — TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the arithmetic that FIDESlib delegates to OpenFHE 1.5.1 (patched tag
 * fideslib-ref-v1.5.1.1, a git submodule that is not vendored in the reference tree) and of the FIDESlib
 * kernels that implement it on the GPU.  It is used by the test-suite, by the package smoke check and by the
 * CPU-baseline leg of the benchmark — never by the product path, which lives in fideslib_gb300/csrc and fails
 * loudly when its CUDA library is missing.
 *
 * Conventions (each function's comment cites the reference lines it follows):
 *   - residues are uint64, moduli < 2^62 (the configurations use < 2^60);
 *   - "evaluation" format is the negacyclic NTT output in bit-reversed order, exactly as OpenFHE's
 *     ForwardTransformToBitReverse and FIDESlib's NTT kernels produce it;
 *   - a ciphertext at t active towers is u64[2][t][N] (c0 then c1, limb-major);
 *   - a key-switching key is u64[2][dnum][nq+np][N] with index 0 = the "a" vectors and index 1 = the "b"
 *     vectors, the layout of RawKeySwitchKey::r_key (src/CKKS/openfhe-interface/RawCiphertext.cu:650-666);
 *   - towers 0..nq-1 are the Q primes, towers nq..nq+np-1 the special P primes.
 *
 * Parity pins: the NTT restatement is checked bit-for-bit against the reference's own CPU NTT
 * (test/cpuNTT_nega.cpp, compiled by oracle/build_ref.sh) and against the round-trip known-answer case of
 * test/NegacyclicNTTtests.cu:44-68.  The key-switching / rescale restatements follow OpenFHE's published
 * algorithms as FIDESlib's kernels consume their tables (see each function); no OpenFHE build exists in this
 * tree, so those are pinned by the algebraic identities the tests check (decryption, linearity, round trips).
 */
#ifndef CKKS_ORACLE_H
#define CKKS_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MAXT 64

/* ---- scalar modular arithmetic ---- */
uint64_t orc_mulmod(uint64_t a, uint64_t b, uint64_t p);
uint64_t orc_powmod(uint64_t a, uint64_t e, uint64_t p);
uint64_t orc_invmod(uint64_t a, uint64_t p);
int orc_is_prime(uint64_t n);
/* Descending search below 2^bits for `count` primes p == 1 (mod twoN), skipping `exclude`. Returns count found. */
int orc_gen_primes(int bits, int count, uint64_t twoN, const uint64_t* exclude, int nexclude, uint64_t* out);
/* Primitive `order`-th root of unity g^((p-1)/order) for the smallest generator g. */
uint64_t orc_root_of_unity(uint64_t p, uint64_t order);
uint32_t orc_bitrev(uint32_t x, int bits);

/* ---- NTT ---- */
void orc_ntt_tables(uint64_t N, uint64_t p, uint64_t psi, uint64_t* tab, uint64_t* itab);
void orc_ntt_fwd(uint64_t* a, uint64_t N, uint64_t p, const uint64_t* tab);
void orc_ntt_inv(uint64_t* a, uint64_t N, uint64_t p, const uint64_t* itab);
/* Batched transforms over limbs: limb i uses modulus moduli[prime_of[i]] and tables tabs[prime_of[i]*N ...]. */
void orc_ntt_batch(uint64_t* data, int nlimbs, uint64_t N, const int* prime_of, const uint64_t* moduli,
                   const uint64_t* tabs, int inverse, int nthreads);

/* ---- context ---- */
typedef struct orc_ctx orc_ctx;
orc_ctx* orc_ctx_new(uint64_t N, int nq, int np, int dnum, const uint64_t* moduli, const uint64_t* psis);
void orc_ctx_free(orc_ctx* c);
void orc_ctx_set_threads(orc_ctx* c, int nthreads);
int orc_ctx_alpha(const orc_ctx* c);
const uint64_t* orc_ctx_table(const orc_ctx* c, int tower, int inverse);

/* ---- hot-path ops (evaluation format in and out unless stated) ---- */
void orc_to_coeff(const orc_ctx* c, uint64_t* x, int ntowers, const int* tower_ids);
void orc_to_eval(const orc_ctx* c, uint64_t* x, int ntowers, const int* tower_ids);
void orc_modup(const orc_ctx* c, const uint64_t* a, int t, uint64_t* digits);
void orc_ks_inner(const orc_ctx* c, const uint64_t* digits, int t, const uint64_t* key, uint64_t* out);
void orc_moddown(const orc_ctx* c, const uint64_t* x, int t, uint64_t* out);
void orc_keyswitch(const orc_ctx* c, const uint64_t* a, int t, const uint64_t* key, uint64_t* out);
void orc_automorph(const orc_ctx* c, const uint64_t* in, int nlimbs, uint32_t galois, uint64_t* out);
uint32_t orc_galois_for_index(uint64_t N, int32_t index);
void orc_rotate(const orc_ctx* c, const uint64_t* ct, int t, uint32_t galois, const uint64_t* key, uint64_t* out);
void orc_rotate_hoisted(const orc_ctx* c, const uint64_t* ct, int t, int n, const uint32_t* galois,
                        const uint64_t* const* keys, uint64_t* const* outs);
void orc_tensor(const orc_ctx* c, const uint64_t* x, const uint64_t* y, int t, uint64_t* out3);
void orc_mult(const orc_ctx* c, const uint64_t* x, const uint64_t* y, int t, const uint64_t* rlk, uint64_t* out);
void orc_square(const orc_ctx* c, const uint64_t* x, int t, const uint64_t* rlk, uint64_t* out);
void orc_rescale(const orc_ctx* c, const uint64_t* ct, int t, uint64_t* out);
void orc_add(const orc_ctx* c, const uint64_t* x, const uint64_t* y, int nlimbs_per_poly, int npolys, uint64_t* out);
void orc_sub(const orc_ctx* c, const uint64_t* x, const uint64_t* y, int nlimbs_per_poly, int npolys, uint64_t* out);

/* ---- bootstrap building blocks ---- */
/* mode 0: (c0*pt, c1*pt); 1: (c0+pt, c1); 2: (c0-pt, c1).  ct u64[2][t][N], pt u64[>=t][N]. */
void orc_plain_op(const orc_ctx* c, const uint64_t* ct, const uint64_t* pt, int t, int mode, uint64_t* out);
/* out[p][j] = ct[p][j]*mul[j] (+ add[j] on c0). */
void orc_scalar_op(const orc_ctx* c, const uint64_t* ct, int t, const uint64_t* mul, const uint64_t* add,
                   uint64_t* out);
/* ModRaise: tower 0 of ct (u64[2][t_in][N]) lifted, centred, to T towers (out u64[2][T][N]). */
void orc_mod_raise(const orc_ctx* c, const uint64_t* ct, int t_in, int T, uint64_t* out);
/* ct * X^k (0 <= k < 2N), by a negacyclic coefficient shift. */
void orc_mult_monomial(const orc_ctx* c, const uint64_t* ct, int t, uint32_t k, uint64_t* out);

/* ---- synthetic key material and messages (test inputs) ---- */
void orc_rng_fill_uniform(const orc_ctx* c, uint64_t seed, uint64_t* x, int ntowers, const int* tower_ids);
void orc_keygen_secret(const orc_ctx* c, uint64_t seed, int hamming_weight, int64_t* s_coeffs);
void orc_secret_eval(const orc_ctx* c, const int64_t* s_coeffs, uint64_t* s_eval);
void orc_ksk_gen(const orc_ctx* c, uint64_t seed, const int64_t* s_from, const int64_t* s_to, uint64_t* key);
void orc_relin_keygen(const orc_ctx* c, uint64_t seed, const int64_t* s, uint64_t* key);
void orc_rot_keygen(const orc_ctx* c, uint64_t seed, const int64_t* s, uint32_t galois, uint64_t* key);
void orc_encode(const orc_ctx* c, const double* re, const double* im, int slots, double scale, int t, uint64_t* pt);
/* The same into nt rows modulo tower_ids[j] (NULL: 0..nt-1), e.g. Q towers followed by special primes. */
void orc_encode_ids(const orc_ctx* c, const double* re, const double* im, int slots, double scale, int nt,
                    const int* tower_ids, uint64_t* pt);
/* Element-wise product (op 0) or sum (op 1) over limbs with explicit tower ids; ypolys = 1 broadcasts y. */
void orc_ew_ids(const orc_ctx* c, const uint64_t* x, const uint64_t* y, int nl, int npolys, int ypolys,
                const int* tower_ids, int op, uint64_t* out);
void orc_decode(const orc_ctx* c, const uint64_t* pt, int t, double scale, int slots, double* re, double* im);
void orc_encrypt_sk(const orc_ctx* c, uint64_t seed, const int64_t* s, const uint64_t* pt, int t, uint64_t* ct);
void orc_decrypt(const orc_ctx* c, const int64_t* s, const uint64_t* ct, int t, uint64_t* pt);

#ifdef __cplusplus
}
#endif
#endif
