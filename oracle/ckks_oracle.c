/*
 * CPU oracle for the CKKS evaluation hot path — TEST INFRASTRUCTURE ONLY (see ckks_oracle.h).
 *
 * Plain C99 + unsigned __int128.  Every residue is computed with exact 128-bit products and `%`, the way
 * OpenFHE's NativeInteger reference paths and FIDESlib's own CPU test helpers (test/cpuNTT_nega.cpp:24-90,
 * src/Math.cu:7-40) do it, so there is no lazy-reduction state to get wrong here.
 */
#include "ckks_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;

/* ------------------------------------------------------------------------------------------------ */
/* scalar arithmetic — src/Math.cu:7-40                                                             */
/* ------------------------------------------------------------------------------------------------ */

uint64_t orc_mulmod(uint64_t a, uint64_t b, uint64_t p) { return (uint64_t)(((u128)a * b) % p); }

uint64_t orc_powmod(uint64_t a, uint64_t e, uint64_t p) {
  uint64_t r = 1 % p;
  a %= p;
  while (e) {
    if (e & 1) r = orc_mulmod(r, a, p);
    a = orc_mulmod(a, a, p);
    e >>= 1;
  }
  return r;
}

uint64_t orc_invmod(uint64_t a, uint64_t p) { return orc_powmod(a, p - 2, p); }

static inline uint64_t addmod(uint64_t a, uint64_t b, uint64_t p) {
  uint64_t c = a + b;
  return c >= p ? c - p : c;
}
static inline uint64_t submod(uint64_t a, uint64_t b, uint64_t p) { return a >= b ? a - b : a + p - b; }

/* Deterministic Miller–Rabin for 64-bit n (bases of Jaeschke / Sinclair). */
int orc_is_prime(uint64_t n) {
  if (n < 2) return 0;
  static const uint64_t small[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
  for (int i = 0; i < 12; i++) {
    if (n == small[i]) return 1;
    if (n % small[i] == 0) return 0;
  }
  uint64_t d = n - 1;
  int r = 0;
  while ((d & 1) == 0) { d >>= 1; r++; }
  static const uint64_t bases[] = {2, 325, 9375, 28178, 450775, 9780504, 1795265022};
  for (int i = 0; i < 7; i++) {
    uint64_t a = bases[i] % n;
    if (a == 0) continue;
    uint64_t x = orc_powmod(a, d, n);
    if (x == 1 || x == n - 1) continue;
    int comp = 1;
    for (int k = 1; k < r; k++) {
      x = orc_mulmod(x, x, n);
      if (x == n - 1) { comp = 0; break; }
    }
    if (comp) return 0;
  }
  return 1;
}

int orc_gen_primes(int bits, int count, uint64_t twoN, const uint64_t* exclude, int nexclude, uint64_t* out) {
  uint64_t top = (bits >= 64) ? ~0ull : ((1ull << bits) - 1);
  uint64_t cand = top - (top % twoN) + 1; /* largest value == 1 mod 2N not above 2^bits */
  if (cand > top) cand -= twoN;
  int found = 0;
  while (found < count && cand > twoN) {
    if (orc_is_prime(cand)) {
      int skip = 0;
      for (int i = 0; i < nexclude; i++)
        if (exclude[i] == cand) skip = 1;
      for (int i = 0; i < found; i++)
        if (out[i] == cand) skip = 1;
      if (!skip) out[found++] = cand;
    }
    cand -= twoN;
  }
  return found;
}

/* Smallest generator, then g^((p-1)/order): the reference's fallback when OpenFHE roots are not supplied
 * (src/ConstantsGPU.cu:37-67, `generator` and `unity_root`). */
uint64_t orc_root_of_unity(uint64_t p, uint64_t order) {
  uint64_t phi = p - 1, n = phi;
  uint64_t fact[64];
  int nf = 0;
  for (uint64_t i = 2; i * i <= n; ++i) {
    if (n % i == 0) {
      fact[nf++] = i;
      while (n % i == 0) n /= i;
    }
    if (i > 1000000 && nf > 0) {
      /* p-1 = 2^k * m with m possibly having a large prime factor; trial division up to 1e6 then test m */
      break;
    }
  }
  if (n > 1) {
    /* the remaining cofactor: if it is composite beyond trial range we still only need prime divisors of
       phi; treat it as prime when it passes Miller–Rabin, otherwise continue trial division */
    if (orc_is_prime(n)) {
      fact[nf++] = n;
    } else {
      for (uint64_t i = 1000001; i * i <= n; i += 2) {
        if (n % i == 0) {
          fact[nf++] = i;
          while (n % i == 0) n /= i;
          if (n > 1 && orc_is_prime(n)) { fact[nf++] = n; n = 1; break; }
        }
      }
      if (n > 1) fact[nf++] = n;
    }
  }
  for (uint64_t g = 2; g < p; ++g) {
    int ok = 1;
    for (int i = 0; i < nf && ok; ++i) ok = orc_powmod(g, phi / fact[i], p) != 1;
    if (ok) return orc_powmod(g, phi / order, p);
  }
  return 0;
}

uint32_t orc_bitrev(uint32_t x, int bits) {
  uint32_t r = 0;
  for (int i = 0; i < bits; i++) r |= ((x >> i) & 1u) << (bits - 1 - i);
  return r;
}

static int ilog2(uint64_t n) {
  int l = 0;
  while ((1ull << l) < n) l++;
  return l;
}

/* ------------------------------------------------------------------------------------------------ */
/* NTT — forward CT with the bit-reversed psi table, output bit-reversed (test/cpuNTT_nega.cpp:38-85,  */
/* table layout src/ConstantsGPU.cu:222-255); inverse GS with the inverse table and N^-1.               */
/* ------------------------------------------------------------------------------------------------ */

void orc_ntt_tables(uint64_t N, uint64_t p, uint64_t psi, uint64_t* tab, uint64_t* itab) {
  int logN = ilog2(N);
  uint64_t ipsi = orc_invmod(psi, p);
  uint64_t* pw = (uint64_t*)malloc(sizeof(uint64_t) * N);
  uint64_t* ipw = (uint64_t*)malloc(sizeof(uint64_t) * N);
  pw[0] = 1;
  ipw[0] = 1;
  for (uint64_t i = 1; i < N; i++) {
    pw[i] = orc_mulmod(pw[i - 1], psi, p);
    ipw[i] = orc_mulmod(ipw[i - 1], ipsi, p);
  }
  for (uint64_t i = 0; i < N; i++) {
    tab[i] = pw[orc_bitrev((uint32_t)i, logN)];
    itab[i] = ipw[orc_bitrev((uint32_t)i, logN)];
  }
  free(pw);
  free(ipw);
}

void orc_ntt_fwd(uint64_t* a, uint64_t N, uint64_t p, const uint64_t* tab) {
  uint64_t t = N >> 1;
  for (uint64_t m = 1; m < N; m <<= 1, t >>= 1) {
    for (uint64_t i = 0; i < m; i++) {
      uint64_t w = tab[m + i];
      uint64_t j1 = 2 * i * t;
      for (uint64_t lo = j1; lo < j1 + t; lo++) {
        uint64_t u = a[lo];
        uint64_t v = orc_mulmod(a[lo + t], w, p);
        a[lo] = addmod(u, v, p);
        a[lo + t] = submod(u, v, p);
      }
    }
  }
}

void orc_ntt_inv(uint64_t* a, uint64_t N, uint64_t p, const uint64_t* itab) {
  uint64_t t = 1;
  for (uint64_t m = N >> 1; m >= 1; m >>= 1, t <<= 1) {
    for (uint64_t i = 0; i < m; i++) {
      uint64_t w = itab[m + i];
      uint64_t j1 = 2 * i * t;
      for (uint64_t lo = j1; lo < j1 + t; lo++) {
        uint64_t u = a[lo], v = a[lo + t];
        a[lo] = addmod(u, v, p);
        a[lo + t] = orc_mulmod(submod(u, v, p), w, p);
      }
    }
  }
  uint64_t ninv = orc_invmod(N % p, p);
  for (uint64_t i = 0; i < N; i++) a[i] = orc_mulmod(a[i], ninv, p);
}

void orc_ntt_batch(uint64_t* data, int nlimbs, uint64_t N, const int* prime_of, const uint64_t* moduli,
                   const uint64_t* tabs, int inverse, int nthreads) {
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
  for (int l = 0; l < nlimbs; l++) {
    int pi = prime_of[l];
    if (inverse)
      orc_ntt_inv(data + (size_t)l * N, N, moduli[pi], tabs + (size_t)pi * N);
    else
      orc_ntt_fwd(data + (size_t)l * N, N, moduli[pi], tabs + (size_t)pi * N);
  }
}

/* ------------------------------------------------------------------------------------------------ */
/* context                                                                                          */
/* ------------------------------------------------------------------------------------------------ */

struct orc_ctx {
  uint64_t N;
  int logN, nq, np, dnum, alpha, nthreads;
  uint64_t mod[ORC_MAXT];
  uint64_t* tab[ORC_MAXT];
  uint64_t* itab[ORC_MAXT];
};

orc_ctx* orc_ctx_new(uint64_t N, int nq, int np, int dnum, const uint64_t* moduli, const uint64_t* psis) {
  if (nq + np > ORC_MAXT || nq < 1 || dnum < 1) return NULL;
  orc_ctx* c = (orc_ctx*)calloc(1, sizeof(orc_ctx));
  c->N = N;
  c->logN = ilog2(N);
  c->nq = nq;
  c->np = np;
  c->dnum = dnum;
  c->alpha = (nq + dnum - 1) / dnum; /* towers per digit, OpenFHE GetNumPerPartQ */
  c->nthreads = 1;
  for (int i = 0; i < nq + np; i++) {
    c->mod[i] = moduli[i];
    c->tab[i] = (uint64_t*)malloc(sizeof(uint64_t) * N);
    c->itab[i] = (uint64_t*)malloc(sizeof(uint64_t) * N);
    uint64_t psi = psis ? psis[i] : orc_root_of_unity(moduli[i], 2 * N);
    orc_ntt_tables(N, moduli[i], psi, c->tab[i], c->itab[i]);
  }
  return c;
}

void orc_ctx_free(orc_ctx* c) {
  if (!c) return;
  for (int i = 0; i < c->nq + c->np; i++) {
    free(c->tab[i]);
    free(c->itab[i]);
  }
  free(c);
}

void orc_ctx_set_threads(orc_ctx* c, int nthreads) { c->nthreads = nthreads < 1 ? 1 : nthreads; }
int orc_ctx_alpha(const orc_ctx* c) { return c->alpha; }
const uint64_t* orc_ctx_table(const orc_ctx* c, int tower, int inverse) {
  return inverse ? c->itab[tower] : c->tab[tower];
}

void orc_to_coeff(const orc_ctx* c, uint64_t* x, int ntowers, const int* tower_ids) {
#pragma omp parallel for num_threads(c->nthreads)
  for (int i = 0; i < ntowers; i++) {
    int id = tower_ids ? tower_ids[i] : i;
    orc_ntt_inv(x + (size_t)i * c->N, c->N, c->mod[id], c->itab[id]);
  }
}

void orc_to_eval(const orc_ctx* c, uint64_t* x, int ntowers, const int* tower_ids) {
#pragma omp parallel for num_threads(c->nthreads)
  for (int i = 0; i < ntowers; i++) {
    int id = tower_ids ? tower_ids[i] : i;
    orc_ntt_fwd(x + (size_t)i * c->N, c->N, c->mod[id], c->tab[id]);
  }
}

/* Tower id of position j in the extended basis Q_t ∪ P. */
static inline int ext_id(const orc_ctx* c, int t, int j) { return j < t ? j : c->nq + (j - t); }

/* ------------------------------------------------------------------------------------------------ */
/* fast basis conversion — OpenFHE ApproxSwitchCRTBasis as consumed by FIDESlib's ModUp               */
/* (src/CKKS/Conv.cu:292-367: x_i*[Qhat_i^-1]_{q_i}, 128-bit accumulation of *[Qhat_i]_{m_j}, one      */
/* reduction) and ModDown (src/CKKS/Conv.cu:35-88).                                                   */
/* ------------------------------------------------------------------------------------------------ */

/* in: coefficient-form towers `src_ids[0..ns)`; out: coefficient-form towers `dst_ids[0..nd)` */
static void approx_switch_basis(const orc_ctx* c, const uint64_t* in, const int* src_ids, int ns, uint64_t* out,
                                const int* dst_ids, int nd) {
  uint64_t qhat_inv[ORC_MAXT];
  uint64_t qhat_mod[ORC_MAXT][ORC_MAXT];
  for (int i = 0; i < ns; i++) {
    uint64_t qi = c->mod[src_ids[i]];
    uint64_t prod = 1;
    for (int k = 0; k < ns; k++)
      if (k != i) prod = orc_mulmod(prod, c->mod[src_ids[k]] % qi, qi);
    qhat_inv[i] = orc_invmod(prod, qi);
    for (int j = 0; j < nd; j++) {
      uint64_t mj = c->mod[dst_ids[j]];
      uint64_t pr = 1;
      for (int k = 0; k < ns; k++)
        if (k != i) pr = orc_mulmod(pr, c->mod[src_ids[k]] % mj, mj);
      qhat_mod[i][j] = pr;
    }
  }
  uint64_t N = c->N;
#pragma omp parallel for num_threads(c->nthreads)
  for (uint64_t k = 0; k < N; k++) {
    uint64_t y[ORC_MAXT];
    for (int i = 0; i < ns; i++) y[i] = orc_mulmod(in[(size_t)i * N + k], qhat_inv[i], c->mod[src_ids[i]]);
    for (int j = 0; j < nd; j++) {
      u128 acc = 0;
      for (int i = 0; i < ns; i++) acc += (u128)y[i] * qhat_mod[i][j];
      out[(size_t)j * N + k] = (uint64_t)(acc % c->mod[dst_ids[j]]);
    }
  }
}

/* ModUp of one polynomial at t towers into beta = ceil(t/alpha) digits, each over Q_t ∪ P (t+np towers),
 * evaluation form.  Digit d covers towers [d*alpha, min((d+1)*alpha, t)); its own towers are copied from
 * the input, the others come from the basis conversion followed by a forward NTT
 * (OpenFHE EvalKeySwitchPrecomputeCore as restated by src/CKKS/LimbPartition.cu:693-808). */
void orc_modup(const orc_ctx* c, const uint64_t* a, int t, uint64_t* digits) {
  uint64_t N = c->N;
  int alpha = c->alpha, beta = (t + alpha - 1) / alpha, ext = t + c->np;
  for (int d = 0; d < beta; d++) {
    int start = d * alpha, size = (t - start) < alpha ? (t - start) : alpha;
    int src_ids[ORC_MAXT], dst_ids[ORC_MAXT], dst_pos[ORC_MAXT];
    uint64_t* coeff = (uint64_t*)malloc(sizeof(uint64_t) * N * size);
    for (int i = 0; i < size; i++) src_ids[i] = start + i;
    memcpy(coeff, a + (size_t)start * N, sizeof(uint64_t) * N * size);
    orc_to_coeff(c, coeff, size, src_ids);
    int nd = 0;
    for (int j = 0; j < ext; j++) {
      if (j >= start && j < start + size) continue;
      dst_ids[nd] = ext_id(c, t, j);
      dst_pos[nd] = j;
      nd++;
    }
    uint64_t* conv = (uint64_t*)malloc(sizeof(uint64_t) * N * (nd ? nd : 1));
    approx_switch_basis(c, coeff, src_ids, size, conv, dst_ids, nd);
    orc_to_eval(c, conv, nd, dst_ids);
    uint64_t* D = digits + (size_t)d * ext * N;
    for (int i = 0; i < size; i++) memcpy(D + (size_t)(start + i) * N, a + (size_t)(start + i) * N, sizeof(uint64_t) * N);
    for (int j = 0; j < nd; j++) memcpy(D + (size_t)dst_pos[j] * N, conv + (size_t)j * N, sizeof(uint64_t) * N);
    free(coeff);
    free(conv);
  }
}

/* Key inner product over Q_t ∪ P: out[0] = sum_d D_d * b_d, out[1] = sum_d D_d * a_d
 * (OpenFHE EvalFastKeySwitchCoreExt; FIDESlib fusedDotKSK_2_ src/CKKS/ElemenwiseBatchKernels.cu:202-275).
 * Key towers: Q tower j < t uses key tower j, special k uses key tower nq + k. */
void orc_ks_inner(const orc_ctx* c, const uint64_t* digits, int t, const uint64_t* key, uint64_t* out) {
  uint64_t N = c->N;
  int beta = (t + c->alpha - 1) / c->alpha, ext = t + c->np, full = c->nq + c->np;
  const uint64_t* A = key;                                /* [dnum][full][N] */
  const uint64_t* B = key + (size_t)c->dnum * full * N;   /* [dnum][full][N] */
#pragma omp parallel for num_threads(c->nthreads)
  for (int j = 0; j < ext; j++) {
    int id = ext_id(c, t, j);
    uint64_t p = c->mod[id];
    uint64_t* o0 = out + (size_t)j * N;
    uint64_t* o1 = out + (size_t)(ext + j) * N;
    for (uint64_t k = 0; k < N; k++) {
      uint64_t s0 = 0, s1 = 0;
      for (int d = 0; d < beta; d++) {
        uint64_t x = digits[((size_t)d * ext + j) * N + k];
        s0 = addmod(s0, orc_mulmod(x, B[((size_t)d * full + id) * N + k], p), p);
        s1 = addmod(s1, orc_mulmod(x, A[((size_t)d * full + id) * N + k], p), p);
      }
      o0[k] = s0;
      o1[k] = s1;
    }
  }
}

/* ModDown of one polynomial over Q_t ∪ P to Q_t: out_j = (x_j - NTT(conv_P->q_j(INTT(x_P)))) * P^-1
 * (OpenFHE ApproxModDown; FIDESlib ModDown2 src/CKKS/Conv.cu:26-133 + moddown_fusion
 * src/NTTfusions.cuh:237-252). */
void orc_moddown(const orc_ctx* c, const uint64_t* x, int t, uint64_t* out) {
  uint64_t N = c->N;
  int np = c->np;
  int src_ids[ORC_MAXT], dst_ids[ORC_MAXT];
  for (int k = 0; k < np; k++) src_ids[k] = c->nq + k;
  for (int j = 0; j < t; j++) dst_ids[j] = j;
  uint64_t* xp = (uint64_t*)malloc(sizeof(uint64_t) * N * np);
  memcpy(xp, x + (size_t)t * N, sizeof(uint64_t) * N * np);
  orc_to_coeff(c, xp, np, src_ids);
  uint64_t* conv = (uint64_t*)malloc(sizeof(uint64_t) * N * t);
  approx_switch_basis(c, xp, src_ids, np, conv, dst_ids, t);
  orc_to_eval(c, conv, t, dst_ids);
#pragma omp parallel for num_threads(c->nthreads)
  for (int j = 0; j < t; j++) {
    uint64_t q = c->mod[j];
    uint64_t P = 1;
    for (int k = 0; k < np; k++) P = orc_mulmod(P, c->mod[c->nq + k] % q, q);
    uint64_t pinv = orc_invmod(P, q);
    for (uint64_t k = 0; k < N; k++)
      out[(size_t)j * N + k] = orc_mulmod(submod(x[(size_t)j * N + k], conv[(size_t)j * N + k], q), pinv, q);
  }
  free(xp);
  free(conv);
}

/* KeySwitchCore: (ModDown(sum D_d b_d), ModDown(sum D_d a_d)), out u64[2][t][N]. */
void orc_keyswitch(const orc_ctx* c, const uint64_t* a, int t, const uint64_t* key, uint64_t* out) {
  uint64_t N = c->N;
  int beta = (t + c->alpha - 1) / c->alpha, ext = t + c->np;
  uint64_t* digits = (uint64_t*)malloc(sizeof(uint64_t) * N * ext * beta);
  uint64_t* inner = (uint64_t*)malloc(sizeof(uint64_t) * N * ext * 2);
  orc_modup(c, a, t, digits);
  orc_ks_inner(c, digits, t, key, inner);
  orc_moddown(c, inner, t, out);
  orc_moddown(c, inner + (size_t)ext * N, t, out + (size_t)t * N);
  free(digits);
  free(inner);
}

/* Evaluation-form automorphism X -> X^k: out[brev(j)] = in[brev(((2j+1)k mod 2N) >> 1)]
 * (OpenFHE PrecomputeAutoMap/AutomorphismTransform; FIDESlib automorph_slot src/Rotation.cuh:14-26, which
 * scatters with the inverse element 5^(2N-idx), src/CKKS/RNSPoly.cpp:632-634). */
void orc_automorph(const orc_ctx* c, const uint64_t* in, int nlimbs, uint32_t galois, uint64_t* out) {
  uint64_t N = c->N, mask = 2 * N - 1;
  int logN = c->logN;
  uint32_t* map = (uint32_t*)malloc(sizeof(uint32_t) * N);
  for (uint64_t j = 0; j < N; j++) {
    uint64_t idx = ((((2 * j + 1) * (uint64_t)galois) & mask) >> 1);
    map[orc_bitrev((uint32_t)j, logN)] = orc_bitrev((uint32_t)idx, logN);
  }
#pragma omp parallel for num_threads(c->nthreads)
  for (int l = 0; l < nlimbs; l++)
    for (uint64_t j = 0; j < N; j++) out[(size_t)l * N + j] = in[(size_t)l * N + map[j]];
  free(map);
}

/* OpenFHE FindAutomorphismIndex2nComplex: 5^index mod 2N (5^-1 for negative indices), 2N-1 = conjugation. */
uint32_t orc_galois_for_index(uint64_t N, int32_t index) {
  uint64_t M = 2 * N;
  if (index == 0) return 1;
  if ((uint64_t)index == M - 1) return (uint32_t)(M - 1);
  uint64_t g0 = 5;
  if (index < 0) {
    /* inverse of 5 modulo the power of two M */
    uint64_t inv = 1;
    for (uint64_t k = 1; k < M; k += 2)
      if ((k * 5) % M == 1) { inv = k; break; }
    g0 = inv;
  }
  uint64_t e = (uint64_t)(index < 0 ? -(int64_t)index : index);
  uint64_t g = 1;
  for (uint64_t k = 0; k < e; k++) g = (g * g0) % M;
  return (uint32_t)g;
}

/* EvalRotate / EvalAutomorphism: KeySwitch(c1) (with ModDown), add c0, then the automorphism on both
 * polynomials — OpenFHE's order (the reference's fused kernel applies the automorphism before ModDown,
 * src/CKKS/ElemenwiseBatchKernels.cu:333-376, which is why its Rotate test only checks precision). */
void orc_rotate(const orc_ctx* c, const uint64_t* ct, int t, uint32_t galois, const uint64_t* key, uint64_t* out) {
  uint64_t N = c->N;
  uint64_t* ks = (uint64_t*)malloc(sizeof(uint64_t) * N * t * 2);
  orc_keyswitch(c, ct + (size_t)t * N, t, key, ks);
  orc_add(c, ks, ct, t, 1, ks);
  orc_automorph(c, ks, 2 * t, galois, out);
  free(ks);
}

/* EvalFastRotation: ModUp(c1) once, then per index the key inner product, ModDown, +c0 and automorphism. */
void orc_rotate_hoisted(const orc_ctx* c, const uint64_t* ct, int t, int n, const uint32_t* galois,
                        const uint64_t* const* keys, uint64_t* const* outs) {
  uint64_t N = c->N;
  int beta = (t + c->alpha - 1) / c->alpha, ext = t + c->np;
  uint64_t* digits = (uint64_t*)malloc(sizeof(uint64_t) * N * ext * beta);
  uint64_t* inner = (uint64_t*)malloc(sizeof(uint64_t) * N * ext * 2);
  uint64_t* ks = (uint64_t*)malloc(sizeof(uint64_t) * N * t * 2);
  orc_modup(c, ct + (size_t)t * N, t, digits);
  for (int r = 0; r < n; r++) {
    orc_ks_inner(c, digits, t, keys[r], inner);
    orc_moddown(c, inner, t, ks);
    orc_moddown(c, inner + (size_t)ext * N, t, ks + (size_t)t * N);
    orc_add(c, ks, ct, t, 1, ks);
    orc_automorph(c, ks, 2 * t, galois[r], outs[r]);
  }
  free(digits);
  free(inner);
  free(ks);
}

/* Tensor product (c0d0, c0d1 + c1d0, c1d1) — FIDESlib binomialMult_ (ElemenwiseBatchKernels.cu:1363-1400). */
void orc_tensor(const orc_ctx* c, const uint64_t* x, const uint64_t* y, int t, uint64_t* out3) {
  uint64_t N = c->N;
#pragma omp parallel for num_threads(c->nthreads)
  for (int j = 0; j < t; j++) {
    uint64_t p = c->mod[j];
    const uint64_t *x0 = x + (size_t)j * N, *x1 = x + (size_t)(t + j) * N;
    const uint64_t *y0 = y + (size_t)j * N, *y1 = y + (size_t)(t + j) * N;
    uint64_t *d0 = out3 + (size_t)j * N, *d1 = out3 + (size_t)(t + j) * N, *d2 = out3 + (size_t)(2 * t + j) * N;
    for (uint64_t k = 0; k < N; k++) {
      d0[k] = orc_mulmod(x0[k], y0[k], p);
      d1[k] = addmod(orc_mulmod(x0[k], y1[k], p), orc_mulmod(x1[k], y0[k], p), p);
      d2[k] = orc_mulmod(x1[k], y1[k], p);
    }
  }
}

/* EvalMult with relinearisation (OpenFHE EvalMult + KeySwitchInPlace on a 3-element ciphertext;
 * FIDESlib Ciphertext::mult src/CKKS/Ciphertext.cpp:458-677). */
void orc_mult(const orc_ctx* c, const uint64_t* x, const uint64_t* y, int t, const uint64_t* rlk, uint64_t* out) {
  uint64_t N = c->N;
  uint64_t* d = (uint64_t*)malloc(sizeof(uint64_t) * N * t * 3);
  uint64_t* ks = (uint64_t*)malloc(sizeof(uint64_t) * N * t * 2);
  orc_tensor(c, x, y, t, d);
  orc_keyswitch(c, d + (size_t)2 * t * N, t, rlk, ks);
  orc_add(c, d, ks, t, 2, out);
  free(d);
  free(ks);
}

void orc_square(const orc_ctx* c, const uint64_t* x, int t, const uint64_t* rlk, uint64_t* out) {
  orc_mult(c, x, x, t, rlk, out);
}

/* OpenFHE NativeVector::SwitchModulus (quoted at src/CKKS/Rescale.cuh:12-44): centred lift of v mod om. */
static inline uint64_t switch_modulus(uint64_t v, uint64_t om, uint64_t nm) {
  uint64_t half = om >> 1;
  if (nm > om) {
    if (v > half) v = v + (nm - om);
    return v;
  }
  uint64_t diff = nm - (om % nm);
  if (v > half) v = v + diff;
  if (v >= nm) v = v % nm;
  return v;
}

/* Rescale (ModReduce / DropLastElementAndScale): x_i' = (x_i - NTT_i(SwitchModulus(INTT(x_top))))*q_top^-1
 * (src/CKKS/LimbPartition.cu:575-652, rescale_fusion src/NTTfusions.cuh:214-235). */
void orc_rescale(const orc_ctx* c, const uint64_t* ct, int t, uint64_t* out) {
  uint64_t N = c->N;
  uint64_t qt = c->mod[t - 1];
  for (int poly = 0; poly < 2; poly++) {
    const uint64_t* X = ct + (size_t)poly * t * N;
    uint64_t* top = (uint64_t*)malloc(sizeof(uint64_t) * N);
    memcpy(top, X + (size_t)(t - 1) * N, sizeof(uint64_t) * N);
    orc_ntt_inv(top, N, qt, c->itab[t - 1]);
#pragma omp parallel for num_threads(c->nthreads)
    for (int i = 0; i < t - 1; i++) {
      uint64_t q = c->mod[i];
      uint64_t* tmp = (uint64_t*)malloc(sizeof(uint64_t) * N);
      for (uint64_t k = 0; k < N; k++) tmp[k] = switch_modulus(top[k], qt, q);
      orc_ntt_fwd(tmp, N, q, c->tab[i]);
      uint64_t qinv = orc_invmod(qt % q, q);
      uint64_t* O = out + ((size_t)poly * (t - 1) + i) * N;
      for (uint64_t k = 0; k < N; k++) O[k] = orc_mulmod(submod(X[(size_t)i * N + k], tmp[k], q), qinv, q);
      free(tmp);
    }
    free(top);
  }
}

void orc_add(const orc_ctx* c, const uint64_t* x, const uint64_t* y, int nl, int npolys, uint64_t* out) {
  uint64_t N = c->N;
  for (int poly = 0; poly < npolys; poly++)
    for (int j = 0; j < nl; j++) {
      uint64_t p = c->mod[j];
      size_t off = ((size_t)poly * nl + j) * N;
      for (uint64_t k = 0; k < N; k++) out[off + k] = addmod(x[off + k], y[off + k], p);
    }
}

void orc_sub(const orc_ctx* c, const uint64_t* x, const uint64_t* y, int nl, int npolys, uint64_t* out) {
  uint64_t N = c->N;
  for (int poly = 0; poly < npolys; poly++)
    for (int j = 0; j < nl; j++) {
      uint64_t p = c->mod[j];
      size_t off = ((size_t)poly * nl + j) * N;
      for (uint64_t k = 0; k < N; k++) out[off + k] = submod(x[off + k], y[off + k], p);
    }
}

/* ------------------------------------------------------------------------------------------------ */
/* bootstrap building blocks — multPt / addPt (src/CKKS/LimbPartition.cu:654-691, src/AddSub.cu:10-123),  */
/* scalar ops (ElemenwiseBatchKernels.cu Scalar_mult_, AddSub.cu scalar_add_), ModRaise                 */
/* (src/CKKS/Bootstrap.cu:393-...: coefficient form of tower 0, SwitchModulus into every tower, NTT).   */
/* ------------------------------------------------------------------------------------------------ */

void orc_plain_op(const orc_ctx* c, const uint64_t* ct, const uint64_t* pt, int t, int mode, uint64_t* out) {
  uint64_t N = c->N;
  for (int j = 0; j < t; j++) {
    uint64_t q = c->mod[j];
    for (uint64_t k = 0; k < N; k++) {
      size_t o0 = (size_t)j * N + k, o1 = ((size_t)t + j) * N + k;
      uint64_t w = pt[(size_t)j * N + k];
      if (mode == 0) {
        out[o0] = orc_mulmod(ct[o0], w, q);
        out[o1] = orc_mulmod(ct[o1], w, q);
      } else {
        out[o0] = mode == 1 ? addmod(ct[o0], w, q) : submod(ct[o0], w, q);
        out[o1] = ct[o1];
      }
    }
  }
}

void orc_scalar_op(const orc_ctx* c, const uint64_t* ct, int t, const uint64_t* mul, const uint64_t* add,
                   uint64_t* out) {
  uint64_t N = c->N;
  for (int p = 0; p < 2; p++)
    for (int j = 0; j < t; j++) {
      uint64_t q = c->mod[j];
      for (uint64_t k = 0; k < N; k++) {
        size_t o = ((size_t)p * t + j) * N + k;
        uint64_t v = orc_mulmod(ct[o], mul[j], q);
        out[o] = p == 0 ? addmod(v, add[j], q) : v;
      }
    }
}

void orc_mod_raise(const orc_ctx* c, const uint64_t* ct, int t_in, int T, uint64_t* out) {
  uint64_t N = c->N, q0 = c->mod[0];
  uint64_t* top = (uint64_t*)malloc(sizeof(uint64_t) * N);
  for (int p = 0; p < 2; p++) {
    memcpy(top, ct + (size_t)p * t_in * N, sizeof(uint64_t) * N);
    orc_ntt_inv(top, N, q0, c->itab[0]);
    for (int j = 0; j < T; j++) {
      uint64_t* O = out + ((size_t)p * T + j) * N;
      for (uint64_t k = 0; k < N; k++) O[k] = switch_modulus(top[k], q0, c->mod[j]);
      orc_ntt_fwd(O, N, c->mod[j], c->tab[j]);
    }
  }
  free(top);
}

/* Multiplication by X^k (0 <= k < 2N) as a negacyclic shift of the coefficients (X^N = -1): the definition
 * behind Ciphertext::multMonomial (src/CKKS/Bootstrap.cu:262), computed in the coefficient domain so that it
 * checks the evaluation-domain product independently. */
void orc_mult_monomial(const orc_ctx* c, const uint64_t* ct, int t, uint32_t k, uint64_t* out) {
  uint64_t N = c->N;
  k &= (uint32_t)(2 * N - 1);
  uint64_t* a = (uint64_t*)malloc(sizeof(uint64_t) * N);
  for (int p = 0; p < 2; p++)
    for (int j = 0; j < t; j++) {
      const uint64_t q = c->mod[j];
      memcpy(a, ct + ((size_t)p * t + j) * N, sizeof(uint64_t) * N);
      orc_ntt_inv(a, N, q, c->itab[j]);
      uint64_t* O = out + ((size_t)p * t + j) * N;
      for (uint64_t i = 0; i < N; i++) {
        uint64_t e = (i + k) % (2 * N);
        uint64_t v = a[i];
        if (e >= N) {
          e -= N;
          v = v ? q - v : 0;
        }
        O[e] = v;
      }
      orc_ntt_fwd(O, N, q, c->tab[j]);
    }
  free(a);
}

/* ------------------------------------------------------------------------------------------------ */
/* synthetic inputs: SplitMix64 streams, ternary / sparse secrets, rounded-Gaussian errors (sigma 3.19) */
/* ------------------------------------------------------------------------------------------------ */

static inline uint64_t splitmix(uint64_t* s) {
  uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
static inline uint64_t uniform_mod(uint64_t* s, uint64_t p) {
  /* rejection sampling: exact uniform on [0,p) */
  uint64_t lim = ~0ull - (~0ull % p);
  uint64_t r;
  do { r = splitmix(s); } while (r >= lim);
  return r % p;
}
static int64_t gauss(uint64_t* s, double sigma) {
  double u1 = ((splitmix(s) >> 11) + 1.0) * (1.0 / 9007199254740993.0);
  double u2 = (splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
  double z = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
  return (int64_t)llround(z * sigma);
}
static inline uint64_t to_residue(int64_t v, uint64_t p) {
  if (v >= 0) return (uint64_t)v % p;
  uint64_t m = (uint64_t)(-(v + 1)) % p; /* avoid overflow at INT64_MIN */
  return (p - 1 - m) % p;
}

void orc_rng_fill_uniform(const orc_ctx* c, uint64_t seed, uint64_t* x, int ntowers, const int* tower_ids) {
  for (int i = 0; i < ntowers; i++) {
    int id = tower_ids ? tower_ids[i] : i;
    uint64_t s = seed ^ (0x51ED2701ull * (uint64_t)(i + 1));
    for (uint64_t k = 0; k < c->N; k++) x[(size_t)i * c->N + k] = uniform_mod(&s, c->mod[id]);
  }
}

void orc_keygen_secret(const orc_ctx* c, uint64_t seed, int h, int64_t* s_coeffs) {
  uint64_t st = seed;
  uint64_t N = c->N;
  if (h <= 0) {
    for (uint64_t k = 0; k < N; k++) s_coeffs[k] = (int64_t)(splitmix(&st) % 3) - 1;
    return;
  }
  memset(s_coeffs, 0, sizeof(int64_t) * N);
  int placed = 0;
  while (placed < h) {
    uint64_t pos = splitmix(&st) % N;
    if (s_coeffs[pos] != 0) continue;
    s_coeffs[pos] = (splitmix(&st) & 1) ? 1 : -1;
    placed++;
  }
}

/* Secret in evaluation form over all nq+np towers: u64[nq+np][N]. */
void orc_secret_eval(const orc_ctx* c, const int64_t* s, uint64_t* s_eval) {
  int full = c->nq + c->np;
  for (int i = 0; i < full; i++)
    for (uint64_t k = 0; k < c->N; k++) s_eval[(size_t)i * c->N + k] = to_residue(s[k], c->mod[i]);
  orc_to_eval(c, s_eval, full, NULL);
}

/* Hybrid key-switching key from s_from to s_to (both given as coefficient vectors already permuted as needed
 * is not general enough: the relinearisation key needs s^2), so this worker takes evaluation forms.
 * b_d = -a_d*s_to + e_d + [P]_{q_i}*s_from on the towers of digit d (OpenFHE KeySwitchHYBRID::KeySwitchGen). */
static void ksk_gen_eval(const orc_ctx* c, uint64_t seed, const uint64_t* from_eval, const uint64_t* to_eval,
                         uint64_t* key) {
  uint64_t N = c->N;
  int full = c->nq + c->np;
  uint64_t* A = key;
  uint64_t* B = key + (size_t)c->dnum * full * N;
  uint64_t* e = (uint64_t*)malloc(sizeof(uint64_t) * N * full);
  int64_t* ec = (int64_t*)malloc(sizeof(int64_t) * N);
  for (int d = 0; d < c->dnum; d++) {
    uint64_t st = seed ^ (0xA5A5A5A5ull * (uint64_t)(d + 1));
    for (uint64_t k = 0; k < N; k++) ec[k] = gauss(&st, 3.19);
    for (int i = 0; i < full; i++)
      for (uint64_t k = 0; k < N; k++) e[(size_t)i * N + k] = to_residue(ec[k], c->mod[i]);
    orc_to_eval(c, e, full, NULL);
    int start = d * c->alpha, end = start + c->alpha;
    if (end > c->nq) end = c->nq;
    for (int i = 0; i < full; i++) {
      uint64_t p = c->mod[i];
      uint64_t Pm = 1;
      for (int k = 0; k < c->np; k++) Pm = orc_mulmod(Pm, c->mod[c->nq + k] % p, p);
      uint64_t ss = st ^ (0x1234567ull * (uint64_t)(i + 1));
      for (uint64_t k = 0; k < N; k++) {
        uint64_t a = uniform_mod(&ss, p);
        A[((size_t)d * full + i) * N + k] = a;
        uint64_t b = submod(e[(size_t)i * N + k], orc_mulmod(a, to_eval[(size_t)i * N + k], p), p);
        if (i >= start && i < end) b = addmod(b, orc_mulmod(Pm, from_eval[(size_t)i * N + k], p), p);
        B[((size_t)d * full + i) * N + k] = b;
      }
    }
  }
  free(e);
  free(ec);
}

void orc_ksk_gen(const orc_ctx* c, uint64_t seed, const int64_t* s_from, const int64_t* s_to, uint64_t* key) {
  size_t sz = sizeof(uint64_t) * c->N * (c->nq + c->np);
  uint64_t *f = (uint64_t*)malloc(sz), *t = (uint64_t*)malloc(sz);
  orc_secret_eval(c, s_from, f);
  orc_secret_eval(c, s_to, t);
  ksk_gen_eval(c, seed, f, t, key);
  free(f);
  free(t);
}

void orc_relin_keygen(const orc_ctx* c, uint64_t seed, const int64_t* s, uint64_t* key) {
  int full = c->nq + c->np;
  size_t sz = sizeof(uint64_t) * c->N * full;
  uint64_t *se = (uint64_t*)malloc(sz), *s2 = (uint64_t*)malloc(sz);
  orc_secret_eval(c, s, se);
  for (int i = 0; i < full; i++)
    for (uint64_t k = 0; k < c->N; k++) {
      size_t o = (size_t)i * c->N + k;
      s2[o] = orc_mulmod(se[o], se[o], c->mod[i]);
    }
  ksk_gen_eval(c, seed, s2, se, key);
  free(se);
  free(s2);
}

/* Rotation key for Galois element k, used as "key-switch c1 then apply X->X^k": it switches s to
 * tau_{k^-1}(s), so that tau_k of the result decrypts under s. */
void orc_rot_keygen(const orc_ctx* c, uint64_t seed, const int64_t* s, uint32_t galois, uint64_t* key) {
  int full = c->nq + c->np;
  uint64_t M = 2 * c->N;
  uint64_t kinv = 0;
  for (uint64_t k = 1; k < M; k += 2)
    if (((uint64_t)galois * k) % M == 1) { kinv = k; break; }
  size_t sz = sizeof(uint64_t) * c->N * full;
  uint64_t *se = (uint64_t*)malloc(sz), *st = (uint64_t*)malloc(sz);
  orc_secret_eval(c, s, se);
  orc_automorph(c, se, full, (uint32_t)kinv, st);
  ksk_gen_eval(c, seed, se, st, key);
  free(se);
  free(st);
}

/* ------------------------------------------------------------------------------------------------ */
/* canonical-embedding encode / decode (slot j <-> zeta^(5^j), zeta = exp(i*pi/N)), used only to state    */
/* decrypted precision; sparse packing replicates the slot vector (X -> X^(N/2n) subring).                 */
/* ------------------------------------------------------------------------------------------------ */

static void fft_inplace(double* re, double* im, uint64_t n, int sign) {
  int lg = ilog2(n);
  for (uint64_t i = 0; i < n; i++) {
    uint64_t j = orc_bitrev((uint32_t)i, lg);
    if (i < j) {
      double t = re[i]; re[i] = re[j]; re[j] = t;
      t = im[i]; im[i] = im[j]; im[j] = t;
    }
  }
  for (uint64_t len = 2; len <= n; len <<= 1) {
    double ang = sign * 2.0 * 3.14159265358979323846 / (double)len;
    for (uint64_t i = 0; i < n; i += len)
      for (uint64_t j = 0; j < len / 2; j++) {
        double wr = cos(ang * (double)j), wi = sin(ang * (double)j);
        double ur = re[i + j], ui = im[i + j];
        double vr = re[i + j + len / 2] * wr - im[i + j + len / 2] * wi;
        double vi = re[i + j + len / 2] * wi + im[i + j + len / 2] * wr;
        re[i + j] = ur + vr; im[i + j] = ui + vi;
        re[i + j + len / 2] = ur - vr; im[i + j + len / 2] = ui - vi;
      }
  }
}

void orc_encode_ids(const orc_ctx* c, const double* zr, const double* zi, int slots, double scale, int nt,
                    const int* tower_ids, uint64_t* pt) {
  uint64_t N = c->N, M = 2 * N;
  double* re = (double*)calloc(M, sizeof(double));
  double* im = (double*)calloc(M, sizeof(double));
  uint64_t g = 1;
  for (uint64_t j = 0; j < N / 2; j++) {
    uint64_t s = j % (uint64_t)slots;
    re[g] = zr[s]; im[g] = zi[s];
    re[M - g] = zr[s]; im[M - g] = -zi[s];
    g = (g * 5) % M;
  }
  /* m_i = (1/N) sum_k v_k zeta^{-ik}: forward DFT (negative exponent) of length 2N */
  fft_inplace(re, im, M, -1);
  for (int j = 0; j < nt; j++) {
    uint64_t q = c->mod[tower_ids ? tower_ids[j] : j];
    for (uint64_t k = 0; k < N; k++) {
      int64_t v = (int64_t)llround(re[k] / (double)N * scale);
      pt[(size_t)j * N + k] = to_residue(v, q);
    }
  }
  orc_to_eval(c, pt, nt, tower_ids);
  free(re);
  free(im);
}

void orc_encode(const orc_ctx* c, const double* zr, const double* zi, int slots, double scale, int t, uint64_t* pt) {
  orc_encode_ids(c, zr, zi, slots, scale, t, NULL, pt);
}

/* Element-wise x (op) y on npolys polys of nl limbs, limb j modulo tower_ids[j] (op 0 = product, 1 = sum); y has
 * ypolys polys (1 = the same plaintext for every poly of x).  The extended-basis arithmetic of the double-hoisted
 * linear transform (pt products and sums over Q_t ∪ P). */
void orc_ew_ids(const orc_ctx* c, const uint64_t* x, const uint64_t* y, int nl, int npolys, int ypolys,
                const int* tower_ids, int op, uint64_t* out) {
  uint64_t N = c->N;
  for (int poly = 0; poly < npolys; poly++)
    for (int j = 0; j < nl; j++) {
      uint64_t p = c->mod[tower_ids[j]];
      size_t xo = ((size_t)poly * nl + j) * N, yo = ((size_t)(ypolys == 1 ? 0 : poly) * nl + j) * N;
      for (uint64_t k = 0; k < N; k++)
        out[xo + k] = op == 0 ? orc_mulmod(x[xo + k], y[yo + k], p) : addmod(x[xo + k], y[yo + k], p);
    }
}

/* CRT reconstruction to a centred double (multi-word integer arithmetic). */
static void crt_centered(const orc_ctx* c, const uint64_t* x, int t, double* out) {
  uint64_t N = c->N;
  int W = t + 1;
  uint64_t* Q = (uint64_t*)calloc(W, sizeof(uint64_t));
  uint64_t* Qhat = (uint64_t*)calloc((size_t)t * W, sizeof(uint64_t));
  uint64_t qhinv[ORC_MAXT];
  Q[0] = 1;
  for (int i = 0; i < t; i++) { /* Q *= q_i */
    u128 carry = 0;
    for (int w = 0; w < W; w++) {
      u128 v = (u128)Q[w] * c->mod[i] + carry;
      Q[w] = (uint64_t)v;
      carry = v >> 64;
    }
  }
  for (int i = 0; i < t; i++) {
    uint64_t* H = Qhat + (size_t)i * W;
    H[0] = 1;
    for (int k = 0; k < t; k++) {
      if (k == i) continue;
      u128 carry = 0;
      for (int w = 0; w < W; w++) {
        u128 v = (u128)H[w] * c->mod[k] + carry;
        H[w] = (uint64_t)v;
        carry = v >> 64;
      }
    }
    uint64_t r = 0; /* Qhat mod q_i */
    for (int w = W - 1; w >= 0; w--) r = (uint64_t)((((u128)r << 64) | H[w]) % c->mod[i]);
    qhinv[i] = orc_invmod(r, c->mod[i]);
  }
#pragma omp parallel for num_threads(c->nthreads)
  for (uint64_t k = 0; k < N; k++) {
    uint64_t acc[ORC_MAXT + 2];
    memset(acc, 0, sizeof(uint64_t) * (W + 1));
    for (int i = 0; i < t; i++) {
      uint64_t y = orc_mulmod(x[(size_t)i * N + k], qhinv[i], c->mod[i]);
      const uint64_t* H = Qhat + (size_t)i * W;
      u128 carry = 0;
      for (int w = 0; w < W; w++) {
        u128 v = (u128)H[w] * y + acc[w] + carry;
        acc[w] = (uint64_t)v;
        carry = v >> 64;
      }
      acc[W] += (uint64_t)carry;
    }
    /* reduce mod Q by repeated subtraction (acc < t*Q) */
    for (;;) {
      int ge = 1;
      if (acc[W] == 0) {
        for (int w = W - 1; w >= 0; w--) {
          if (acc[w] != Q[w]) { ge = acc[w] > Q[w]; break; }
        }
      }
      if (!ge) break;
      uint64_t borrow = 0;
      for (int w = 0; w < W; w++) {
        u128 v = (u128)acc[w] - Q[w] - borrow;
        acc[w] = (uint64_t)v;
        borrow = (uint64_t)(v >> 127) & 1;
      }
      acc[W] -= borrow;
    }
    /* centre: if 2*acc > Q use acc - Q */
    uint64_t twice[ORC_MAXT + 2];
    uint64_t carry = 0;
    for (int w = 0; w < W; w++) {
      twice[w] = (acc[w] << 1) | carry;
      carry = acc[w] >> 63;
    }
    int gt = carry != 0;
    if (!gt)
      for (int w = W - 1; w >= 0; w--)
        if (twice[w] != Q[w]) { gt = twice[w] > Q[w]; break; }
    double v = 0.0;
    if (gt) {
      uint64_t diff[ORC_MAXT + 2];
      uint64_t borrow = 0;
      for (int w = 0; w < W; w++) {
        u128 d = (u128)Q[w] - acc[w] - borrow;
        diff[w] = (uint64_t)d;
        borrow = (uint64_t)(d >> 127) & 1;
      }
      for (int w = W - 1; w >= 0; w--) v = v * 18446744073709551616.0 + (double)diff[w];
      v = -v;
    } else {
      for (int w = W - 1; w >= 0; w--) v = v * 18446744073709551616.0 + (double)acc[w];
    }
    out[k] = v;
  }
  free(Q);
  free(Qhat);
}

void orc_decode(const orc_ctx* c, const uint64_t* pt, int t, double scale, int slots, double* zr, double* zi) {
  uint64_t N = c->N, M = 2 * N;
  uint64_t* x = (uint64_t*)malloc(sizeof(uint64_t) * N * t);
  memcpy(x, pt, sizeof(uint64_t) * N * t);
  orc_to_coeff(c, x, t, NULL);
  double* coef = (double*)malloc(sizeof(double) * N);
  crt_centered(c, x, t, coef);
  double* re = (double*)calloc(M, sizeof(double));
  double* im = (double*)calloc(M, sizeof(double));
  for (uint64_t k = 0; k < N; k++) re[k] = coef[k] / scale;
  fft_inplace(re, im, M, +1); /* V_k = sum_i m_i zeta^{ik} */
  uint64_t g = 1;
  for (int j = 0; j < slots; j++) {
    zr[j] = re[g];
    zi[j] = im[g];
    g = (g * 5) % M;
  }
  free(x);
  free(coef);
  free(re);
  free(im);
}

void orc_encrypt_sk(const orc_ctx* c, uint64_t seed, const int64_t* s, const uint64_t* pt, int t, uint64_t* ct) {
  uint64_t N = c->N;
  int full = c->nq + c->np;
  uint64_t* se = (uint64_t*)malloc(sizeof(uint64_t) * N * full);
  orc_secret_eval(c, s, se);
  uint64_t st = seed;
  int64_t* ec = (int64_t*)malloc(sizeof(int64_t) * N);
  for (uint64_t k = 0; k < N; k++) ec[k] = gauss(&st, 3.19);
  uint64_t* e = (uint64_t*)malloc(sizeof(uint64_t) * N * t);
  for (int i = 0; i < t; i++)
    for (uint64_t k = 0; k < N; k++) e[(size_t)i * N + k] = to_residue(ec[k], c->mod[i]);
  orc_to_eval(c, e, t, NULL);
  for (int i = 0; i < t; i++) {
    uint64_t p = c->mod[i];
    uint64_t ss = st ^ (0x77777ull * (uint64_t)(i + 1));
    for (uint64_t k = 0; k < N; k++) {
      size_t o = (size_t)i * N + k;
      uint64_t a = uniform_mod(&ss, p);
      ct[(size_t)t * N + o] = a;
      ct[o] = addmod(submod(e[o], orc_mulmod(a, se[o], p), p), pt[o], p);
    }
  }
  free(se);
  free(ec);
  free(e);
}

void orc_decrypt(const orc_ctx* c, const int64_t* s, const uint64_t* ct, int t, uint64_t* pt) {
  uint64_t N = c->N;
  int full = c->nq + c->np;
  uint64_t* se = (uint64_t*)malloc(sizeof(uint64_t) * N * full);
  orc_secret_eval(c, s, se);
  for (int i = 0; i < t; i++) {
    uint64_t p = c->mod[i];
    for (uint64_t k = 0; k < N; k++) {
      size_t o = (size_t)i * N + k;
      pt[o] = addmod(ct[o], orc_mulmod(ct[(size_t)t * N + o], se[o], p), p);
    }
  }
  free(se);
}
