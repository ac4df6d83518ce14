// Element-wise and basis-conversion kernels of the CKKS key-switching pipeline (launchers).
#pragma once
#include <cuda_runtime.h>

#include "arith.cuh"

namespace fgb {

// CRT tables resident on the device (built once per context; see Context::build_tables).
struct CrtTables {
  int nq, np, alpha, dnum, ntow;
  // ModUp, digit d with s towers: base b = (d*alpha + s-1)*alpha
  const ulonglong2* mu_qhinv;  // [b + i] = {[Qhat_i^-1]_{q_i}, shoup}
  const uint32_t* mu_qhat;     // [((b + i)*ntow + tower)*2 + {0,1}] = 30-bit slices (lo, hi) of [Qhat_i]_{m_tower}
  // ModDown
  const ulonglong2* md_phinv;  // [k] = {[Phat_k^-1]_{p_k}, shoup}
  const uint32_t* md_phat;     // [(k*nq + j)*2 + {0,1}] = 30-bit slices of [Phat_k]_{q_j}
  const ulonglong2* md_pinv;   // [j] = {[P^-1]_{q_j}, shoup}
  // Rescale: top tower l, target i < l
  const ulonglong2* rs_qinv;   // [l*nq + i] = {[q_l^-1]_{q_i}, shoup}
};

struct KsDims {
  int N, logN;
  int t;      // active Q towers
  int beta;   // digits in use
};

// coeff: [t][N] coefficient-form input; conv: per digit d rows [t + np - s_d][N] at conv + d*conv_stride.
cudaError_t launch_modup_conv(const u64* coeff, u64* conv, long long conv_stride, const KsDims& k,
                              const CrtTables& c, const PrimeConst* pc, cudaStream_t s);

// digits: own towers are read from a_eval, converted towers from conv; key: [2][dnum][nq+np][N] (0 = a, 1 = b).
// inner: [2][t+np][N], inner[0] = sum D*b, inner[1] = sum D*a.
cudaError_t launch_ks_inner(const u64* a_eval, const u64* conv, long long conv_stride, const u64* key, u64* inner,
                            const KsDims& k, const CrtTables& c, const PrimeConst* pc, cudaStream_t s);

// inner P towers (coefficient form) of npolys polys laid out [poly][t+np][N]: conv_out [poly][t][N] coefficient form.
cudaError_t launch_moddown_conv(const u64* inner, long long poly_stride_in, u64* conv_out, long long poly_stride_out,
                                int npolys, const KsDims& k, const CrtTables& c, const PrimeConst* pc, cudaStream_t s);

// out[p][j][sigma(n)] = ((inner[p][j][n] - conv[p][j][n]) * P^-1 + add_p[j][n]) mod q_j, sigma = automorphism
// scatter for the Galois element whose inverse is `galois_inv` (1 = identity).
cudaError_t launch_moddown_epilogue(const u64* inner, long long in_stride, const u64* conv, long long conv_stride,
                                    const u64* add0, const u64* add1, u64* out, long long out_stride, int npolys,
                                    uint32_t galois_inv, const KsDims& k, const CrtTables& c, const PrimeConst* pc,
                                    cudaStream_t s);

// (x0, x1) (y0, y1) -> (x0y0, x0y1 + x1y0, x1y1); square when y == x.
cudaError_t launch_tensor(const u64* x, const u64* y, u64* d, int t, int N, const PrimeConst* pc, cudaStream_t s);

// out = x +/- y over npolys x t towers (same tower layout), element-wise.
cudaError_t launch_addsub(const u64* x, const u64* y, u64* out, int npolys, int t, int N, bool sub,
                          const PrimeConst* pc, cudaStream_t s);

// Rescale helpers. top: [npolys][N] coefficient-form top towers (mod q_{t-1}); tmp: [npolys][t-1][N].
cudaError_t launch_rescale_switch(const u64* top, long long top_stride, u64* tmp, int npolys, int t, int N,
                                  const PrimeConst* pc, cudaStream_t s);
// out[p][i] = (x[p][i] - tmp[p][i]) * q_{t-1}^-1 mod q_i, i < t-1.
cudaError_t launch_rescale_epilogue(const u64* x, long long x_stride, const u64* tmp, u64* out, int npolys, int t,
                                    int N, const CrtTables& c, const PrimeConst* pc, cudaStream_t s);

// Evaluation-form automorphism (gather): out[brev(j)] = in[brev(((2j+1)galois mod 2N) >> 1)].
cudaError_t launch_automorph(const u64* in, u64* out, int nlimbs, int N, int logN, uint32_t galois, cudaStream_t s);

}  // namespace fgb
