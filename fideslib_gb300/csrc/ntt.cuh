// Batched 64-bit negacyclic NTT / INTT for sm_103a.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "arith.cuh"

namespace fgb {

// A segment is `npolys` polynomials of `limbs` towers each, tower j of poly k at data + k*poly_stride + j*N,
// transformed modulo prime index prime_of[j].  A batch launches all limbs of all segments at once.
struct NttSeg {
  u64* data;
  long long poly_stride;
  int limbs;
  int npolys;
  int limb_begin;  // first global limb index of this segment (filled by the launcher)
  uint8_t prime_of[64];
};

constexpr int kMaxNttSegs = 8;

struct NttBatch {
  int nseg;
  int total_limbs;
  NttSeg seg[kMaxNttSegs];
};

struct DeviceTables {
  const PrimeConst* pc;     // [ntowers]
  const ulonglong2* tw_fwd; // [ntowers][N] {psi^brev(i), shoup}
  const ulonglong2* tw_inv; // [ntowers][N] {psi^-brev(i), shoup}
  int logN;
};

// Host launcher: forward (inverse=false: natural -> bit-reversed evaluation order) or inverse.
cudaError_t launch_ntt(const NttBatch& b, const DeviceTables& t, bool inverse, cudaStream_t s);

}  // namespace fgb
