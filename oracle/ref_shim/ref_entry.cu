// C entry points over the reference's CPU negacyclic NTT (test/cpuNTT_nega.cpp:24-90), built from the
// reference sources by oracle/build_ref.sh into oracle/_ref/.  Test infrastructure only.
#include <cstdint>
#include <vector>

#include "CKKS/Context.cuh"
#include "cpuNTT_nega.hpp"

namespace FIDESlib::CKKS {
RefShimContext* GetCurrentContext() {
  static RefShimContext ctx;
  return &ctx;
}
}  // namespace FIDESlib::CKKS

extern "C" {
// In-place nega_fft on n residues with the reference's psi / inverse-psi tables (bit-reversed powers, the
// layout of src/ConstantsGPU.cu:222-255).  Output is in natural order (the function bit-reverses at the end).
void ref_nega_fft(uint64_t* a, int n, int invert, const uint64_t* psi, const uint64_t* inv_psi, uint64_t mod) {
  std::vector<uint64_t> v(a, a + n);
  FIDESlib::Testing::nega_fft(v, invert != 0, psi, inv_psi, mod, 1000);
  for (int i = 0; i < n; i++) a[i] = v[i];
}
// nega_fft2: explicit psi^i twist + cyclic FFT (test/cpuNTT_nega.cpp:155-170), natural order.
void ref_nega_fft2(uint64_t* a, int n, int invert, const uint64_t* psi, const uint64_t* inv_psi, uint64_t mod) {
  std::vector<uint64_t> v(a, a + n);
  FIDESlib::Testing::nega_fft2(v, invert != 0, psi, inv_psi, mod, 1000);
  for (int i = 0; i < n; i++) a[i] = v[i];
}
// The reference's root-of-unity choice when OpenFHE does not supply one lives in src/ConstantsGPU.cu and is
// not compiled here (that file needs OpenFHE); the oracle restates it.
}
