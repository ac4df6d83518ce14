// Test-only probe: prints, as JSON, the byte layout of the reference's FIDESlib::Constants (the __constant__
// block its kernels read) and FIDESlib::Global::Globals (the device table block passed to them), from
// src/ConstantsGPU.cuh, so that oracle/ref_kernels/harness.py can fill both without restating the structs.
// LP64 layout: the same on the x86_64 host that runs this and on the aarch64 GPU host.
#include <cstddef>
#include <cstdio>

#include "ConstantsGPU.cuh"

#define F(S, f) std::printf("  \"%s.%s\": %zu,\n", #S, #f, offsetof(S, f))

int main() {
  using FIDESlib::Constants;
  using G = FIDESlib::Global::Globals;
  std::printf("{\n");
  F(Constants, N); F(Constants, L); F(Constants, K); F(Constants, logN); F(Constants, type);
  F(Constants, primes); F(Constants, prime_better_barret_mu); F(Constants, prime_bits);
  F(Constants, N_shoup); F(Constants, one_shoup); F(Constants, N_inv); F(Constants, N_inv_shoup);
  F(Constants, root); F(Constants, root_shoup); F(Constants, inv_root); F(Constants, inv_root_shoup);
  F(Constants, dnum); F(Constants, P); F(Constants, P_shoup); F(Constants, P_inv); F(Constants, P_inv_shoup);
  F(Constants, num_primeid_digit_from); F(Constants, num_primeid_digit_to); F(Constants, primeid_digit);
  F(Constants, pos_in_digit); F(Constants, primeid_partition); F(Constants, primeid_digit_from);
  F(Constants, primeid_digit_to); F(Constants, primeid_special_partition);
  F(G, psi); F(G, inv_psi); F(G, psi_middle_scale); F(G, inv_psi_middle_scale); F(G, psi_no); F(G, inv_psi_no);
  F(G, psi_shoup); F(G, inv_psi_shoup); F(G, q_inv); F(G, QlQlInvModqlDivqlModq); F(G, ModDown_pre_scale);
  F(G, ModDown_pre_scale_shoup); F(G, ModDown_matrix); F(G, ModDown_matrix_shoup); F(G, DecompAndModUp_pre_scale);
  F(G, DecompAndModUp_pre_scale_shoup); F(G, DecompAndModUp_matrix); F(G, DecompAndModUp_matrix_shoup);
  std::printf("  \"MAXP\": %d,\n  \"MAXD\": %d,\n", FIDESlib::MAXP, FIDESlib::MAXD);
  std::printf("  \"sizeof.Constants\": %zu,\n  \"sizeof.Globals\": %zu\n}\n", sizeof(Constants), sizeof(G));
  return 0;
}
