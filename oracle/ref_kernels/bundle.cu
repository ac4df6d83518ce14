// Test-only bundle: the reference's ModUp / ModDown conversion kernels (src/CKKS/Conv.cu), its two-pass NTT /
// INTT kernels with their fused epilogues (src/NTT.cu, src/NTTfusions.cuh) and its element-wise batch kernels (the key
// inner product fusedDotKSK_2_ and the tensor product binomialMult_, src/CKKS/ElemenwiseBatchKernels.cu), compiled
// from the sources where they lie into ONE device module (oracle/_ref/ref_kernels.cubin), so that the kernels share one `constants` symbol.
// Built by oracle/build_ref.sh; loaded by oracle/ref_kernels/harness.py through the CUDA driver API to pin the
// oracle to the reference's own kernels and to time them beside the engine's.  Never linked into the product.
#include "CKKS/Conv.cu"
#include "NTT.cu"
#include "CKKS/ElemenwiseBatchKernels.cu"
