// Stand-in for the reference's CKKS/Context.cuh, which pulls in OpenFHE (absent from this tree).  It declares
// only what test/cpuNTT.cpp and test/cpuNTT_nega.cpp touch: GetCurrentContext()->precom.{constants,globals}.
// Part of the oracle's reference-build recipe (oracle/build_ref.sh); never linked into the product.
#pragma once
#include <vector>

#include "ConstantsGPU.cuh"

namespace FIDESlib::CKKS {
struct RefShimPrecom {
  std::vector<FIDESlib::Constants> constants;
  FIDESlib::Global* globals = nullptr;
};
struct RefShimContext {
  RefShimPrecom precom;
};
RefShimContext* GetCurrentContext();
}  // namespace FIDESlib::CKKS
