// Operand alignment of the automatic scaling techniques (implementation and reference citations: autoscale.cu).
#pragma once
#include <vector>

#include "engine.hpp"

namespace fgb {

// Brings the operands of one request to a common level and scale the way the reference does before an addition
// or multiplication, with engine ops issued on stream `s`.  Adjusted operands are temporaries owned by the scaler
// (freed, stream-ordered, when it is destroyed, so keep it alive until the request's own launches are issued);
// the caller's ciphertexts are never modified.  Every method returns FIDES_OK or a FIDES_E* code with the message
// set for fides_last_error.
class AutoScaler {
 public:
  AutoScaler(Context* c, cudaStream_t s) : c_(c), s_(s) {}
  ~AutoScaler();
  // ADD / SUB / MULT: align a and b (copies of the caller's metadata, data pointers replaced when adjusted).
  int prepare_binary(int op, DevCt& a, DevCt& b);
  // SQUARE and products with plaintexts or scalars: rescales a degree-2 operand under an automatic technique.
  int prepare_unary(DevCt& a);

 private:
  int align(int op, DevCt& a, DevCt& b);
  int for_add(DevCt& x, const DevCt& y, bool* ok);
  int for_mult(DevCt& x, const DevCt& y, bool* ok);
  int scale_and_level(DevCt& x, int deg2, int t2, double scale2, bool* ok);
  int rescale(DevCt& x);
  int drop(DevCt& x, int t);
  int mult_const(DevCt& x, double operand);
  int alloc(int t, DevCt* out);
  void replace(DevCt& x, const DevCt& y);
  Context* c_;
  cudaStream_t s_;
  std::vector<u64*> temps_;
};

}  // namespace fgb
