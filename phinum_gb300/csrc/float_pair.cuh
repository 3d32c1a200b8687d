// Unevaluated sums of two floats (hi + lo) for reductions that keep FP64
// off GB300's narrow FP64 pipe: the value h + l is added in FP32 and widened
// once, by the thread that writes the result.
#pragma once

namespace phn {

// (h, l) += (h2, l2): TwoSum of the high words (Knuth, TAOCP vol. 2, 4.2.2),
// the low words into the error, Fast2Sum.
__device__ __forceinline__ void fpair_add(float &h, float &l, float h2, float l2) {
  const float t = __fadd_rn(h, h2);
  const float bb = __fsub_rn(t, h);
  const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(t, bb)), __fsub_rn(h2, bb));
  const float lo = __fadd_rn(e, __fadd_rn(l, l2));
  h = __fadd_rn(t, lo);
  l = __fsub_rn(lo, __fsub_rn(h, t));
}

}  // namespace phn
