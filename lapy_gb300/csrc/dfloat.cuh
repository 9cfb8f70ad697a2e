// Double-float ("df") arithmetic: a value as an unevaluated sum hi + lo of
// two FP32 numbers (about 48 significant bits), computed with FP32
// instructions, of which this GPU issues about 64 times more per clock than
// FP64 ones.  Products use the error-free split of fmaf; sums the two-sum.
// The round-to-nearest intrinsics keep the compiler from contracting steps
// into FMAs (which would break the exactness of the transformations).
#pragma once
#include <cuda_runtime.h>

namespace lapy {

__device__ __forceinline__ float2 df_split(double v) {
  const float h = __double2float_rn(v);
  return make_float2(h, __double2float_rn(v - (double)h));
}

// (h, l) += (bh, bl), renormalised; commutative, so a butterfly of these
// leaves the same sum in every lane
__device__ __forceinline__ void df_add(float& h, float& l, float bh, float bl) {
  const float s = __fadd_rn(h, bh);
  const float v = __fsub_rn(s, h);
  const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, v)), __fsub_rn(bh, v));
  const float t = __fadd_rn(__fadd_rn(l, bl), e);
  h = __fadd_rn(s, t);
  l = __fsub_rn(t, __fsub_rn(h, s));
}

__device__ __forceinline__ void df_fma(float2 x, float2 y, float& sh, float& sl) {
  const float p = __fmul_rn(x.x, y.x);
  float e = fmaf(x.x, y.x, -p);
  e = fmaf(x.x, y.y, e);
  e = fmaf(x.y, y.x, e);
  const float t = __fadd_rn(sh, p);
  const float v = __fsub_rn(t, sh);
  const float r = __fadd_rn(__fsub_rn(sh, __fsub_rn(t, v)), __fsub_rn(p, v));
  sl = __fadd_rn(sl, __fadd_rn(r, e));
  sh = t;
}


// hi + lo as FP64
__device__ __forceinline__ double df_to_double(float2 v) { return (double)v.x + (double)v.y; }

}  // namespace lapy
