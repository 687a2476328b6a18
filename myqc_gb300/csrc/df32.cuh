// df32.cuh -- double-float arithmetic on the FP32 pipes (shared by the Fock
// digestion and the purification kernels).
#pragma once

namespace mq {

// ---- double-float arithmetic on the FP32 pipes ----------------------------
// GB300 issues FP32 at many times its FP64 rate, so the digestion keeps its
// sums as unevaluated float pairs (hi + lo, ~48-bit significand).  A double x
// is split with integer operations only, without branches:
//   hi = x truncated to 24 significant bits: the sign, the exponent rebiased
//        from 1023 to 127, the top 23 fraction bits;
//   lo = the remaining 29 fraction bits (an integer r times the ulp
//        2^(E-1075) of x) converted to float (rounded to 24 bits) and scaled.
// |x - hi - lo| <= 2^-48 |x| for 2^-74 <= |x| < 2^128; below 2^-74 lo is 0
// (an absolute error under 2^-97) and below 2^-126 hi is 0 as well.
__device__ __forceinline__ float2 split_f64(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned sign = hi & 0x80000000u;
  const unsigned E = (hi >> 20) & 0x7ffu;
  const unsigned hb = sign | (((hi & 0x7fffffffu) - 0x38000000u) << 3) | (lo >> 29);
  const float h = __uint_as_float(E > 896u ? hb : sign);
  const unsigned sc = E > 948u ? (((E - 948u) << 23) | sign) : 0u;
  const float l = __uint2float_rn(lo & 0x1fffffffu) * __uint_as_float(sc);
  return make_float2(h, l);
}

// s += x * d in double-float: exact hi product (FMA), cross terms, two-sum
__device__ __forceinline__ void dfma(float2 &s, float2 x, float2 d) {
  const float ph = x.x * d.x;
  const float pe = fmaf(x.x, d.x, -ph);
  const float cr = fmaf(x.x, d.y, x.y * d.x);
  const float t = s.x + ph;
  const float bb = t - s.x;
  const float err = (s.x - (t - bb)) + (ph - bb);
  s.x = t;
  s.y += err + (pe + cr);
}

// double value of a double-float pair
__device__ __forceinline__ double df_val(float2 s) { return (double)s.x + (double)s.y; }

}  // namespace mq
