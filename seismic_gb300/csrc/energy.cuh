// Event energies (sums of squares) without FP64 arithmetic per sample,
// shared by the spectra kernel and the lag-GEMM prep kernel.
#pragma once

#include <cuda_runtime.h>

namespace seismic {

// Energy of a thread's samples without FP64 arithmetic per sample (FP64 runs
// at 1/64 of the FP32 rate on this GPU): x*x is split exactly into p + pe
// (FMA), p is added to the running sum `hi` by Knuth's TwoSum, and the
// rounding errors collect in `lo`.  hi + lo carries about 46 bits, so the
// FP64 group sum of (double)hi + (double)lo equals an FP64 accumulation to
// within ~1e-13 relative; the group sum, sqrt and 1/norm are FP64.  The
// samples come in scaled by a power of two so that x*x can neither overflow
// nor, for the terms that matter, fall below FP32's normal range.
// The _rn intrinsics keep the compiler from contracting the products and
// sums into FMAs, which would break the exact splits.
__device__ __forceinline__ void add_square(float x, float &hi, float &lo) {
  const float p = __fmul_rn(x, x);
  const float pe = fmaf(x, x, -p);  // p + pe == x * x exactly
  const float s = __fadd_rn(hi, p);
  const float bb = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));  // hi + p == s + e exactly
  hi = s;
  lo = __fadd_rn(lo, __fadd_rn(e, pe));
}

// (hi, lo) += (h2, l2): the high parts by TwoSum, the rounding error and the
// low parts into lo.
__device__ __forceinline__ void add_pair(float &hi, float &lo, float h2, float l2) {
  const float s = __fadd_rn(hi, h2);
  const float bb = __fsub_rn(s, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(h2, bb));
  hi = s;
  lo = __fadd_rn(lo, __fadd_rn(l2, e));
}

// Power-of-two exponent e with |x| * 2^-e < 1 for every |x| <= m (0 for
// m == 0), read from m's exponent bits (subnormal m: e = -125).
__device__ __forceinline__ int energy_exponent(float m) {
  if (!(m > 0.f)) return 0;
  const int biased = (__float_as_int(m) >> 23) & 0xff;
  return (biased > 0 ? biased : 1) - 126;
}
// 2^k as a float for k in [-126, 127].
__device__ __forceinline__ float exp2_int(int k) { return __int_as_float((127 + k) << 23); }
// x * 2^-e, exact, as two factors inside FP32's range (e in [-125, 129]).
struct EnergyScale {
  float s1, s2;
  __device__ __forceinline__ explicit EnergyScale(int e) : s1(exp2_int(-e / 2)), s2(exp2_int(-e - (-e / 2))) {}
  __device__ __forceinline__ float operator()(float x) const { return __fmul_rn(__fmul_rn(x, s1), s2); }
};

}  // namespace seismic
