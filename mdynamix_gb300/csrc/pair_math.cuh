// pair_math.cuh -- FP64 exp(-y) and 1/d for the FP64 pair sweeps, in fewer
// FP64 instructions than the general library routines (GB300 issues one
// FP64 warp instruction per 64 cycles on each scheduler, so the sweeps'
// time is their FP64 instruction count).  Both stay within a few units in
// the last place of the correctly rounded value (checked against the CUDA
// library on the device by mdx_probe_pair_math).
#pragma once

#include "exp_table.cuh"

// exp(-y) for 0 <= y (clamped at 700, where the result is still normal).
// Table-driven method of P. T. P. Tang, "Table-driven implementation of the
// exponential function in IEEE floating-point arithmetic", ACM TOMS 15(2),
// 1989: -y = n ln2/256 + r with n = round(-y 256/ln2), |r| <= ln2/512
// (Cody-Waite two-part ln2/256), n = 256 m + j, so
// exp(-y) = 2^m 2^(j/256) exp(r); exp(r) by its Taylor polynomial to r^4
// (truncation below 4e-17 relative), 2^m added to the exponent field.
__device__ __forceinline__ double exp_neg(double y) {
  if (__double_as_longlong(y) > 0x4085E00000000000LL) y = 700.0;  // y > 700 (y >= 0)
  const double magic = 6755399441055744.0;  // 1.5 * 2^52: t + magic rounds t to an integer
  const double tm = fma(y, -EXP_INV_L, magic);
  const int n = __double2loint(tm);
  const double nd = tm - magic;
  double r = fma(-nd, EXP_L_HI, -y);
  r = fma(-nd, EXP_L_LO, r);
  double q = fma(r, 1.0 / 24.0, 1.0 / 6.0);
  q = fma(q, r, 0.5);
  q = fma(q, r, 1.0);
  const double p = fma(q, r, 1.0);
  const double t = __ldg(&k_exp2_256[n & 255]) * p;
  return __longlong_as_double(__double_as_longlong(t) + ((long long)(n >> 8) << 52));
}

// 1/d for d >= 1: an FP32 reciprocal as the seed, then two Newton-Raphson
// steps in FMA form (e = 1 - d y, y += y e); each step squares the relative
// error (2^-22 -> 2^-44 -> below the FP64 rounding).
__device__ __forceinline__ double rcp_nr(double d) {
  double y = (double)__fdividef(1.0f, __double2float_rn(d));
  double e = fma(-d, y, 1.0);
  y = fma(y, e, y);
  e = fma(-d, y, 1.0);
  return fma(y, e, y);
}
