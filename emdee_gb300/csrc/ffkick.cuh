// ffkick.cuh -- kinetic energies of deferred kicks in float-float arithmetic, with no
// FP64 operation: an FP64 momentum split into two floats (hi + lo, 48 of its 53 bits)
// by integer operations, the kick P + CF F with CF = cfh + cfl and F an exact FP32
// value, its square and the running sums as (hi, lo) pairs on the FP32 pipe
// (error-free products by fused multiply-add, Knuth's two-sum).  Each term lands
// within ~2^-46 of its FP64 value.  Every product is explicitly rounded, so the
// error-free transformations hold in files compiled with FMA contraction too.
// Used by the kinetic pass of EmDee_boost (motion.cu).
#pragma once

#include "fpconv.h"

namespace emdee {

// Values outside the ranges the integer paths cover (zero is covered; tiny, huge,
// infinite and NaN values are not) take the hardware conversions in a separate
// function, a branch the common path never takes.
static __device__ __noinline__ float ffk_round_slow(double x) { return (float)x; }
static __device__ __noinline__ void ffk_split_slow(double x, float& hi, float& lo) {
  hi = (float)x;
  lo = (float)(x - (double)hi);
}

// round to nearest float
__device__ __forceinline__ float ffk_round(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  if (d2f_normal(b)) return __uint_as_float(d2f_bits(b));
  if ((b << 1) == 0) return __uint_as_float((unsigned int)(b >> 32));   // +-0
  return ffk_round_slow(x);
}

// x = hi + lo with hi = RN(x) and lo = RN(x - hi); x - hi is exact: the mantissa
// bits below the float's rounding point, an integer of at most 29 bits in units of
// 2^(E - 1075) (E the biased FP64 exponent), converted to float with one rounding
__device__ __forceinline__ void ffk_split(double x, float& hi, float& lo) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int E = (int)((b >> 52) & 0x7FF);
  const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
  if (E < 949 || E > 1149) {   // hi or lo outside the normal float range
    if ((b << 1) == 0) {
      hi = lo = __uint_as_float(sign);
      return;
    }
    ffk_split_slow(x, hi, lo);
    return;
  }
  const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
  unsigned int r = ((unsigned int)(E - 896) << 23) | (unsigned int)(m >> 29);
  const int rest = (int)(m & 0x1FFFFFFFu);
  const bool up = rest > 0x10000000 || (rest == 0x10000000 && (r & 1u));
  r += up ? 1u : 0u;
  hi = __uint_as_float(sign | r);
  const float scale = __uint_as_float((unsigned int)(E - 948) << 23);   // 2^(E - 1075)
  const float l = __fmul_rn((float)(up ? rest - 0x20000000 : rest), scale);
  lo = __uint_as_float(__float_as_uint(l) ^ sign);
}

// (h, l) = (ah + al) + (bh + bl), renormalised
__device__ __forceinline__ void ffk_add(float ah, float al, float bh, float bl, float& h, float& l) {
  const float t = ah + bh, bp = t - ah;
  const float te = ((ah - (t - bp)) + (bh - bp)) + (al + bl);
  h = t + te;
  l = te - (h - t);
}

// (Ah, Al) += (h + l)^2
__device__ __forceinline__ void ffk_sq_acc(float h, float l, float& Ah, float& Al) {
  const float sq = __fmul_rn(h, h);
  float e = fmaf(h, h, -sq);
  e = fmaf(2.f * h, l, e);
  const float t = Ah + sq, bp = t - Ah, err = (Ah - (t - bp)) + (sq - bp);
  Ah = t;
  Al = Al + e + err;
}

// 2KE terms of one momentum component p with force f (an exact float): (p + cf f)^2
// into (a1h, a1l) and (p + 2 cf f)^2 into (a2h, a2l), cf = cfh + cfl
__device__ __forceinline__ void ffk_two_kicks(double p, float f, float cfh, float cfl, float& a1h, float& a1l,
                                              float& a2h, float& a2l) {
  float ph, pl;
  ffk_split(p, ph, pl);
  const float q = __fmul_rn(cfh, f);                   // cf f = q + qe, exact up to cfl's rounding
  const float qe = fmaf(cfl, f, fmaf(cfh, f, -q));
  float h1, l1, h2, l2;
  ffk_add(ph, pl, q, qe, h1, l1);   // p + cf f
  ffk_sq_acc(h1, l1, a1h, a1l);
  ffk_add(h1, l1, q, qe, h2, l2);   // p + 2 cf f
  ffk_sq_acc(h2, l2, a2h, a2l);
}

}  // namespace emdee
