// fpconv.h -- IEEE-754 round-to-nearest-even conversion of a double to a float
// with integer operations, for results in the normal float range (callers use
// the hardware conversion otherwise).  On GB300 it keeps the slow FP64 pipe out
// of the FP32 packing of positions.  Pure integer arithmetic, so the host and
// the device agree; tests compare it with the C conversion on the host.
#pragma once

#ifdef __CUDACC__
#define EMD_HD_INLINE __host__ __device__ __forceinline__
#else
#define EMD_HD_INLINE inline
#endif

namespace emdee {

// float bits of the double with bits b
EMD_HD_INLINE unsigned int d2f_bits(unsigned long long b) {
  const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7FF) - 1023 + 127;   // biased float exponent
  const unsigned long long m = b & 0xFFFFFFFFFFFFFull;    // 52 mantissa bits
  unsigned int r = ((unsigned int)e << 23) | (unsigned int)(m >> 29);
  const unsigned int rest = (unsigned int)(m & 0x1FFFFFFFu), half = 0x10000000u;
  if (rest > half || (rest == half && (r & 1u))) r += 1u;   // a carry may raise the exponent
  return sign | r;
}

// true if d2f_bits applies: the rounded result is a normal, finite float
EMD_HD_INLINE bool d2f_normal(unsigned long long b) {
  const int e = (int)((b >> 52) & 0x7FF) - 1023 + 127;
  return e >= 1 && e <= 253;
}


}  // namespace emdee
