// Conversions between FP64 and FP32 done with integer instructions.
//
// On GB300 the FP64 pipe issues about one warp instruction every 16 cycles per
// SM, and the hardware conversions F2F.F32.F64 / F2F.F64.F32 are executed on
// that pipe. The batched mixed-precision solver converts every matrix element
// once per system and every residual entry once per refinement step, so these
// conversions compete with the FP64 residual for the same scarce pipe. The
// functions below do the same conversions on the integer ALU for normal-range
// values (round to nearest even, bit-identical to the hardware conversion) and
// use the hardware conversion only for zeros, subnormals, infinities, NaNs and
// values outside the FP32 exponent range.
//
// Plain C++ on the host (tests compare them with the compiler's conversions);
// __host__ __device__ under nvcc.
#ifndef LA_F64CONV_H
#define LA_F64CONV_H

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define LA_HD __host__ __device__ __forceinline__
#else
#define LA_HD inline
#endif

LA_HD uint64_t la_bits_f64(double d) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(d);
#else
  uint64_t b;
  memcpy(&b, &d, 8);
  return b;
#endif
}
LA_HD double la_f64_from_bits(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double d;
  memcpy(&d, &b, 8);
  return d;
#endif
}
LA_HD uint32_t la_bits_f32(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t b;
  memcpy(&b, &f, 4);
  return b;
#endif
}
LA_HD float la_f32_from_bits(uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  float f;
  memcpy(&f, &b, 4);
  return f;
#endif
}

// double -> float, round to nearest even. A double whose biased exponent e
// lies in [897, 1150] is a normal float after rounding (or rounds up to
// infinity at the top, which the carry into the exponent field produces).
LA_HD float la_f64_to_f32(double d) {
  const uint64_t b = la_bits_f64(d);
  const uint32_t hi = (uint32_t)(b >> 32);
  const uint32_t e = (hi >> 20) & 0x7ffu;
  if (e - 897u <= 1150u - 897u) {
    const uint32_t sign = hi & 0x80000000u;
    const uint64_t mant = b & 0x000fffffffffffffull;
    const uint32_t m23 = (uint32_t)(mant >> 29);
    const uint32_t rem = (uint32_t)mant & 0x1fffffffu;
    uint32_t f = sign | ((e - 896u) << 23) | m23;
    f += (rem > 0x10000000u || (rem == 0x10000000u && (m23 & 1u))) ? 1u : 0u;
    return la_f32_from_bits(f);
  }
#if defined(__CUDA_ARCH__)
  return __double2float_rn(d);
#else
  return (float)d;
#endif
}

// float -> double (exact). Normal floats are widened with integer shifts.
LA_HD double la_f32_to_f64(float f) {
  const uint32_t b = la_bits_f32(f);
  const uint32_t e = (b >> 23) & 0xffu;
  if (e - 1u <= 253u) {
    const uint64_t sign = (uint64_t)(b & 0x80000000u) << 32;
    const uint64_t mant = (uint64_t)(b & 0x007fffffu) << 29;
    return la_f64_from_bits(sign | ((uint64_t)(e + 896u) << 52) | mant);
  }
  return (double)f;
}

// |d| as an unsigned integer that orders like |d| for every non-NaN double
// (NaN magnitudes order above infinity).
LA_HD uint64_t la_absbits_f64(double d) { return la_bits_f64(d) & 0x7fffffffffffffffull; }

#endif  // LA_F64CONV_H
