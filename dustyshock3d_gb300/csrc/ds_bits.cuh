// ds_bits.cuh -- FP64 helpers on the integer pipe.
//
// GB300 executes FP64 instructions (arithmetic, compares and the FP64 <-> FP32
// conversions) at 2 lanes per SM per clock, so the per-particle kernels of the
// FP32 path are bound by that pipe.  These functions give the same results as
// the FP64 instructions they replace, from the bit patterns with 32-bit integer
// operations.  Host and device: the host build is what the CPU test checks
// against the compiler's own conversion.
#ifndef DS_BITS_CUH
#define DS_BITS_CUH

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define DS_HD __host__ __device__ __forceinline__
#else
#define DS_HD inline
#endif

DS_HD uint64_t ds_bits_of(double v) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(v);
#else
  uint64_t b;
  memcpy(&b, &v, sizeof(b));
  return b;
#endif
}

DS_HD float ds_float_of(uint32_t b) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(b);
#else
  float f;
  memcpy(&f, &b, sizeof(f));
  return f;
#endif
}

// FP64 -> FP32, round to nearest even (the IEEE conversion), for every input:
// results in the normal FP32 range are rounded here from the bits; magnitudes
// below half the smallest FP32 subnormal give a signed zero; subnormal
// results, overflow, infinities and NaNs take the FP64 conversion itself.
DS_HD float ds_d2f(double v) {
  const uint64_t b = ds_bits_of(v);
  const uint32_t hi = (uint32_t)(b >> 32), lo = (uint32_t)b;
  const uint32_t sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7ffu) - 1023 + 127;  // FP32 biased exponent
  if (e >= 1 && e <= 254) {
    const uint32_t m = ((hi & 0xfffffu) << 3) | (lo >> 29);  // the top 23 of 52 mantissa bits
    const uint32_t rest = lo & 0x1fffffffu;                  // the 29 dropped bits
    uint32_t r = ((uint32_t)e << 23) | m;
    // ties to even; a carry out of the mantissa steps the exponent (to
    // infinity from the largest binade, as the IEEE conversion does)
    r += (rest > 0x10000000u || (rest == 0x10000000u && (m & 1u))) ? 1u : 0u;
    return ds_float_of(sign | r);
  }
  if (e < -23) return ds_float_of(sign);  // |v| < 2^-150: rounds to zero
  return (float)v;
}

// Integer key ordered as the doubles are (negatives mapped below positives,
// -0.0 equal to +0.0): key(a) < key(b) exactly when a < b, for non-NaN a, b.
DS_HD int64_t ds_order_key(double v) {
  const int64_t b = (int64_t)ds_bits_of(v);
  const int64_t neg = b >> 63;  // all ones for a negative sign
  return (b ^ (neg & INT64_MAX)) - neg;
}

#undef DS_HD
#endif
