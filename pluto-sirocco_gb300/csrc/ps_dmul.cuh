// ps_dmul.cuh -- binary64 multiplication on the integer pipes.
//
// GB300's double-precision unit retires two lanes per cycle per SM (one warp
// instruction every 16 cycles), while the integer multiply-add and logic
// pipes take 64 to 128 lanes per cycle.  Kernels that are bound by the FP64
// unit leave most issue slots idle; a product formed on the integer pipes
// takes about sixty of those slots (39 ALU, 19 multiply-add) in place of
// one FP64 slot, and the two kinds of product overlap.
//
// dmul_int(a, b, bad) returns the IEEE 754 binary64 product of a and b
// rounded to nearest, ties to even (IEEE 754-2019, 4.3.1), the same bit
// pattern as the hardware multiply, formed from the 53-bit significands in
// 32-bit limbs (the schoolbook method of the software multiplication in
// Muller et al., Handbook of Floating-Point Arithmetic, 2nd ed., 8.5):
//   * four 32x32->64 multiply-adds give the exact 106-bit product P;
//   * Q = floor(P / 2^52) holds 53 or 54 bits; with 54 the product is >= 2,
//     Q is shifted right once and the exponent raised by one;
//   * the round bit and a sticky bit (any bit below it) decide the increment
//     of Q: up when the round bit is set and either the sticky bit or Q's
//     last bit is, which is one carry test (rh + 2^19 - 1 + x >= 2^20, rh the
//     20 bits below Q, x = Q's last bit | the sticky bits below rh);
//   * sign, exponent and Q are added into one pattern, Q's leading one and a
//     rounding carry out of it both landing in the exponent field.
// Zeros give the signed zero.  For subnormal, infinite or NaN operands and
// for products outside the normal range the result is not formed: `bad` is
// set and the caller redoes that cell's phase with the hardware multiply
// at the same places, so that the results are the hardware's in every case.
#pragma once

#include <stdint.h>
#include <string.h>

namespace ps {

// The bit pattern through an opaque move: with a plain reinterpretation the
// compiler turns integer tests of the pattern (a zero test, say) back into
// double-precision compares, which run on the FP64 unit.
__host__ __device__ __forceinline__ uint64_t dm_bits(double x)
{
#ifdef __CUDA_ARCH__
  uint64_t u;
  asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
  return u;
#else
  uint64_t u;
  memcpy(&u, &x, sizeof u);
  return u;
#endif
}

__host__ __device__ __forceinline__ double dm_double(uint64_t u)
{
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)u);
#else
  double x;
  memcpy(&x, &u, sizeof x);
  return x;
#endif
}

__host__ __device__ __forceinline__ double dmul_int(double a, double b, bool &bad)
{
  const uint64_t A = dm_bits(a), B = dm_bits(b);
  const uint32_t ah = (uint32_t)(A >> 32), al = (uint32_t)A;
  const uint32_t bh = (uint32_t)(B >> 32), bl = (uint32_t)B;
  // the operands' checks first, so that their exponent fields die early
  const uint32_t ea = (ah >> 20) & 0x7ffu, eb = (bh >> 20) & 0x7ffu;
  const bool za = ((ah << 1) | al) == 0u, zb = ((bh << 1) | bl) == 0u;
  const bool z = za | zb;
  bad = bad | (ea - 1u >= 2046u && !za) | (eb - 1u >= 2046u && !zb);
  const int e0 = (int)(ea + eb) - 1024;        // biased exponent - 1, before normalising
  const uint32_t sign = (ah ^ bh) & 0x80000000u;
  // significands with the leading one: high limbs of 21 bits, low of 32
  const uint32_t mah = (ah & 0xfffffu) | 0x100000u, mbh = (bh & 0xfffffu) | 0x100000u;
  // P = H 2^64 + w 2^32 + p0lo; each partial sum stays below 2^64
  const uint64_t p0 = (uint64_t)al * bl;
  const uint64_t t1 = (uint64_t)al * mbh + (p0 >> 32);
  const uint64_t t2 = (uint64_t)mah * bl + t1;
  const uint64_t H = (uint64_t)mah * mbh + (t2 >> 32);
  const uint32_t w = (uint32_t)t2, p0lo = (uint32_t)p0;
  uint64_t Q = (H << 12) | (w >> 20);          // floor(P / 2^52), 2^52 <= Q < 2^54
  const uint32_t s = (uint32_t)(Q >> 53);      // 1: P >= 2^105
  Q >>= s;
  const uint32_t rh = (w >> s) & 0xfffffu;     // the 20 bits below Q's last bit
  const uint32_t x = ((uint32_t)Q | (s & w) | (uint32_t)(p0lo != 0u)) & 1u;
  Q += (rh + 0x7ffffu + x) >> 20;               // round to nearest, ties to even
  const int em1 = e0 + (int)s;                  // the result's biased exponent - 1
  bad = bad | (!z && (uint32_t)em1 >= 2046u);
  const uint64_t R = ((uint64_t)(sign | ((uint32_t)em1 << 20)) << 32) + Q;
  return dm_double(z ? (uint64_t)sign << 32 : R);
}

// x 2^-K (K = 1, 2), exact when x and the result are normal: the exponent
// field less K (zeros pass through; anything else sets `bad`)
template <int K>
__host__ __device__ __forceinline__ double dpow2m_int(double x, bool &bad)
{
  static_assert(K == 1 || K == 2, "halving or quartering");
  const uint64_t X = dm_bits(x);
  const uint32_t e = (uint32_t)(X >> 52) & 0x7ffu;
  const bool z = (X << 1) == 0u;
  bad = bad | (!z && e - (1u + K) >= 2046u - K);
  return z ? x : dm_double(X - ((uint64_t)K << 52));
}
__host__ __device__ __forceinline__ double dhalf_int(double x, bool &bad)
{
  return dpow2m_int<1>(x, bad);
}
// 4 x, exact when x and the result are normal
__host__ __device__ __forceinline__ double dquad_int(double x, bool &bad)
{
  const uint64_t X = dm_bits(x);
  const uint32_t e = (uint32_t)(X >> 52) & 0x7ffu;
  const bool z = (X << 1) == 0u;
  bad = bad | (!z && e - 1u >= 2044u);
  return z ? x : dm_double(X + (2ull << 52));
}
// 2 x, exact when x and the result are normal
__host__ __device__ __forceinline__ double dtwice_int(double x, bool &bad)
{
  const uint64_t X = dm_bits(x);
  const uint32_t e = (uint32_t)(X >> 52) & 0x7ffu;
  const bool z = (X << 1) == 0u;
  bad = bad | (!z && e - 1u >= 2045u);
  return z ? x : dm_double(X + (1ull << 52));
}
// a b > 0 without the product: both nonzero with one sign, and (unless
// `bad` is set) both normal with a product far above the underflow
// threshold (biased exponents summing to at least 1026, the product at
// least 2^-1020), so that the rounded product is positive exactly when the
// signs agree
__host__ __device__ __forceinline__ bool dposprod_int(double a, double b, bool &bad)
{
  const uint64_t A = dm_bits(a), B = dm_bits(b);
  const uint32_t ea = (uint32_t)(A >> 52) & 0x7ffu, eb = (uint32_t)(B >> 52) & 0x7ffu;
  const bool z = (A << 1) == 0u || (B << 1) == 0u;
  bad = bad | (!z && (ea - 1u >= 2046u || eb - 1u >= 2046u || ea + eb < 1026u));
  return !z && ((A ^ B) >> 63) == 0u;
}

#ifdef __CUDACC__
// The product on the integer pipes (INT) or on the FP64 unit.  The hardware
// form is __dmul_rn, which the compiler does not fuse into a neighbouring
// add, so that a kernel written with dmul_t gives the same bits in either
// form and can redo a warp's work with INT = false when `bad` is set.
template <bool INT>
__device__ __forceinline__ double dmul_t(double a, double b, bool &bad)
{
  if constexpr (INT)
    return dmul_int(a, b, bad);
  else
    return __dmul_rn(a, b);
}
template <bool INT>
__device__ __forceinline__ double dhalf_t(double x, bool &bad)
{
  if constexpr (INT)
    return dhalf_int(x, bad);
  else
    return __dmul_rn(0.5, x);
}
template <bool INT>
__device__ __forceinline__ double dquad_t(double x, bool &bad)
{
  if constexpr (INT)
    return dquad_int(x, bad);
  else
    return __dmul_rn(4.0, x);
}
#endif

}  // namespace ps
