// FP64 comparisons and conversions on the integer pipe.
//
// GB300 runs FP64 instructions at 1/64 of the FP32 rate, and a double
// compare, a double<->float or integer->double conversion and a double
// min/max occupy that pipe as long as an FP64 add does.  The transport
// kernels are bound by the FP64 pipe, and most of their FP64 instructions
// are such compares and conversions, not arithmetic.  The functions below
// give the same results as the IEEE-754 operations they replace, computed
// from the bit patterns with integer instructions (a 64-bit integer compare
// is a few integer instructions, each far cheaper than one FP64 slot).
//
// Conventions: "not NaN" arguments are required where stated; -0 and +0
// compare equal, as in IEEE-754.
#pragma once

#include <cstdint>

namespace omc {
namespace fpi {

constexpr long long MAG = 0x7FFFFFFFFFFFFFFFLL;  // all bits but the sign
constexpr long long EXP_INF = 0x7FF0000000000000LL;

__device__ __forceinline__ long long bits(double x) { return __double_as_longlong(x); }

// Order-preserving integer key of a double that is not NaN: -0 and +0 map
// to 0, negatives to minus their magnitude bits.
__device__ __forceinline__ long long key(double x)
{
  const long long b = bits(x);
  const long long m = b & MAG;
  return b < 0 ? -m : m;
}

// a < b, a <= b, a == b for doubles that are not NaN
__device__ __forceinline__ bool lt(double a, double b) { return key(a) < key(b); }
__device__ __forceinline__ bool le(double a, double b) { return key(a) <= key(b); }
__device__ __forceinline__ bool eq(double a, double b) { return key(a) == key(b); }

// x < 0, x > 0, x == 0, x >= 0 (exact IEEE results, NaN included)
__device__ __forceinline__ bool neg(double x)
{
  const long long b = bits(x);
  const long long m = b & MAG;
  return b < 0 && m != 0 && m <= EXP_INF;
}
__device__ __forceinline__ bool pos(double x)
{
  const long long b = bits(x);
  return b > 0 && b <= EXP_INF;
}
__device__ __forceinline__ bool zero(double x) { return (bits(x) & MAG) == 0; }
__device__ __forceinline__ bool nonneg(double x)
{
  const long long b = bits(x);
  return (b >= 0 && b <= EXP_INF) || (b & MAG) == 0;
}

// |x| < c and |x| > c for a constant c > 0 (NaN x: false for both)
__device__ __forceinline__ bool abs_lt(double x, double c) { return (bits(x) & MAG) < bits(c); }
__device__ __forceinline__ bool abs_gt(double x, double c)
{
  const long long m = bits(x) & MAG;
  return m > bits(c) && m <= EXP_INF;
}

// uint64 word w -> w x 2^-64 rounded to the nearest double (ties to even),
// the value __ull2double_rn(w) * 0x1p-64 has (the scaling is exact)
__device__ __forceinline__ double u64_scaled_2m64(unsigned long long w)
{
  if (w == 0) return 0.0;
  const int lz = __clzll(static_cast<long long>(w));
  const unsigned long long m = w << lz;  // leading one at bit 63
  unsigned long long hi = m >> 11;       // 53 significant bits
  const unsigned long long rem = m & 0x7FFull;
  if (rem > 0x400ull || (rem == 0x400ull && (hi & 1ull))) hi += 1;  // may carry to 2^53
  // value = 1.f x 2^(-1 - lz); the carry of hi into bit 53 bumps the exponent
  const unsigned long long e = static_cast<unsigned long long>(1023 - 1 - lz);
  return __longlong_as_double(static_cast<long long>((e << 52) + (hi - (1ull << 52))));
}

// double -> float rounded to nearest (ties to even), as __double2float_rn;
// results that are not normal floats (zero, subnormal, overflow, inf, NaN)
// take the hardware conversion
__device__ __forceinline__ float to_float(double x)
{
  const long long b = bits(x);
  const int e = static_cast<int>((b >> 52) & 0x7FF) - 1023 + 127;
  if (e < 1 || e > 254) return __double2float_rn(x);
  const unsigned long long mant = static_cast<unsigned long long>(b) & 0xFFFFFFFFFFFFFull;
  const unsigned r = static_cast<unsigned>(mant & 0x1FFFFFFFull);  // the 29 dropped bits
  unsigned f = (static_cast<unsigned>(e) << 23) | static_cast<unsigned>(mant >> 29);
  if (r > 0x10000000u || (r == 0x10000000u && (f & 1u))) f += 1;  // carries into the exponent (to inf at the top)
  if (b < 0) f |= 0x80000000u;
  return __uint_as_float(f);
}

// float -> double (exact); subnormal, inf and NaN floats take the hardware
// conversion
__device__ __forceinline__ double to_double(float x)
{
  const unsigned u = __float_as_uint(x);
  const unsigned e = (u >> 23) & 0xFFu;
  if ((u & 0x7FFFFFFFu) == 0) return (u >> 31) ? -0.0 : 0.0;
  if (e == 0 || e == 0xFFu) return static_cast<double>(x);
  const unsigned long long d = (static_cast<unsigned long long>(u >> 31) << 63) |
                               (static_cast<unsigned long long>(e - 127 + 1023) << 52) |
                               (static_cast<unsigned long long>(u & 0x7FFFFFu) << 29);
  return __longlong_as_double(static_cast<long long>(d));
}

// int -> double (exact)
__device__ __forceinline__ double to_double(int v)
{
  if (v == 0) return 0.0;
  const unsigned long long s = v < 0 ? (1ull << 63) : 0ull;
  const unsigned a = v < 0 ? 0u - static_cast<unsigned>(v) : static_cast<unsigned>(v);
  const int lz = __clz(static_cast<int>(a));
  const unsigned long long frac = static_cast<unsigned long long>(a << lz) & 0x7FFFFFFFull;  // below the leading one
  const unsigned long long e = static_cast<unsigned long long>(1023 + 31 - lz);
  return __longlong_as_double(static_cast<long long>(s | (e << 52) | (frac << 21)));
}

// i + 0.5 (exact): the odd integer 2i + 1 converted, its exponent lowered by one
__device__ __forceinline__ double half_odd(int i)
{
  return __longlong_as_double(bits(to_double(2 * i + 1)) - (1LL << 52));
}

// x - c with the subtraction skipped when c is +0 (x - (+0) == x for every x)
__device__ __forceinline__ double sub(double x, double c) { return bits(c) == 0 ? x : x - c; }

// min(a, b) as fmin for doubles that are not NaN (returns b when equal)
__device__ __forceinline__ double min(double a, double b) { return lt(a, b) ? a : b; }

}  // namespace fpi
}  // namespace omc
