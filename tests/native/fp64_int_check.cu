// Self-check of openmc_gb300/csrc/fp64_int.cuh: every integer-pipe FP64
// compare and conversion against the hardware operation it replaces, on
// seeded random bit patterns plus special values (+-0, +-inf, NaN,
// subnormals, the largest and smallest normals, rounding ties).  Prints one
// line per function with its mismatch count; exits 1 on any mismatch.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../openmc_gb300/csrc/fp64_int.cuh"

using namespace omc;

__host__ __device__ inline unsigned long long mix(unsigned long long z)
{
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__device__ double pick_double(unsigned long long i)
{
  const unsigned long long h = mix(i);
  switch (i % 16) {
  case 0: {  // specials
    const double sp[] = {0.0, -0.0, INFINITY, -INFINITY, NAN, -NAN, 1.7976931348623157e308, 2.2250738585072014e-308,
                         4.9e-324, -4.9e-324, 1e-12, -1e-12, 1e-14, 0.5, 1.0, -1.0};
    return sp[(h >> 8) % 16];
  }
  case 1: return __longlong_as_double(static_cast<long long>(h));  // any bit pattern
  case 2: return __longlong_as_double(static_cast<long long>(h & 0x800FFFFFFFFFFFFFull));  // subnormals
  case 3: {  // doubles whose float rounding is a tie or near it
    const unsigned long long b = (h & 0xFFFFFFFFE0000000ull) | (((h >> 3) & 1) ? 0x10000000ull : 0x0FFFFFFFull);
    return __longlong_as_double(static_cast<long long>(b));
  }
  case 4: return __longlong_as_double(static_cast<long long>((h & 0x800FFFFFFFFFFFFFull) | (0x36Aull << 52)));  // near float subnormal range
  case 5: return __longlong_as_double(static_cast<long long>((h & 0x800FFFFFFFFFFFFFull) | (0x47Eull << 52)));  // near float max
  default: {  // ordinary magnitudes 1e-20 .. 1e20, both signs
    const double m = static_cast<double>(h >> 11) * 0x1p-53;
    const double e = static_cast<double>((h >> 3) % 41) - 20.0;
    return ((h & 1) ? -1.0 : 1.0) * m * pow(10.0, e);
  }
  }
}

struct Counts {
  unsigned long long cmp, sign, absc, u64, d2f, f2d, i2d, mn, half, sub;
};

__device__ bool same(double a, double b)
{
  if (isnan(a) && isnan(b)) return true;
  return __double_as_longlong(a) == __double_as_longlong(b);
}

__device__ bool samef(float a, float b)
{
  if (isnan(a) && isnan(b)) return true;
  return __float_as_uint(a) == __float_as_uint(b);
}

__global__ void check(unsigned long long n, Counts* c)
{
  for (unsigned long long i = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<unsigned long long>(gridDim.x) * blockDim.x) {
    const double a = pick_double(2 * i), b = (i % 7 == 0) ? a : pick_double(2 * i + 1);
    if (!isnan(a) && !isnan(b)) {
      if (fpi::lt(a, b) != (a < b) || fpi::le(a, b) != (a <= b) || fpi::eq(a, b) != (a == b))
        atomicAdd(&c->cmp, 1ull);
      if (!same(fpi::min(a, b), (a < b) ? a : b)) atomicAdd(&c->mn, 1ull);
    }
    if (fpi::neg(a) != (a < 0.0) || fpi::pos(a) != (a > 0.0) || fpi::zero(a) != (a == 0.0) ||
        fpi::nonneg(a) != (a >= 0.0))
      atomicAdd(&c->sign, 1ull);
    const double cs[] = {1e-12, 1e-14, 1e-10, 1e-5, 1.0, 1.7976931348623157e308, INFINITY};
    for (double k : cs)
      if (fpi::abs_lt(a, k) != (fabs(a) < k) || fpi::abs_gt(a, k) != (fabs(a) > k)) atomicAdd(&c->absc, 1ull);
    // generator words: random, small, and with rounding ties below the 53 kept bits
    const unsigned long long h = mix(3 * i + 7);
    unsigned long long w = h;
    if (i % 3 == 1) w = h >> (h % 64);
    if (i % 3 == 2) w = (h | 1ull << 63) & ~0x3FFull | ((h & 1) ? 0x400ull : 0xC00ull);
    if (!same(fpi::u64_scaled_2m64(w), __ull2double_rn(w) * 0x1p-64)) atomicAdd(&c->u64, 1ull);
    if (!samef(fpi::to_float(a), __double2float_rn(a))) atomicAdd(&c->d2f, 1ull);
    const float f = __uint_as_float(static_cast<unsigned>(h >> 32));
    if (!same(fpi::to_double(f), static_cast<double>(f))) atomicAdd(&c->f2d, 1ull);
    const int v = static_cast<int>(h);
    const int vs[] = {v, v >> (h % 31), 0, -1, 1, 2147483647, -2147483647 - 1};
    for (int x : vs)
      if (!same(fpi::to_double(x), static_cast<double>(x))) atomicAdd(&c->i2d, 1ull);
    const int hv[] = {v >> 2, (v >> 2) >> (h % 29), 0, -1, 1, 536870911, -536870912};
    for (int x : hv)
      if (!same(fpi::half_odd(x), x + 0.5)) atomicAdd(&c->half, 1ull);
    const double zs[] = {0.0, -0.0, b};
    for (double z : zs)
      if (!same(fpi::sub(a, z), a - z)) atomicAdd(&c->sub, 1ull);
  }
}

int main()
{
  Counts* d = nullptr;
  if (cudaMalloc(&d, sizeof(Counts)) != cudaSuccess) return 2;
  cudaMemset(d, 0, sizeof(Counts));
  const unsigned long long n = 1ull << 26;
  check<<<152 * 8, 256>>>(n, d);
  if (cudaDeviceSynchronize() != cudaSuccess) return 2;
  Counts c;
  cudaMemcpy(&c, d, sizeof(c), cudaMemcpyDeviceToHost);
  cudaFree(d);
  std::printf("samples %llu\ncompare %llu\nsign %llu\nabs %llu\nu64_scaled %llu\nto_float %llu\n"
              "float_to_double %llu\nint_to_double %llu\nmin %llu\nhalf_odd %llu\nsub %llu\n",
              n, c.cmp, c.sign, c.absc, c.u64, c.d2f, c.f2d, c.i2d, c.mn, c.half, c.sub);
  const unsigned long long bad = c.cmp + c.sign + c.absc + c.u64 + c.d2f + c.f2d + c.i2d + c.mn + c.half + c.sub;
  return bad ? 1 : 0;
}
