// Oracle test infrastructure: C-linkage shim over the reference's own
// src/random_lcg.cpp and src/random_dist.cpp (compiled from the reference
// tree, never copied), so the oracle's restated prn/future_seed/init_seed and
// its Maxwell, Watt, normal and uniform samplers can be compared bit-for-bit;
// also the grid search lower_bound_index of include/openmc/search.h.
#include <cstdint>

#include "openmc/search.h"

namespace openmc {
double prn(uint64_t* seed);
uint64_t future_seed(uint64_t n, uint64_t seed);
uint64_t init_seed(int64_t id, int offset);
double uniform_distribution(double a, double b, uint64_t* seed);
}
// declared with C linkage by the reference (include/openmc/random_dist.h)
extern "C" double maxwell_spectrum(double T, uint64_t* seed);
extern "C" double watt_spectrum(double a, double b, uint64_t* seed);
extern "C" double normal_variate(double mean, double standard_deviation, uint64_t* seed);
extern "C" void openmc_set_seed(int64_t new_seed);
extern "C" void openmc_set_stride(uint64_t new_stride);

extern "C" {
double ref_prn(uint64_t* seed) { return openmc::prn(seed); }
uint64_t ref_future_seed(uint64_t n, uint64_t seed) { return openmc::future_seed(n, seed); }
int64_t ref_lower_bound_index(const double* first, int64_t n, double value)
{
  return openmc::lower_bound_index(first, first + n, value);
}
double ref_uniform(double a, double b, uint64_t* seed) { return openmc::uniform_distribution(a, b, seed); }
double ref_maxwell(double T, uint64_t* seed) { return maxwell_spectrum(T, seed); }
double ref_watt(double a, double b, uint64_t* seed) { return watt_spectrum(a, b, seed); }
double ref_normal(double mean, double sd, uint64_t* seed) { return normal_variate(mean, sd, seed); }
uint64_t ref_init_seed(int64_t id, int offset, int64_t master, uint64_t stride)
{
  openmc_set_seed(master);
  openmc_set_stride(stride);
  return openmc::init_seed(id, offset);
}
}
