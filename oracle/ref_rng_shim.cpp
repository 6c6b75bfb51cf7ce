// Oracle test infrastructure: C-linkage shim over the reference's own
// src/random_lcg.cpp (compiled from the reference tree, never copied), so the
// oracle's restated prn/future_seed/init_seed can be compared bit-for-bit.
#include <cstdint>

namespace openmc {
double prn(uint64_t* seed);
uint64_t future_seed(uint64_t n, uint64_t seed);
uint64_t init_seed(int64_t id, int offset);
}
extern "C" void openmc_set_seed(int64_t new_seed);
extern "C" void openmc_set_stride(uint64_t new_stride);

extern "C" {
double ref_prn(uint64_t* seed) { return openmc::prn(seed); }
uint64_t ref_future_seed(uint64_t n, uint64_t seed) { return openmc::future_seed(n, seed); }
uint64_t ref_init_seed(int64_t id, int offset, int64_t master, uint64_t stride)
{
  openmc_set_seed(master);
  openmc_set_stride(stride);
  return openmc::init_seed(id, offset);
}
}
