// Picks the transport build for a model's coordinate depth and table
// precision.  transport.cu is compiled three times: for at most 2 levels
// (omc::l2), whose per-level particle state then fits in registers, and for at
// most 4 levels (omc::l4), both with every FP64 multiply and add rounded
// separately (the reference's arithmetic, identical results in both); and for
// at most 2 levels with multiply-adds fused into FMAs (omc::l2f), which the
// FP32-table mode runs by default: it still computes positions, directions,
// distances and tallies in FP64, with one rounding per multiply-add instead
// of two, and its results are checked statistically against the FP64-table
// path rather than bit for bit.
#include <stdexcept>

#include "transport.h"

namespace omc {

struct GpuSim {
  int levels = 4;
  bool fused = false;  // the l2f build
  l2::GpuSim* g2 = nullptr;
  l4::GpuSim* g4 = nullptr;
  l2f::GpuSim* g2f = nullptr;
};

GpuSim* gpu_create(const HModel& m, const GpuOptions& opt)
{
  auto* g = new GpuSim();
  try {
    int want = opt.max_levels > 0 ? opt.max_levels : m.n_coord_levels;
    if (want < m.n_coord_levels) want = m.n_coord_levels;
    if (want <= 2 && opt.xs_fp32 && opt.contract) {
      g->levels = 2;
      g->fused = true;
      g->g2f = l2f::gpu_create(m, opt);
    } else if (want <= 2) {
      g->levels = 2;
      g->g2 = l2::gpu_create(m, opt);
    } else {
      g->levels = 4;
      g->g4 = l4::gpu_create(m, opt);
    }
  } catch (...) {
    delete g;
    throw;
  }
  return g;
}

void gpu_destroy(GpuSim* g)
{
  if (!g) return;
  if (g->g2) l2::gpu_destroy(g->g2);
  if (g->g4) l4::gpu_destroy(g->g4);
  if (g->g2f) l2f::gpu_destroy(g->g2f);
  delete g;
}

#define OMC_FORWARD(name, ...)                                                   \
  return g->fused ? l2f::name(g->g2f, ##__VA_ARGS__)                             \
                  : (g->levels == 2 ? l2::name(g->g2, ##__VA_ARGS__) : l4::name(g->g4, ##__VA_ARGS__))

BatchStats gpu_run_batch(GpuSim* g, HModel& m, int batch, bool accumulate)
{
  OMC_FORWARD(gpu_run_batch, m, batch, accumulate);
}

BatchStats gpu_run_batch_profiled(GpuSim* g, HModel& m, int batch, bool accumulate)
{
  OMC_FORWARD(gpu_run_batch_profiled, m, batch, accumulate);
}

void gpu_fetch_tallies(GpuSim* g, HModel& m) { OMC_FORWARD(gpu_fetch_tallies, m); }
void gpu_reset_tallies(GpuSim* g, HModel& m) { OMC_FORWARD(gpu_reset_tallies, m); }

void gpu_set_trace(GpuSim* g, long long n_hist, int cap, int batch, long long first)
{
  OMC_FORWARD(gpu_set_trace, n_hist, cap, batch, first);
}

void gpu_get_trace(GpuSim* g, void* records, int* counts) { OMC_FORWARD(gpu_get_trace, records, counts); }

void gpu_set_ww_bounds(GpuSim* g, const double* lower, const double* upper, long long n)
{
  OMC_FORWARD(gpu_set_ww_bounds, lower, upper, n);
}

void gpu_set_ww_on(GpuSim* g, bool on) { OMC_FORWARD(gpu_set_ww_on, on); }

void gpu_update_magic(GpuSim* g, const MagicArgs& a, double* lower, double* upper)
{
  OMC_FORWARD(gpu_update_magic, a, lower, upper);
}

GenerationStats gpu_finish_generation(GpuSim* g, int batch) { OMC_FORWARD(gpu_finish_generation, batch); }
void gpu_set_keff(GpuSim* g, double keff) { OMC_FORWARD(gpu_set_keff, keff); }
long long gpu_capacity(GpuSim* g) { OMC_FORWARD(gpu_capacity); }
int gpu_levels(GpuSim* g) { return g ? g->levels : 0; }

void gpu_material_xs(GpuSim* g, long long n, const int* mat, const double* E, double* total, double* absorption,
                     unsigned* grid_hash)
{
  OMC_FORWARD(gpu_material_xs, n, mat, E, total, absorption, grid_hash);
}

}  // namespace omc
