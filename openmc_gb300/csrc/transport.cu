// Event-based transport on one GB300: particle bank as structure-of-arrays in
// HBM, compacted event queues (warp ballot + one atomic per warp), optional
// counting sort of the cross-section queue by (material, energy octave), and
// one CUDA graph per batch whose conditional while-node runs event iterations
// until every history of the batch has ended.
//
// Kernel <-> reference mapping
//   k_source_bank sample_external_source src/source.cpp:355-415, 627-660 and
//                 the particle seeds of initialize_history
//                 src/simulation.cpp:573-616, for every history of the batch
//   k_refill      process_init_events  src/event.cpp:62-71 + initialize_history
//                 src/simulation.cpp:573-649 (or a waiting split particle)
//   k_xs          process_calculate_xs_events src/event.cpp:73-105 ->
//                 Particle::event_calculate_xs src/particle.cpp:160-230
//                 (by default inside k_advance)
//   k_advance     process_advance_particle_events src/event.cpp:107-128 ->
//                 Particle::event_advance src/particle.cpp:232-286 + track-length
//                 tallies src/tallies/tally_scoring.cpp:2416-2541 (+ by default
//                 the surface crossing, below)
//   k_surface     process_surface_crossing_events src/event.cpp:130-147 ->
//                 event_cross_surface src/particle.cpp:288-329 + revive
//   k_collision   process_collision_events src/event.cpp:149-166 ->
//                 event_collide src/particle.cpp:331-415 + collision-estimator
//                 tallies src/tallies/tally_scoring.cpp:2543-2600 + revive
//   k_tail        the history-based loop for the last histories of a batch
//   k_history     transport_history_based src/simulation.cpp:804-831
//   k_accumulate  Tally::accumulate src/tallies/tally.cpp:821-880
//
// Queues replace SharedArray::thread_safe_append (include/openmc/
// shared_array.h:71-89).  Dead slots are refilled from the batch's remaining
// source particles every iteration instead of running fixed sub-iterations of
// max_particles_in_flight; each history depends only on its own id-derived
// seeds, so the per-history physics is unchanged.
//
// Semantics kept from the history-based loop where the event-based loop of
// the reference differs only for particles that die inside advance (time
// cutoff, lost particle): their secondaries are still revived.
// Particle time is advanced only when a neutron time cutoff is set (nothing
// else on this path reads it; time filters are not supported).
//
// Every kernel that reads the cell, surface, universe or material tables
// sets the block's table pointers first (tables_enter, device.cuh); tally
// bins are incremented with warp-aggregated FP64 atomics (atomic_add_agg).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include <cooperative_groups.h>
#include <cooperative_groups/reduce.h>

#include "device.cuh"
#include "host_model.h"
#include "transport.h"

namespace omc {
namespace OMC_NS {

// --------------------------------------------------------------- helpers
__device__ __forceinline__ void warp_append(int* q, int* counter, int val, bool pred)
{
  unsigned m = __ballot_sync(0xffffffffu, pred);
  if (!m) return;
  int lane = threadIdx.x & 31;
  int leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(counter, __popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (pred) q[base + __popc(m & ((1u << lane) - 1u))] = val;
}

__device__ __forceinline__ int sort_key(int s);

// Appends slot s to the next cross-section queue, with its sort key when the
// queue is sorted (read here, right after the event wrote the particle's
// material and energy, instead of by both sort passes).
__device__ __forceinline__ void append_next(int s, bool pred)
{
  unsigned m = __ballot_sync(0xffffffffu, pred);
  if (!m) return;
  int lane = threadIdx.x & 31;
  int leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(&dq.cnt->n_next, __popc(m));
  base = __shfl_sync(0xffffffffu, base, leader);
  if (pred) {
    const int pos = base + __popc(m & ((1u << lane) - 1u));
    dq.q_tmp[pos] = s;
    if (dq.key_tmp) dq.key_tmp[pos] = sort_key(s);
  }
}

// Adds v over the warp with one atomic; all 32 lanes must call it.
__device__ __forceinline__ void warp_count(unsigned long long* ctr, unsigned v)
{
  unsigned sum = __reduce_add_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0 && sum) atomicAdd(ctr, static_cast<unsigned long long>(sum));
}

__device__ __forceinline__ bool traced(long long id)
{
  return dq.trace != nullptr && dq.batch == dq.trace_batch && id >= dq.trace_first &&
         id < dq.trace_first + dq.trace_hist;
}

// The trace record of an event after which the particle is dead without a
// crossing or a collision (event kind 0, weight 0).
__device__ __forceinline__ TraceRec* trace_slot(long long id);
__device__ __forceinline__ void trace_dead(long long pid)
{
  TraceRec* rec = trace_slot(pid);
  if (rec) {
    rec->kind = 0;
    rec->surface_or_nuclide = 0;
    rec->wgt = 0.0;
  }
  dq.trace_n[pid - dq.trace_first] += 1;
}

// Whether slot s holds a traced history (its id in pid); reads the id only
// while a trace is being recorded.
__device__ __forceinline__ bool traced_slot(long long s, long long& pid)
{
  if (dq.trace == nullptr || dq.batch != dq.trace_batch) return false;
  pid = db.id[s];
  return traced(pid);
}

__device__ __forceinline__ TraceRec* trace_slot(long long id)
{
  long long k = id - dq.trace_first;
  int n = dq.trace_n[k];
  if (n >= dq.trace_cap) return nullptr;
  return dq.trace + k * dq.trace_cap + n;
}

__device__ void set_error(int flag) { atomicOr(&dq.cnt->error, flag); }

__device__ void mark_lost(long long s)
{
  db.wgt[s] = 0.0;
  atomicAdd(&dq.cnt->n_lost, 1);
  atomicExch(reinterpret_cast<unsigned long long*>(&dq.cnt->lost_id), static_cast<unsigned long long>(db.id[s]));
}

// ------------------------------------------------------ mesh raytrace
// src/mesh.cpp:1328-1369 RegularMesh helpers
// ceil((r - lower_left) / width) decided in FP32: the quotient estimated as
// FP32(r - lower_left) x FP32(1 / width) (three roundings, relative error
// below 2e-7) settles the ceiling when it lies at least 1e-4 + 2e-6 |q| from
// an integer (and |q| < 2^20), i.e. when r is at least 1e-4 widths from a
// cell face.  Returns false otherwise.
__device__ __forceinline__ bool mesh_index_fp32(const DMesh& m, double r, int i, int& idx)
{
  const double t = r - m.ll[i];
  const float q32 = __fmul_rn(fpi::to_float(t), m.inv_width32[i]);
  const float fr = q32 - rintf(q32);
  if (fabsf(q32) < 1048576.0f && fabsf(fr) > 1e-4f + 2e-6f * fabsf(q32)) {
    idx = static_cast<int>(ceilf(q32));
    return true;
  }
  return false;
}

// ceil((r - lower_left) / width): FP32 where that is decided, else the FP64
// division.  The returned index equals the FP64 ceiling.
__device__ __forceinline__ int mesh_index_in_direction(const DMesh& m, double r, int i)
{
  int idx;
  if (mesh_index_fp32(m, r, i, idx)) return idx;
  return static_cast<int>(ceil((r - m.ll[i]) / m.width[i]));
}

__device__ __forceinline__ void mesh_get_indices(const DMesh& m, double x, double y, double z, int* ijk, bool& in_mesh)
{
  const double r[3] = {x, y, z};
  in_mesh = true;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (i >= m.ndim) break;
    ijk[i] = mesh_index_in_direction(m, r[i], i);
    if (ijk[i] < 1 || ijk[i] > m.shape[i]) in_mesh = false;
  }
}

__device__ __forceinline__ int mesh_bin(const DMesh& m, const int* ijk)
{
  switch (m.ndim) {
  case 1: return ijk[0] - 1;
  case 2: return (ijk[1] - 1) * m.shape[0] + ijk[0] - 1;
  default: return ((ijk[2] - 1) * m.shape[1] + (ijk[1] - 1)) * m.shape[0] + ijk[0] - 1;
  }
}

struct MeshDist {
  int next_index;
  bool max_surface;
  double distance;
};

__device__ __forceinline__ MeshDist mesh_dist(const DMesh& m, const int* ijk, int i, const double* r0, const double* u)
{
  MeshDist d;
  d.next_index = ijk[i];
  d.max_surface = true;
  d.distance = INFTY;
  if (fpi::abs_lt(u[i], FP_PRECISION)) return d;
  d.max_surface = fpi::pos(u[i]);
  // grid plane ll + j width with j converted to double on the integer pipe
  if (d.max_surface && (ijk[i] <= m.shape[i])) {
    d.next_index++;
    const double f = (m.ll[i] + fpi::to_double(ijk[i]) * m.width[i]) - r0[i];
    d.distance = f / u[i];
  } else if (!d.max_surface && (ijk[i] >= 1)) {
    d.next_index--;
    const double f = (m.ll[i] + fpi::to_double(ijk[i] - 1) * m.width[i]) - r0[i];
    d.distance = f / u[i];
  }
  return d;
}

// Index along one axis of the mesh cell that a point q widths from the mesh
// corner lies in, the point moving in direction uk: within 1e-6 (relative)
// of a face it counts as on the face and takes the cell ahead, which is what
// the reference's TINY_BIT nudge along u decides; elsewhere ceil(q).
__device__ __forceinline__ int mesh_cell_ahead(float q, float uk)
{
  q = fminf(fmaxf(q, -1.0e9f), 1.0e9f);
  const float j = rintf(q);
  if (fabsf(q - j) <= 1.0e-6f * fmaxf(1.0f, fabsf(q))) return static_cast<int>(j) + (uk > 0.0f ? 1 : 0);
  return static_cast<int>(ceilf(q));
}

// FP32-table mode track walk: src/mesh.cpp:999-1146 raytrace_mesh with the
// track's start taken relative to the mesh corner (one FP64 subtraction per
// axis) and everything after that in FP32: start cell, face distances
// (face - start) / u from the flight's reciprocal direction, segment
// fractions of the advance distance.  Each start is within an FP32 rounding
// of its distance from the corner (under 1e-5 cm at 200 cm from it), which
// is all the track length a face can move between two cells; a start on a
// face (a particle that has just crossed it) takes the cell ahead.  Tallies
// stay FP64 sums of FP64 flux x FP32 fraction.  Calls f(bin, fraction).
template<class F>
__device__ void mesh_bins_crossed_f32(const DMesh& m, const double* r0, const double* u, const double* inv_u,
  double track, F f)
{
  if (fpi::zero(track)) return;
  const int n = m.ndim;
  float t[3] = {0.0f, 0.0f, 0.0f}, uf[3] = {0.0f, 0.0f, 0.0f}, iu[3] = {0.0f, 0.0f, 0.0f};
  bool par[3] = {true, true, true};  // |u| below FP_PRECISION: no face ahead
  int ijk[3] = {0, 0, 0};
  bool in_mesh = true;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (k >= n) break;
    t[k] = fpi::to_float(r0[k] - m.ll[k]);
    uf[k] = fpi::to_float(u[k]);
    iu[k] = fpi::to_float(inv_u[k]);
    par[k] = fpi::abs_lt(u[k], FP_PRECISION);
    ijk[k] = mesh_cell_ahead(t[k] * m.inv_width32[k], uf[k]);
    in_mesh = in_mesh && ijk[k] >= 1 && ijk[k] <= m.shape[k];
  }
  if (fpi::lt(track, 2 * TINY_BIT)) {
    if (in_mesh) f(mesh_bin(m, ijk), 1.0);
    return;
  }
  const float D = fpi::to_float(track), inv_D = 1.0f / D;
  // distance from the start to the next face on axis k (INFINITY when
  // parallel or leaving the mesh) and the index beyond it
  float dist[3] = {INFINITY, INFINITY, INFINITY};
  int next[3] = {0, 0, 0};
  auto face = [&](int k) {
    next[k] = ijk[k];
    dist[k] = INFINITY;
    if (par[k]) return;
    if (uf[k] > 0.0f) {
      if (ijk[k] <= m.shape[k]) {
        next[k] = ijk[k] + 1;
        dist[k] = (static_cast<float>(ijk[k]) * m.width32[k] - t[k]) * iu[k];
      }
    } else if (ijk[k] >= 1) {
      next[k] = ijk[k] - 1;
      dist[k] = (static_cast<float>(ijk[k] - 1) * m.width32[k] - t[k]) * iu[k];
    }
  };
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (k < n) face(k);
  float traveled = 0.0f;
  for (int guard = 0; guard < 1 << 24; ++guard) {
    if (in_mesh) {
      int k = 0;
      float dk = dist[0];
      if (dist[1] < dk) { k = 1; dk = dist[1]; }
      if (dist[2] < dk) { k = 2; dk = dist[2]; }
      const float seg = fminf(dk, D) - traveled;
      f(mesh_bin(m, ijk), fpi::to_double(seg * inv_D));
      traveled = dk;
      if (D <= traveled) return;
#pragma unroll
      for (int kk = 0; kk < 3; ++kk) {
        if (kk != k) continue;
        ijk[kk] = next[kk];
        face(kk);
        in_mesh = ijk[kk] >= 1 && ijk[kk] <= m.shape[kk];
      }
    } else {
      // outside: move to the farthest face ahead on the axes that are out
      // of range; with none the track does not enter the mesh
      int k_max = -1;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (k >= n) break;
        if ((ijk[k] < 1 || ijk[k] > m.shape[k]) && dist[k] < INFINITY && dist[k] > traveled) {
          traveled = dist[k];
          k_max = k;
        }
      }
      if (k_max == -1 || traveled >= D) return;
      in_mesh = true;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (k >= n) break;
        ijk[k] = mesh_cell_ahead((t[k] + traveled * uf[k]) * m.inv_width32[k], uf[k]);
        in_mesh = in_mesh && ijk[k] >= 1 && ijk[k] <= m.shape[k];
      }
#pragma unroll
      for (int k = 0; k < 3; ++k)
        if (k < n) face(k);
    }
  }
}

// src/mesh.cpp:999-1146 raytrace_mesh/bins_crossed; calls f(bin, fraction).
// inv_u (FP32-table mode): the FP32 walk above, from the advance distance.
template<class F>
__device__ void mesh_bins_crossed(const DMesh& m, const double* r0, const double* r1, const double* u, F f,
  const double* inv_u = nullptr, double track = 0.0)
{
  if (inv_u) {
    mesh_bins_crossed_f32(m, r0, u, inv_u, track, f);
    return;
  }
  double dx = r1[0] - r0[0], dy = r1[1] - r0[1], dz = r1[2] - r0[2];
  const double total_distance = sqrt(dx * dx + dy * dy + dz * dz);
  if (fpi::zero(total_distance)) return;
  const int n = m.ndim;
  bool in_mesh;
  double traveled = 0.0;
  int ijk[3] = {0, 0, 0};
  mesh_get_indices(m, r0[0] + TINY_BIT * u[0], r0[1] + TINY_BIT * u[1], r0[2] + TINY_BIT * u[2], ijk, in_mesh);
  if (fpi::lt(total_distance, 2 * TINY_BIT)) {
    if (in_mesh) f(mesh_bin(m, ijk), 1.0);
    return;
  }
  // A track that ends in the in-mesh cell it starts in (most tracks of a mesh
  // as fine as the lattice): when the end point lies in that cell on every
  // axis at least 1e-4 widths from its faces (decided in FP32), the distance
  // from the start to each face ahead exceeds the track length by that
  // margin, so the walk below would score this cell once with fraction
  // total / total = 1 and stop.  Scored directly.  Tracks that end on a face
  // (a lattice boundary on the mesh) take the walk.
  if (in_mesh) {
    bool same = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (k >= n) break;
      int e = -1;
      same = same && mesh_index_fp32(m, r1[k], k, e) && e == ijk[k];
    }
    if (same) {
      f(mesh_bin(m, ijk), 1.0);
      return;
    }
  }
  // the per-axis arrays are indexed by unrolled compile-time axes only, so
  // that they stay in registers
  MeshDist dist[3];
  dist[0].distance = dist[1].distance = dist[2].distance = INFTY;
  dist[0].next_index = dist[1].next_index = dist[2].next_index = 0;
  dist[0].max_surface = dist[1].max_surface = dist[2].max_surface = true;
#pragma unroll
  for (int k = 0; k < 3; ++k)
    if (k < n) dist[k] = mesh_dist(m, ijk, k, r0, u);
  for (int guard = 0; guard < 1 << 24; ++guard) {
    if (in_mesh) {
      int k = 0;
      double dk = dist[0].distance;
      if (fpi::lt(dist[1].distance, dk)) { k = 1; dk = dist[1].distance; }
      if (fpi::lt(dist[2].distance, dk)) { k = 2; dk = dist[2].distance; }
      const double seg = fpi::min(dk, total_distance) - traveled;
      f(mesh_bin(m, ijk), seg / total_distance);
      traveled = dk;
      if (fpi::le(total_distance, traveled)) return;
#pragma unroll
      for (int kk = 0; kk < 3; ++kk) {
        if (kk != k) continue;
        ijk[kk] = dist[kk].next_index;
        dist[kk] = mesh_dist(m, ijk, kk, r0, u);
        in_mesh = ((ijk[kk] >= 1) && (ijk[kk] <= m.shape[kk]));
      }
    } else {
      int k_max = -1;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        if (k >= n) break;
        if ((ijk[k] < 1 || ijk[k] > m.shape[k]) && (dist[k].distance > traveled)) {
          traveled = dist[k].distance;
          k_max = k;
        }
      }
      if (k_max == -1) traveled += TINY_BIT;
      if (traveled >= total_distance) return;
      double t = traveled + TINY_BIT;
      mesh_get_indices(m, r0[0] + t * u[0], r0[1] + t * u[1], r0[2] + t * u[2], ijk, in_mesh);
#pragma unroll
      for (int k = 0; k < 3; ++k)
        if (k < n) dist[k] = mesh_dist(m, ijk, k, r0, u);
    }
  }
}

// Warp-aggregated FP64 atomic add (src/tallies/tally_scoring.cpp:1103-1106
// adds each score with its own atomic): the lanes that execute this call
// together and add to the same bin first combine their values, and one lane
// per distinct bin issues the atomic.  The sum of a bin is the same up to
// the order of FP64 additions, which atomics leave open anyway.
__device__ __forceinline__ void atomic_add_agg(double* p, double v)
{
  namespace cg = cooperative_groups;
  cg::coalesced_group active = cg::coalesced_threads();
  if (active.size() == 1) {
    atomicAdd(p, v);
    return;
  }
  cg::coalesced_group peers = cg::labeled_partition(active, reinterpret_cast<unsigned long long>(p));
  if (peers.size() == 1) {
    atomicAdd(p, v);
    return;
  }
  const double sum = cg::reduce(peers, v, cg::plus<double>());
  if (peers.thread_rank() == 0) atomicAdd(p, sum);
}

// Cells of the particle's coordinate levels (cell filters match any level).
struct LevelCells {
  int c[MAXL];
  int n;
};

// Offsets of the non-mesh filter bins of tally T for the particle's state
// (src/tallies/tally_scoring.cpp:31-139 FilterBinIter; the energy filter
// bins the pre-event energy E_last, src/tallies/filter_energy.cpp:59-80; a
// cell filter matches every level whose cell is a bin, filter_cell.cpp:
// 48-58; a material filter the particle's material, filter_material.cpp:
// 47-55).  Returns how many combinations there are (0: no bin matches);
// mesh_slot receives the position of the mesh filter or -1.
__device__ __forceinline__ int tally_offsets(const DTally& T, double E_last, const LevelCells& lc, int material,
  long long (&offs)[MAXL], int& mesh_slot)
{
  int n = 1;
  offs[0] = 0;
  mesh_slot = -1;
  for (int i = 0; i < T.nfilt; ++i) {
    const DFilter& F = dm.filt[T.filt[i]];
    const long long st = T.stride[i];
    if (F.type == 0) {
      mesh_slot = i;
    } else if (F.type == 1) {
      const double* b = dm.ebins + F.e_off;
      // non-negative doubles compare like their bit patterns (integer pipe)
      const long long kE = __double_as_longlong(E_last);
      if (!(kE >= __double_as_longlong(__ldg(b)) && kE <= __double_as_longlong(__ldg(b + F.nbins)))) return 0;
      const long long add = static_cast<long long>(lower_bound_index_pos(b, 0, F.nbins + 1, E_last)) * st;
      for (int k = 0; k < n; ++k) offs[k] += add;
    } else if (F.type == 4) {
      int hit = -1;
      for (int b = 0; b < F.nbins; ++b)
        if (dm.fids[F.i_off + b] == material) { hit = b; break; }
      if (hit < 0) return 0;
      for (int k = 0; k < n; ++k) offs[k] += hit * st;
    } else if (F.type == 3) {
      // at most one cell filter per tally, so n == 1 here
      const long long base = offs[0];
      int m = 0;
#pragma unroll
      for (int l = 0; l < MAXL; ++l) {
        if (l >= lc.n) break;
        for (int b = 0; b < F.nbins; ++b)
          if (dm.fids[F.i_off + b] == lc.c[l]) {
            if (m < MAXL) offs[m++] = base + b * st;
            break;
          }
      }
      if (m == 0) return 0;
      n = m;
    }
  }
  return n;
}

// src/tallies/tally_scoring.cpp:2416-2541 score_tracklength_tally with the
// flux, total and absorption scores of score_general_ce_nonanalog
// (:578-1106): flux = wgt x distance, mesh filters through the raytrace.
__device__ int score_tracklength(const double* r0, const double* r1, const double* u, double E_last,
  double wgt, double distance, double mt, double ma, const LevelCells& lc, int material,
  const double* inv_u = nullptr)
{
  double flux = wgt * distance;
  int n_seg = 0;
  for (int t = 0; t < dm.n_tally; ++t) {
    const DTally& T = dm.tally[t];
    if (T.estimator != 0) continue;
    long long offs[MAXL];
    int mesh_slot;
    const int n_off = tally_offsets(T, E_last, lc, material, offs, mesh_slot);
    double* val = dm.value + T.value_off;
    const int ns = T.nscore;
    auto add = [&](long long index, double weight) {
      for (int s = 0; s < ns; ++s) {
        double score;
        int sc = T.score[s];
        if (sc == 0) score = flux;
        else if (sc == 1) score = mt * flux;
        else score = ma * flux;
        atomic_add_agg(val + index * ns + s, score * weight);
      }
    };
    for (int o = 0; o < n_off; ++o) {
      const long long base = offs[o];
      if (mesh_slot < 0) {
        add(base, 1.0);
        ++n_seg;
      } else {
        const DMesh& M = dm.mesh[dm.filt[T.filt[mesh_slot]].mesh];
        const long long stride = T.stride[mesh_slot];
        mesh_bins_crossed(M, r0, r1, u, [&](int bin, double frac) {
          add(base + bin * stride, 1. * frac);
          ++n_seg;
        }, inv_u, distance);
      }
    }
  }
  return n_seg;
}

// src/tallies/tally_scoring.cpp:2543-2600 score_collision_tally, called
// after the collision (src/particle.cpp:361-364): flux = wgt_last /
// Sigma_t with the pre-collision cross sections, mesh filters bin the
// collision site (src/tallies/filter_mesh.cpp:40-70), energy filters the
// pre-collision energy.
__device__ void score_collision(const double* r, double E_last, double wgt_last, double mt, double ma,
  const LevelCells& lc, int material)
{
  if (mt <= 0.0) return;
  const double flux = wgt_last / mt;
  for (int t = 0; t < dm.n_tally; ++t) {
    const DTally& T = dm.tally[t];
    if (T.estimator != 1) continue;
    long long offs[MAXL];
    int mesh_slot;
    const int n_off = tally_offsets(T, E_last, lc, material, offs, mesh_slot);
    long long mesh_add = 0;
    if (mesh_slot >= 0 && n_off > 0) {
      const DMesh& M = dm.mesh[dm.filt[T.filt[mesh_slot]].mesh];
      int ijk[3] = {0, 0, 0};
      bool in_mesh;
      mesh_get_indices(M, r[0], r[1], r[2], ijk, in_mesh);
      if (!in_mesh) continue;
      mesh_add = static_cast<long long>(mesh_bin(M, ijk)) * T.stride[mesh_slot];
    }
    double* val = dm.value + T.value_off;
    const int ns = T.nscore;
    for (int o = 0; o < n_off; ++o) {
      const long long index = offs[o] + mesh_add;
      for (int s = 0; s < ns; ++s) {
        const int sc = T.score[s];
        const double score = sc == 0 ? flux : (sc == 1 ? mt * flux : ma * flux);
        atomic_add_agg(val + index * ns + s, score);
      }
    }
  }
}

// ------------------------------------------------------- weight windows
// src/weight_windows.cpp:375-411
__device__ bool get_weight_window(double x, double y, double z, double E, double& lower, double& upper)
{
  const DMesh& m = dm.mesh[dm.ww_mesh];
  int ijk[3] = {1, 1, 1};
  bool in_mesh;
  mesh_get_indices(m, x, y, z, ijk, in_mesh);
  if (!in_mesh) return false;
  if (E < dm.ww_e[0] || E > dm.ww_e[dm.ww_ne]) return false;
  int eb = lower_bound_index_pos(dm.ww_e, 0, dm.ww_ne + 1, E);
  long long nm = static_cast<long long>(m.shape[0]) * m.shape[1] * m.shape[2];
  long long k = eb * nm + mesh_bin(m, ijk);
  lower = dm.ww_lower[k];
  upper = dm.ww_upper[k];
  return lower >= 0.0;
}

// Banks n copies of a site on the slot's LIFO chain (Particle::split,
// src/particle.cpp:95-112).  Pool entries the slot has already revived are
// reused first (only this slot's thread touches its chains), so the pool
// bounds the secondaries banked at one time per slot, not those of a batch;
// the rest come from the pool's bump pointer.
// Split-to-slots mode: the n copies go to a global ring from which the
// refill step starts them in free slots, so that the particles of one split
// tree are tracked in parallel.  Copy k gets its own tracking seed, a
// splitmix64 hash of the parent's current seed and k (the reference instead
// continues each banked copy on the parent's stream after the parent dies,
// src/particle.cpp:417-473, which serialises the whole tree in one slot).
// Every copy still carries weight / n, so the estimator stays unbiased.
__device__ __forceinline__ unsigned long long split_seed(unsigned long long seed, int k)
{
  unsigned long long z = seed + static_cast<unsigned long long>(k + 1) * 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

__device__ void push_split_sites(long long s, int n, double wgt, const double* r, const double* u, double E,
  int surf, unsigned long long seed)
{
  const unsigned long long cap = static_cast<unsigned long long>(dq.cnt->split_cap);
  unsigned long long base = atomicAdd(&dq.cnt->split_tail, static_cast<unsigned long long>(n));
  atomicAdd(&dq.cnt->n_sec, n);
  // entries from refill_split_base on may still be read by the running
  // refill (the head only moves in the refill plan, which never runs
  // concurrently with a producer)
  if (base + n - dq.cnt->refill_split_base > cap) {
    set_error(ERR_SECONDARY_OVERFLOW);
    return;
  }
  for (int k = 0; k < n; ++k) {
    DSplitSite& d = dq.split[(base + k) % cap];
    d.r[0] = r[0]; d.r[1] = r[1]; d.r[2] = r[2];
    d.u[0] = u[0]; d.u[1] = u[1]; d.u[2] = u[2];
    d.E = E;
    d.wgt = wgt;
    d.wgt_born = db.wgt_born[s];
    d.wgt_ww_born = db.wgt_ww_born[s];
    d.ww_factor = db.ww_factor[s];
    d.time = dm.track_time ? db.time[s] : 0.0;
    d.seed = split_seed(seed, k);
    d.id = db.id[s];
    d.surf = surf;
    d.n_split = db.n_split[s];
  }
}

__device__ void push_secondaries(long long s, int n, double wgt, const double* r, const double* u, double E, int surf)
{
  if (n <= 0) return;
  int reuse = 0;
  for (int e = db.sec_free[s]; e >= 0 && reuse < n; e = dq.sec[e].prev) ++reuse;
  int base = 0;
  if (n > reuse) {
    base = atomicAdd(&dq.cnt->n_sec, n - reuse);
    if (base + (n - reuse) > dq.cnt->sec_cap) {
      set_error(ERR_SECONDARY_OVERFLOW);
      return;
    }
  }
  int top = db.sec_top[s];
  int fr = db.sec_free[s];
  for (int l = 0; l < n; ++l) {
    int e;
    if (fr >= 0) {
      e = fr;
      fr = dq.sec[e].prev;
    } else {
      e = base++;
    }
    DSecondary& d = dq.sec[e];
    d.r[0] = r[0]; d.r[1] = r[1]; d.r[2] = r[2];
    d.u[0] = u[0]; d.u[1] = u[1]; d.u[2] = u[2];
    d.E = E;
    d.wgt = wgt;
    d.time = dm.track_time ? db.time[s] : 0.0;
    d.surf = surf;
    d.prev = top;
    top = e;
  }
  db.sec_top[s] = top;
  db.sec_free[s] = fr;
}

// src/weight_windows.cpp:56-146 (wgt/seed passed in registers)
__device__ void apply_weight_windows(long long s, double& wgt, unsigned long long& seed, const double* r,
  const double* u, double E, int surface)
{
  if (!dm.ww_on) return;
  if (E <= 0 || wgt == 0.0) return;
  double lower = -1, upper = 1;
  bool valid = get_weight_window(r[0], r[1], r[2], E, lower, upper);
  double wgt_ww_born = db.wgt_ww_born[s];
  if (wgt_ww_born == -1.0) {
    wgt_ww_born = valid ? (lower + upper) / 2 : 1.0;
    db.wgt_ww_born[s] = wgt_ww_born;
  }
  if (!valid) return;
  double survival = lower * dm.ww_surv;
  double factor = db.wgt_born[s] / wgt_ww_born;
  lower *= factor;
  upper *= factor;
  survival *= factor;
  double weight = wgt;
  if (wgt < dm.ww_cut) {
    wgt = 0.0;
    return;
  }
  double ww_factor = db.ww_factor[s];
  if (ww_factor == 0.0 && dm.ww_mlb > 1.0 && wgt > lower * dm.ww_mlb) {
    ww_factor = wgt / (lower * dm.ww_mlb);
    db.ww_factor[s] = ww_factor;
  }
  if (ww_factor > 1.0) {
    lower *= ww_factor;
    upper *= ww_factor;
    survival *= ww_factor;
  }
  if (weight > upper) {
    int n_split_hist = db.n_split[s];
    if (n_split_hist >= dm.max_history_splits) return;
    double n_split = ceil(weight / upper);
    double max_split = dm.ww_max_split;
    n_split = fmin(n_split, max_split);
    db.n_split[s] = static_cast<int>(n_split_hist + n_split);
    int i_split = static_cast<int>(llround(n_split));
    if (dq.split) push_split_sites(s, i_split - 1, weight / n_split, r, u, E, surface, seed);
    else push_secondaries(s, i_split - 1, weight / n_split, r, u, E, surface);
    wgt = weight / n_split;
  } else if (weight <= lower) {
    double weight_survive = fmin(weight * dm.ww_max_split, survival);
    // src/physics_common.cpp:12-19
    if (weight_survive * prn(seed) < wgt) wgt = weight_survive;
    else wgt = 0.;
  }
}

// ------------------------------------------------------- source sampling
__device__ bool satisfies_spatial_constraints(double x, double y, double z)
{
  Geo g;
  g.n_coord = 1;
  coord_reset(g, 0);
  g.r[0][0] = x; g.r[0][1] = y; g.r[0][2] = z;
  g.u[0] = 0.0; g.u[1] = 0.0; g.u[2] = 1.0;
  g.surface = SURFACE_NONE;
  g.material = C_NONE;
  g.material_last = C_NONE;
  bool lost_outer = false;
  if (!exhaustive_find_cell(g, lost_outer)) return false;
  if (dm.dom_type < 0 || dm.n_dom == 0) return true;
  if (dm.dom_type == 1) {
    if (g.material == C_NONE) return false;
    int id = dm.mat_id[g.material];
    for (int k = 0; k < dm.n_dom; ++k) if (dm.dom_ids[k] == id) return true;
    return false;
  }
#pragma unroll
  for (int i = 0; i < MAXL; ++i) {
    if (i >= g.n_coord) break;
    int id = dm.dom_type == 0 ? dm.cell_id[g.cell[i]] : g.univ[i];
    for (int k = 0; k < dm.n_dom; ++k) if (dm.dom_ids[k] == id) return true;
  }
  return false;
}

// Unit direction from FP32 components, scaled in FP64 by the series
// 1 - eps/2 + 3 eps^2 / 8 of 1/sqrt(|u|^2), |u|^2 = 1 + eps (|eps| of order
// 1e-7), so that it is a unit vector to FP64 rounding.
__device__ __forceinline__ void unit_from_f32(const float* v, double* u)
{
  double d[3] = {fpi::to_double(v[0]), fpi::to_double(v[1]), fpi::to_double(v[2])};
  const double eps = (d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) - 1.0;
  const double f = 1.0 + eps * (-0.5 + 0.375 * eps);
  u[0] = d[0] * f;
  u[1] = d[1] * f;
  u[2] = d[2] * f;
}

__device__ double sample_energy(unsigned long long& seed)
{
  if (dm.en_type == 1) {
    if (dm.xs_fp32) {
      // FP32-table mode: src/random_dist.cpp:20-32 with the same three draws
      const float r1 = prn_f(seed), r2 = prn_f(seed), r3 = prn_f(seed);
      const float c = cospif(0.5f * r3);
      return fpi::to_double(-fpi::to_float(dm.en_x[0]) * (logf(r1) + logf(r2) * c * c));
    }
    return maxwell_spectrum(dm.en_x[0], seed);
  }
  int n = dm.n_en;
  if (n <= 1) return dm.en_x[0];
  // src/distribution.cpp:87-101 alias sampling
  int u = static_cast<int>(prn(seed) * n);
  if (prn(seed) < dm.en_prob[u]) return dm.en_x[u];
  return dm.en_x[dm.en_alias[u]];
}

// The source site of history index_source of the current batch
// (src/simulation.cpp:573-616 up to the particle seeds, src/source.cpp:
// 355-415): position, direction, energy, and the tracking-stream seed.
__device__ void sample_source_site(long long index_source, SourceSite& site)
{
  long long id = static_cast<long long>(dq.batch - 1) * dm.n_particles + index_source;
  unsigned long long seed = future_seed(static_cast<unsigned long long>(id) * dm.stride,
    static_cast<unsigned long long>(dm.master_seed + 1));
  double* r = site.r;
  double* u = site.u;
  double E;
  // src/source.cpp:355-415
  int tries = 0;
  for (;;) {
    if (dm.sp_type == 0) {
      r[0] = dm.sp[0]; r[1] = dm.sp[1]; r[2] = dm.sp[2];
    } else {
      double xi0 = prn(seed);
      double xi1 = prn(seed);
      double xi2 = prn(seed);
      r[0] = dm.sp[0] + xi0 * (dm.sp[3] - dm.sp[0]);
      r[1] = dm.sp[1] + xi1 * (dm.sp[4] - dm.sp[1]);
      r[2] = dm.sp[2] + xi2 * (dm.sp[5] - dm.sp[2]);
    }
    if (satisfies_spatial_constraints(r[0], r[1], r[2])) break;
    if (++tries > 1000000) {
      set_error(ERR_REJECTION);
      break;
    }
  }
  if (dm.an_type == 0 && dm.xs_fp32) {
    // FP32-table mode: the same two draws, the direction in FP32
    const float t = prn_f(seed);
    const float mu = 2.0f * prn_f(seed) - 1.0f;
    float sp, cp;
    sincospif(2.0f * t, &sp, &cp);
    const float st = sqrtf(fmaxf(0.0f, 1.0f - mu * mu));
    const float v[3] = {mu, st * cp, st * sp};
    unit_from_f32(v, u);
  } else if (dm.an_type == 0) {
    // src/distribution_multi.cpp:106-112
    double phi = uniform_distribution(0., 2.0 * PI, seed);
    double mu = uniform_distribution(-1., 1., seed);
    u[0] = mu;
    u[1] = sqrt(1.0 - mu * mu) * cos(phi);
    u[2] = sqrt(1.0 - mu * mu) * sin(phi);
  } else {
    u[0] = dm.uref[0]; u[1] = dm.uref[1]; u[2] = dm.uref[2];
  }
  tries = 0;
  for (;;) {
    E = sample_energy(seed);
    if (E < dm.e_max) break;
    if (++tries > 1000000) {
      set_error(ERR_REJECTION);
      break;
    }
  }
  site.E = E;
  site.tseed = future_seed(static_cast<unsigned long long>(id) * dm.stride,
    static_cast<unsigned long long>(dm.master_seed + 0));
}

// src/simulation.cpp:573-649 initialize_history (fixed source) into slot s.
// The site comes from the batch's source bank when one was sampled.
__device__ void initialize_history(long long s, long long index_source)
{
  SourceSite site;
  if (dq.src_n >= index_source) site = dq.src_bank[index_source - 1];
  else sample_source_site(index_source, site);
  const double* r = site.r;
  const double* u = site.u;
  const double E = site.E;
  // from_source (src/particle.cpp:114-158)
  const long long cap = db.cap;
  db.n_coord[s] = 1;
  for (int l = 0; l < MAXL; ++l) {
    long long k = l * cap + s;
    db.cell[k] = C_NONE;
    db.univ[k] = C_NONE;
    db.latt[k] = C_NONE;
    db.lix[k] = 0; db.liy[k] = 0; db.liz[k] = 0;
  }
  db.cell_last0[s] = C_NONE;
  db.cell_born[s] = C_NONE;
  db.surface[s] = SURFACE_NONE;
  db.material[s] = C_NONE;
  db.material_last[s] = C_NONE;
  db.n_collision[s] = 0;
  db.rx[s] = r[0]; db.ry[s] = r[1]; db.rz[s] = r[2];
  set_direction(s, u[0], u[1], u[2]);
  db.E[s] = E;
  // the default source time distribution is a point at 0; later
  // generations of an eigenvalue run start at their fission sites' times
  if (dm.track_time) db.time[s] = (dq.src_time && dq.src_n >= index_source) ? dq.src_time[index_source - 1] : 0.0;
  double wgt = 1.0;
  db.id[s] = index_source;
  db.n_event[s] = 0;
  db.n_split[s] = 0;
  db.ww_factor[s] = 0.0;
  db.wgt_born[s] = wgt;
  db.sec_top[s] = -1;
  unsigned long long tseed = site.tseed;
  db.wgt_ww_born[s] = -1.0;
  apply_weight_windows(s, wgt, tseed, r, u, E, SURFACE_NONE);
  db.wgt[s] = wgt;
  db.seed[s] = tseed;
  atomicAdd(&dq.cnt->total_weight, wgt);
  db.n_total[s] = 0;
  if (dm.eigen) {
    db.k_col[s] = db.k_abs[s] = db.k_tra[s] = 0.0;
    db.n_progeny[s] = 0;
  }
  if (traced(index_source)) dq.trace_n[index_source - dq.trace_first] = 0;
}

// Starts a split particle in slot s (split-to-slots mode): the slot takes
// the parent's state at the split (from_source, src/particle.cpp:114-158,
// with the split copy's weights and window state) and the copy's own seed.
__device__ void start_split_site(long long s, const DSplitSite& d)
{
  const long long cap = db.cap;
  db.n_coord[s] = 1;
  for (int l = 0; l < MAXL; ++l) {
    long long k = l * cap + s;
    db.cell[k] = C_NONE;
    db.univ[k] = C_NONE;
    db.latt[k] = C_NONE;
    db.lix[k] = 0; db.liy[k] = 0; db.liz[k] = 0;
  }
  db.cell_last0[s] = C_NONE;
  db.cell_born[s] = C_NONE;
  db.surface[s] = d.surf;
  db.material[s] = C_NONE;
  db.material_last[s] = C_NONE;
  db.n_collision[s] = 0;
  db.rx[s] = d.r[0]; db.ry[s] = d.r[1]; db.rz[s] = d.r[2];
  set_direction(s, d.u[0], d.u[1], d.u[2]);
  db.E[s] = d.E;
  db.wgt[s] = d.wgt;
  if (dm.track_time) db.time[s] = d.time;
  db.id[s] = d.id;
  db.n_event[s] = 0;
  db.n_split[s] = d.n_split;
  db.ww_factor[s] = d.ww_factor;
  db.wgt_born[s] = d.wgt_born;
  db.wgt_ww_born[s] = d.wgt_ww_born;
  db.sec_top[s] = -1;
  db.seed[s] = d.seed;
  db.n_total[s] = 0;
}

// src/particle.cpp:417-473 event_revive_from_secondary; returns alive.
// Dead slots without secondaries go back to the free list.
__device__ bool revive_or_free(long long s, double wgt)
{
  int ne = db.n_event[s] + 1;
  db.n_total[s] += 1;
  if (ne == dm.max_events) {
    wgt = 0.0;
    db.wgt[s] = 0.0;
  }
  db.n_event[s] = ne;
  if (!fpi::zero(wgt)) return true;
  int top = db.sec_top[s];
  if (top < 0) {
    unsigned long long key = (static_cast<unsigned long long>(db.n_total[s]) << 34) |
                             static_cast<unsigned long long>(db.id[s]);
    atomicMax(&dq.cnt->longest, key);
    if (dm.eigen) {
      // event_death (src/particle.cpp:475-512): the history's k-effective
      // scores into the generation's sums, its progeny count for the sort
      atomicAdd(&dq.cnt->k_abs, db.k_abs[s]);
      atomicAdd(&dq.cnt->k_col, db.k_col[s]);
      atomicAdd(&dq.cnt->k_tra, db.k_tra[s]);
      dq.progeny[db.id[s] - 1] = db.n_progeny[s];
    }
    if (!dq.history) {
      int k = atomicAdd(&dq.cnt->n_free, 1);
      dq.free_list[k] = static_cast<int>(s);
    }
    atomicAdd(reinterpret_cast<unsigned long long*>(&dq.cnt->n_done), 1ull);
    return false;
  }
  const DSecondary& site = dq.sec[top];
  db.sec_top[s] = site.prev;
  const long long cap = db.cap;
  db.n_coord[s] = 1;
  for (int l = 0; l < MAXL; ++l) {
    long long k = l * cap + s;
    db.cell[k] = C_NONE;
    db.univ[k] = C_NONE;
    db.latt[k] = C_NONE;
    db.lix[k] = 0; db.liy[k] = 0; db.liz[k] = 0;
  }
  db.cell_last0[s] = C_NONE;
  db.cell_born[s] = C_NONE;
  db.surface[s] = site.surf;
  db.material[s] = C_NONE;
  db.n_collision[s] = 0;
  db.wgt[s] = site.wgt;
  db.rx[s] = site.r[0]; db.ry[s] = site.r[1]; db.rz[s] = site.r[2];
  set_direction(s, site.u[0], site.u[1], site.u[2]);
  db.E[s] = site.E;
  if (dm.track_time) db.time[s] = site.time;
  db.n_event[s] = 0;
  // the revived entry joins the slot's free chain
  dq.sec[top].prev = db.sec_free[s];
  db.sec_free[s] = top;
  return true;
}

// ================================================================ kernels
// Samples every source site of the batch at full occupancy.  Sampling a site
// is a long dependent chain (two seed skip-aheads, rejection sampling against
// the domain constraint, energy sampling); done at refill time it ran as
// small, latency-bound launches every iteration.
__global__ void __launch_bounds__(256) k_source_bank()
{
  // an eigenvalue run's later generations start from the combed fission bank
  if (dq.src_from_bank) return;
  tables_enter();
  const long long n = dq.src_n;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    SourceSite site;
    sample_source_site(i + 1, site);
    dq.src_bank[i] = site;
  }
}

__global__ void k_batch_init(int batch)
{
  long long cap = db.cap;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < cap;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    dq.free_list[i] = static_cast<int>(i);
    db.sec_free[i] = -1;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    DCounters* c = dq.cnt;
    c->n_q = c->n_surf = c->n_coll = c->n_next = 0;
    c->n_free = static_cast<int>(cap);
    c->next_source = 1;
    c->n_done = 0;
    c->n_sec = 0;
    c->split_head = 0;
    c->split_tail = 0;
    c->refill_split_base = 0;
    c->refill_split = 0;
    c->iter = 0;
    c->total_weight = 0.0;
    c->leakage = 0.0;
    c->n_events = 0;
    c->error = 0;
    c->n_lost = 0;
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 7; ++b) c->stat[a][b] = 0;
    c->n_refill = 0;
    c->more = 1;
    c->tail = 0;
    c->longest = 0;
    c->n_fission = 0;
    c->fbank_full = 0;
    c->k_col = c->k_abs = c->k_tra = 0.0;
  }
  (void)batch;
}

// ------------------------------------------------- per-particle events
// Each event function works on one slot of the bank and is shared by the
// queue kernels (one event per launch) and the tail kernel (whole histories).
enum Next { NEXT_DEAD = 0, NEXT_XS = 1, NEXT_SURF = 2, NEXT_COLL = 3 };

struct EvStats {
  unsigned xs_ev, calc, nuc, seg, coll_nuc, surf, coll;
};

// src/particle.cpp:160-230 event_calculate_xs.  h: the slot's hot record
// held by the caller, kept up to date with what this event stores.
__device__ void ev_xs(long long s, EvStats& st, BankHot* h = nullptr)
{
  st.xs_ev += 1;
  long long pid = 0;
  const bool tr = traced_slot(s, pid);
  int lvl0 = db.n_coord[s] - 1;
  int low_cell = db.cell[lvl0 * db.cap + s];
  int material = db.material[s];
  int material_last = db.material_last[s];
  if (low_cell == C_NONE) {
    Geo g;
    geo_load(g, s);
    bool lost_outer = false;
    if (!exhaustive_find_cell(g, lost_outer)) {
      mark_lost(s);
      if (h) h->wgt = 0.0;
      return;
    }
    if (db.cell_born[s] == C_NONE) db.cell_born[s] = lvl_get(g.cell, g.n_coord - 1);
    db.cell_last0[s] = g.cell[0];
    geo_store(g, s);
    material = g.material;
    material_last = g.material_last;
    low_cell = lvl_get(g.cell, g.n_coord - 1);
  }
  uint32_t hash = 0xffffffffu;
  double E = db.E[s];
  if (material != C_NONE) {
    if (material != material_last || tr) {
      double t, a, nf = 0.0;
      hash = material_xs(material, E, t, a, dm.eigen ? &nf : nullptr);
      db.macro_t[s] = t;
      db.macro_a[s] = a;
      if (h) {
        h->macro_t = t;
        h->macro_a = a;
      }
      if (dm.eigen) db.macro_nf[s] = nf;
      st.calc += 1;
      st.nuc += s_tabs.mat_off[material + 1] - s_tabs.mat_off[material];
    }
  } else {
    db.macro_t[s] = 0.0;
    db.macro_a[s] = 0.0;
    if (h) h->macro_t = h->macro_a = 0.0;
    if (dm.eigen) db.macro_nf[s] = 0.0;
  }
  if (tr) {
    TraceRec* rec = trace_slot(pid);
    if (rec) {
      rec->cell = low_cell;
      rec->material = material;
      rec->grid_hash = static_cast<int32_t>(hash);
      rec->n_coord = db.n_coord[s];
      rec->E = E;
    }
  }
}

// src/particle.cpp:232-286 event_advance (+ track-length tallies)
// -log(xi) / Sigma_t (src/particle.cpp:243).  With FP32 tables Sigma_t
// carries FP32 precision, and the logarithm is taken in FP32 too: of 1 - xi
// through log1pf for xi > 1/2 (no cancellation near xi = 1), of xi itself
// down to 2^-20, and in FP64 below (so that small xi keep finite, exact
// tails); the distance is then FP32-accurate like Sigma_t.  FP64 tables
// keep the reference's FP64 expression.
__device__ __forceinline__ double collision_distance(double xi, double mt)
{
  if (!dm.xs_fp32) return -log(xi) / mt;
  // xi in [0, 1): compared as bit patterns; conversions on the integer pipe
  float lg;
  if (fpi::bits(xi) > fpi::bits(0.5)) lg = log1pf(-fpi::to_float(1.0 - xi));
  else if (fpi::bits(xi) >= fpi::bits(0x1p-20)) lg = logf(fpi::to_float(xi));
  else lg = static_cast<float>(log(xi));
  return fpi::to_double(-lg / fpi::to_float(mt));
}

__device__ int ev_surface_g(long long s, EvStats& st, Geo& g, double wgt, int bsurf, int trans, int blevel);

// src/particle.cpp:46-73 Particle::speed for a neutron of energy E (eV), cm/s
__device__ __forceinline__ double neutron_speed(double E)
{
  return C_LIGHT * sqrt(E * (E + 2 * MASS_NEUTRON_EV)) / (E + MASS_NEUTRON_EV);
}

// with_surf: a particle that reaches the boundary crosses it right away from
// the registers (the surface event always follows such an advance), instead
// of storing its state for a surface pass to reload.
// defer: the track-length tallies are not scored here; the flight is written
// as a track record at the event's queue position qi for k_score_tracks.
// hp: the slot's hot record as the caller holds it (after an XS event in the
// same thread), else it is loaded here.
// may_time false: built for runs without a time cutoff (the time code is
// left out of the build rather than skipped at run time, for registers).
template<bool with_surf, bool defer = false, bool may_time = true>
__device__ int ev_advance(long long s, EvStats& st, int qi = 0, const BankHot* hp = nullptr)
{
  const BankHot h = hp ? *hp : db.hot[s];
  double wgt = h.wgt;
  if (fpi::zero(wgt)) {
    // lost in the cross-section event: no flight (its trace record has no
    // event kind)
    if (defer && dq.trk.w) dq.trk.w[qi] = 0.0;  // no record
    long long pid;
    if (traced_slot(s, pid)) trace_dead(pid);
    return revive_or_free(s, wgt) ? NEXT_XS : NEXT_DEAD;
  }
  Geo g;
  geo_load(g, s);
  double bd;
  int bs, bl, bt;
  bool neg_lat = false;
  // FP32-table mode: reciprocal direction shared by the lattice and mesh
  // distances (FP64 products in place of FP64 quotients).  Recomputed per
  // flight: keeping it in the bank with the direction measured 5 % slower
  // (three more scattered loads cost more than three FP64 divisions).
  // The reciprocals come from one division: with a = 1 - uz^2 (the z-
  // cylinders' coefficient) and p = ux uy uz a, 1/ux = (uy uz a) / p and so
  // on (a few ulps, against three or four correctly rounded quotients);
  // separate divisions when p is zero or tiny.
  double inv_u[4];
  const bool recip = dm.xs_fp32 != 0;
  if (recip) {
    const double ux = g.u[0], uy = g.u[1], uz = g.u[2];
    const double a = 1.0 - uz * uz;
    const double xy = ux * uy, za = uz * a;
    const double p = xy * za;
    if (fpi::abs_gt(p, 0x1p-900)) {
      const double q = 1.0 / p;
      inv_u[0] = q * (uy * za);
      inv_u[1] = q * (ux * za);
      inv_u[2] = q * (xy * a);
      inv_u[3] = q * (xy * uz);
    } else {
      inv_u[0] = 1.0 / ux;
      inv_u[1] = 1.0 / uy;
      inv_u[2] = 1.0 / uz;
      inv_u[3] = 1.0 / a;
    }
  }
  distance_to_boundary(g, bd, bs, bl, bt, neg_lat, recip ? inv_u : nullptr);
  if (neg_lat) mark_lost(s);
  unsigned long long seed = h.seed;
  double mt = h.macro_t;
  double dcoll = fpi::zero(mt) ? __longlong_as_double(0x7ff0000000000000LL) : collision_distance(prn(seed), mt);
  // src/particle.cpp:246-259: the distance the time cutoff leaves, at the
  // speed of the particle's energy (INFTY without a cutoff); the particle
  // moves the least of the three distances and its time advances by
  // distance / speed
  // (the speed is formed again for the time update rather than kept, to
  // hold fewer registers across the flight when no cutoff is set)
  const bool timed = may_time && dm.track_time;
  double d_cut = INFTY;
  if (timed) d_cut = (dm.time_cutoff - db.time[s]) * neutron_speed(g.E);
  double distance = bd;
  if (fpi::lt(dcoll, distance)) distance = dcoll;
  if (fpi::lt(d_cut, distance)) distance = d_cut;
  if (timed) db.time[s] = db.time[s] + distance / neutron_speed(g.E);
  double r0[3] = {g.r[0][0], g.r[0][1], g.r[0][2]};
#pragma unroll
  for (int l = 0; l < MAXL; ++l) {
    if (l >= g.n_coord) break;
    g.r[l][0] = g.r[l][0] + distance * g.u[0];
    g.r[l][1] = g.r[l][1] + distance * g.u[1];
    g.r[l][2] = g.r[l][2] + distance * g.u[2];
  }
  // track-length estimate of k-effective (src/particle.cpp:272-275)
  if (dm.eigen) db.k_tra[s] += wgt * distance * db.macro_nf[s];
  if (defer && dq.trk.w) {
    const DTracks& T = dq.trk;
    T.r0x[qi] = r0[0];
    T.r0y[qi] = r0[1];
    T.r0z[qi] = r0[2];
    T.ux[qi] = g.u[0];
    T.uy[qi] = g.u[1];
    T.uz[qi] = g.u[2];
    if (recip) {
      T.iux[qi] = inv_u[0];
      T.iuy[qi] = inv_u[1];
      T.iuz[qi] = inv_u[2];
    }
    T.d[qi] = distance;
    T.w[qi] = wgt;
    T.E[qi] = g.E;
    if (dm.trk_xs) {
      T.mt[qi] = mt;
      T.ma[qi] = h.macro_a;
    }
    if (dm.trk_mat) T.mat[qi] = g.material;
    if (dm.trk_cells) {
#pragma unroll
      for (int l = 0; l < MAXL; ++l) T.cell[l * db.cap + qi] = l < g.n_coord ? g.cell[l] : C_NONE;
    }
  } else if (!defer && dm.n_tally_tracklength > 0) {
    LevelCells lc;
#pragma unroll
    for (int l = 0; l < MAXL; ++l) lc.c[l] = g.cell[l];
    lc.n = g.n_coord;
    st.seg += score_tracklength(r0, g.r[0], g.u, g.E, wgt, distance, mt, h.macro_a, lc, g.material,
      recip ? inv_u : nullptr);
  }
  if (neg_lat) wgt = 0.0;  // mark_lost zeroed the stored weight
  // killed at the time cutoff, or lost to infinity without one
  if (fpi::eq(distance, d_cut)) {
    wgt = 0.0;
    db.wgt[s] = 0.0;
  }
  db.seed[s] = seed;
  long long pid;
  if (traced_slot(s, pid)) {
    TraceRec* rec = trace_slot(pid);
    if (rec) rec->dist = distance;
    if (fpi::zero(wgt)) trace_dead(pid);  // died in the flight (time cutoff, lost)
  }
  const bool cross = !fpi::zero(wgt) && fpi::lt(bd, dcoll);
  if (with_surf && cross) return ev_surface_g(s, st, g, wgt, bs, bt, bl);
  const long long cap = db.cap;
#pragma unroll
  for (int l = 0; l < MAXL; ++l) {
    if (l >= g.n_coord) break;
    long long k = l * cap + s;
    db.rx[k] = g.r[l][0];
    db.ry[k] = g.r[l][1];
    db.rz[k] = g.r[l][2];
  }
  if (cross) {
    db.bsurf[s] = bs;
    db.blevel[s] = bl;
    db.btrans[s] = bt;
    return NEXT_SURF;
  }
  if (!fpi::zero(wgt)) return NEXT_COLL;
  return revive_or_free(s, wgt) ? NEXT_XS : NEXT_DEAD;
}

// src/geometry.cpp:301-357 cross_lattice up to its cell search: the lattice
// index moves by the translation, the local position is recomputed, and
// the universe of the new lattice element is looked up.  Returns whether
// the new index lies inside the lattice.
__device__ bool lattice_step(Geo& g, int trans)
{
  const int lvl_rt = g.n_coord - 1;  // a lattice level is never the root
  bool valid = false;
#pragma unroll
  for (int lvl = 1; lvl < MAXL; ++lvl) {
    if (lvl != lvl_rt) continue;
    const DLattice& lat = dm.lat[g.lat[lvl]];
    g.li[lvl][0] += trans % 3 - 1;
    g.li[lvl][1] += (trans / 3) % 3 - 1;
    g.li[lvl][2] += trans / 9 - 1;
    const int up = lvl - 1;
    const DCell& cell = s_tabs.cell[g.cell[up]];
    g.r[lvl][0] = fpi::sub(g.r[up][0], cell.tr[0]);
    g.r[lvl][1] = fpi::sub(g.r[up][1], cell.tr[1]);
    g.r[lvl][2] = fpi::sub(g.r[up][2], cell.tr[2]);
    lattice_local_position(lat, g.r[lvl][0], g.r[lvl][1], g.r[lvl][2], g.li[lvl]);
    valid = lattice_valid(lat, g.li[lvl]);
    if (valid) {
      g.univ[lvl] = dm.lat_univ[lat.univ_off + lat.n[0] * lat.n[1] * g.li[lvl][2] + lat.n[0] * g.li[lvl][1] + g.li[lvl][0]];
      g.cell[lvl] = C_NONE;
    }
  }
  return valid;
}

// src/particle.cpp:288-329, 549-710 event_cross_surface (+ revive)
// The crossing itself on a particle state already held in registers (g, at
// the boundary), with the boundary the advance found: signed surface bsurf,
// lattice translation trans and coordinate level blevel.  A lattice
// crossing (src/geometry.cpp:301-357), a reflection (src/particle.cpp:
// 657-710) and a transmission through a surface (src/particle.cpp:600-629)
// each prepare the state their own way and then run one shared cell search
// from the crossing level (so that the lanes of a warp take it together);
// each keeps its own fallbacks when that search fails.
__device__ int ev_surface_g(long long s, EvStats& st, Geo& g, double wgt, int bsurf, int trans, int blevel)
{
  st.surf += 1;
  db.cell_last0[s] = g.cell[0];
  g.surface = bsurf;
  g.n_coord = blevel;
  bool lost_outer = false;
  enum { NONE, LATTICE, REFLECT, TRANSMIT };
  int path = NONE;
  if (trans != 13) {
    if (!lattice_step(g, trans)) {
      g.n_coord = 1;
      if (!exhaustive_find_cell(g, lost_outer)) {
        mark_lost(s);
        wgt = 0.0;
      }
    } else {
      path = LATTICE;
      // exhaustive_find_cell from the new element (src/geometry.cpp:284-298)
      if (lvl_get(g.univ, g.n_coord - 1) == C_NONE) {
        g.univ[0] = dm.root_univ;
        g.n_coord = 1;
      }
    }
  } else if (g.surface == SURFACE_NONE || abs(g.surface) > dm.n_surf) {
    mark_lost(s);
    wgt = 0.0;
  } else {
    const DSurface& surf = s_tabs.surf[abs(g.surface) - 1];
    if (surf.bc == 1) {
      // src/particle.cpp:631-655
      atomicAdd(&dq.cnt->leakage, wgt);
      wgt = 0.0;
      db.wgt[s] = 0.0;
    } else if (surf.bc == 2) {
      // src/boundary_condition.cpp:38-47 + src/particle.cpp:657-710
      double nx, ny, nz;
      surf_normal(surf, g.r[0][0], g.r[0][1], g.r[0][2], nx, ny, nz);
      double ux = g.u[0], uy = g.u[1], uz = g.u[2];
      const double projection = nx * ux + ny * uy + nz * uz;
      const double magnitude = nx * nx + ny * ny + nz * nz;
      const double fac = 2.0 * projection / magnitude;
      ux = ux - nx * fac;
      uy = uy - ny * fac;
      uz = uz - nz * fac;
      double norm = sqrt(ux * ux + uy * uy + uz * uz);
      ux /= norm;
      uy /= norm;
      uz /= norm;
      if (g.n_coord != 1) {
        mark_lost(s);
        wgt = 0.0;
      } else {
        g.u[0] = ux; g.u[1] = uy; g.u[2] = uz;
        g.cell[0] = db.cell_last0[s];
        g.surface = -g.surface;
        g.n_coord = 1;
        path = REFLECT;
      }
    } else {
      path = TRANSMIT;  // neighbour search at the crossing level, then from the root
    }
  }
  if (path != NONE && !find_cell_inner(g, lost_outer)) {
    if (path == REFLECT) {
      mark_lost(s);
      wgt = 0.0;
    } else {
      g.n_coord = 1;
      if (!exhaustive_find_cell(g, lost_outer)) {
        if (path == LATTICE) {
          mark_lost(s);
          wgt = 0.0;
        } else {
          g.surface = SURFACE_NONE;
          g.n_coord = 1;
          g.r[0][0] = g.r[0][0] + TINY_BIT * g.u[0];
          g.r[0][1] = g.r[0][1] + TINY_BIT * g.u[1];
          g.r[0][2] = g.r[0][2] + TINY_BIT * g.u[2];
          if (!exhaustive_find_cell(g, lost_outer)) {
            mark_lost(s);
            wgt = 0.0;
          }
        }
      }
    }
  }
  geo_store(g, s);
  long long pid;
  if (traced_slot(s, pid)) {
    TraceRec* rec = trace_slot(pid);
    if (rec) {
      rec->kind = 1;
      rec->surface_or_nuclide = bsurf;
      rec->wgt = wgt;
    }
    dq.trace_n[pid - dq.trace_first] += 1;
  }
  return revive_or_free(s, wgt) ? NEXT_XS : NEXT_DEAD;
}

__device__ int ev_surface(long long s, EvStats& st)
{
  Geo g;
  geo_load(g, s);
  return ev_surface_g(s, st, g, db.wgt[s], db.bsurf[s], db.btrans[s], db.blevel[s]);
}

// src/physics.cpp:990-1041
__device__ void sample_cxs_target_velocity(double awr, double E, const double* u, double kT,
  unsigned long long& seed, double* vt_out)
{
  double beta_vn = sqrt(awr * E / kT);
  double alpha = 1.0 / (1.0 + sqrt(PI) * beta_vn / 2.0);
  double beta_vt_sq = 0.0;
  double mu = 0.0;
  for (int it = 0;; ++it) {
    double r1 = prn(seed);
    double r2 = prn(seed);
    if (prn(seed) < alpha) {
      beta_vt_sq = -log(r1 * r2);
    } else {
      double c = cos(PI / 2.0 * prn(seed));
      beta_vt_sq = -log(r1) - log(r2) * c * c;
    }
    double beta_vt = sqrt(beta_vt_sq);
    mu = uniform_distribution(-1., 1., seed);
    double accept_prob = sqrt(beta_vn * beta_vn + beta_vt_sq - 2 * beta_vn * beta_vt * mu) / (beta_vn + beta_vt);
    if (prn(seed) < accept_prob) break;
    if (it > 1000000) {
      set_error(ERR_REJECTION);
      break;
    }
  }
  double vt = sqrt(beta_vt_sq * kT / awr);
  double x = u[0], y = u[1], z = u[2];
  rotate_angle(x, y, z, mu, seed);
  vt_out[0] = vt * x;
  vt_out[1] = vt * y;
  vt_out[2] = vt * z;
}

// src/physics.cpp:990-1041 in FP32 (FP32-table mode): the target nucleus's
// velocity, a random variate that only enters the neutron's FP64 kinematics.
// The same draws in the same order as sample_cxs_target_velocity, each an
// FP32 uniform from prn_f; cos(pi/2 r) through cospif; the target direction
// rotated by rotate_angle_f.
__device__ void sample_cxs_target_velocity_f(float awr, float E, const float* u, float kT,
  unsigned long long& seed, float* vt_out)
{
  const float beta_vn = sqrtf(awr * E / kT);
  const float alpha = 1.0f / (1.0f + 0.886226925f * beta_vn);  // sqrt(pi) / 2
  float beta_vt_sq = 0.0f;
  float mu = 0.0f;
  for (int it = 0;; ++it) {
    const float r1 = prn_f(seed);
    const float r2 = prn_f(seed);
    if (prn_f(seed) < alpha) {
      beta_vt_sq = -logf(r1 * r2);
    } else {
      const float c = cospif(0.5f * prn_f(seed));
      beta_vt_sq = -logf(r1) - logf(r2) * c * c;
    }
    const float beta_vt = sqrtf(beta_vt_sq);
    mu = 2.0f * prn_f(seed) - 1.0f;
    const float accept_prob =
      sqrtf(fmaxf(0.0f, beta_vn * beta_vn + beta_vt_sq - 2.0f * beta_vn * beta_vt * mu)) / (beta_vn + beta_vt);
    if (prn_f(seed) < accept_prob) break;
    if (it > 1000000) {
      set_error(ERR_REJECTION);
      break;
    }
  }
  const float vt = sqrtf(beta_vt_sq * kT / awr);
  float x = u[0], y = u[1], z = u[2];
  rotate_angle_f(x, y, z, mu, seed);
  vt_out[0] = vt * x;
  vt_out[1] = vt * y;
  vt_out[2] = vt * z;
}

// Elastic scattering in FP32-table mode: src/physics.cpp:754-818 with the
// same draws in the same order, the centre-of-mass transformation and the
// rotation in FP32 (the target velocity is the FP32 variate of
// sample_cxs_target_velocity_f; the cosine mu_cm the same FP64 uniform,
// rounded).  The outgoing energy is the FP32 result; the outgoing direction,
// |u|^2 = 1 + eps with |eps| of order 1e-7 after the conversion, is scaled in
// FP64 by 1 - eps/2 + 3 eps^2 / 8 (the series of 1/sqrt(1 + eps), error of
// order eps^3), so that it is a unit vector to FP64 rounding: the distance to
// a z-cylinder takes 1 - uz^2 for ux^2 + uy^2.
__device__ void elastic_scatter_f(int nuc, double& E, double* u, unsigned long long& seed)
{
  const double awr_d = dm.awr[nuc], kT_d = dm.kT[nuc];
  const float awr = fpi::to_float(awr_d);
  const float Ef = fpi::to_float(E);
  const float uf[3] = {fpi::to_float(u[0]), fpi::to_float(u[1]), fpi::to_float(u[2])};
  float vel = sqrtf(Ef);
  float vn[3] = {vel * uf[0], vel * uf[1], vel * uf[2]};
  float vt[3] = {0.0f, 0.0f, 0.0f};
  if (!(fpi::le(400.0 * kT_d, E) && fpi::lt(1.0, awr_d)))
    sample_cxs_target_velocity_f(awr, Ef, uf, fpi::to_float(kT_d), seed, vt);
  const float iw = 1.0f / (awr + 1.0f);
  float vcm[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    vcm[k] = (vn[k] + awr * vt[k]) * iw;
    vn[k] = vn[k] - vcm[k];
  }
  vel = sqrtf(vn[0] * vn[0] + vn[1] * vn[1] + vn[2] * vn[2]);
  const float mu_cm = fpi::to_float(uniform_distribution(-1., 1., seed));
  const float iv = 1.0f / vel;
  float ucm[3] = {vn[0] * iv, vn[1] * iv, vn[2] * iv};
  rotate_angle_f(ucm[0], ucm[1], ucm[2], mu_cm, seed);
#pragma unroll
  for (int k = 0; k < 3; ++k) vn[k] = vel * ucm[k] + vcm[k];
  const float E2 = vn[0] * vn[0] + vn[1] * vn[1] + vn[2] * vn[2];
  E = fpi::to_double(E2);
  const float iv2 = 1.0f / sqrtf(E2);
  double ud[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) ud[k] = fpi::to_double(vn[k] * iv2);
  const double eps = (ud[0] * ud[0] + ud[1] * ud[1] + ud[2] * ud[2]) - 1.0;
  const double f = 1.0 + eps * (-0.5 + 0.375 * eps);
#pragma unroll
  for (int k = 0; k < 3; ++k) u[k] = ud[k] * f;
}

// src/physics.cpp:754-818 elastic scattering with free-gas target (FP64
// tables: the reference's expressions; FP32 tables: elastic_scatter_f).
__device__ void elastic_scatter(int nuc, double& E, double* u, unsigned long long& seed)
{
  if (dm.xs_fp32) {
    elastic_scatter_f(nuc, E, u, seed);
    return;
  }
  double vel = sqrt(E);
  double awr = dm.awr[nuc];
  double kT = dm.kT[nuc];
  double vn[3] = {vel * u[0], vel * u[1], vel * u[2]};
  double vt[3] = {0.0, 0.0, 0.0};
  if (!(fpi::le(400.0 * kT, E) && fpi::lt(1.0, awr))) sample_cxs_target_velocity(awr, E, u, kT, seed, vt);
  double vcm[3];
  for (int k = 0; k < 3; ++k) vcm[k] = (vn[k] + awr * vt[k]) / (awr + 1.0);
  for (int k = 0; k < 3; ++k) vn[k] = vn[k] - vcm[k];
  vel = sqrt(vn[0] * vn[0] + vn[1] * vn[1] + vn[2] * vn[2]);
  double mu_cm = uniform_distribution(-1., 1., seed);
  double ucm[3];
  ucm[0] = vn[0] / vel;
  ucm[1] = vn[1] / vel;
  ucm[2] = vn[2] / vel;
  rotate_angle(ucm[0], ucm[1], ucm[2], mu_cm, seed);
  for (int k = 0; k < 3; ++k) vn[k] = vel * ucm[k];
  for (int k = 0; k < 3; ++k) vn[k] = vn[k] + vcm[k];
  E = vn[0] * vn[0] + vn[1] * vn[1] + vn[2] * vn[2];
  vel = sqrt(E);
  u[0] = vn[0] / vel;
  u[1] = vn[1] / vel;
  u[2] = vn[2] / vel;
}

// src/physics.cpp:1043-1115 sample_fission_neutron for a prompt-only MT 18
// (no delayed neutrons: the delayed test draws one number and never
// passes) with isotropic emission and a Maxwell or Watt spectrum with
// restriction energy (src/distribution_energy.cpp:282-360); energies at or
// above the data's maximum are resampled.  Then src/physics.cpp:170-285
// create_fission_sites: nu_t = wgt / keff x nu_fission / total of the
// sampled nuclide, each site appended to the generation's fission bank with
// the parent's source index and progeny number (the bank is put in (parent,
// progeny) order after the generation).  A full bank sets an error flag and
// banks no more sites of this particle.
__device__ void create_fission_sites(long long s, int nuc, double wgt, double E_in, const double* u_in,
  double m_nf, double m_tot, unsigned long long& seed)
{
  const double weight = 1.0;
  const double nu_t = wgt / dm.keff * weight * m_nf / m_tot;
  int nu = static_cast<int>(nu_t);
  if (fpi::le(prn(seed), nu_t - fpi::to_double(nu))) ++nu;
  if (nu == 0) return;
  const DFission& F = dm.fis[nuc];
  const double nu_tot = F.nu1 * E_in + F.nu0;  // Horner over (nu0, nu1); the first step 0 E + nu1 is exact
  const double beta = 0.0 / nu_tot;
  for (int k = 0; k < nu; ++k) {
    if (prn(seed) < beta) break;  // never: no delayed neutron data
    double mu = 0.0, E_out = 0.0;
    for (int n_sample = 0; n_sample < 10000; ++n_sample) {
      mu = uniform_distribution(-1., 1., seed);
      for (int tries = 0; tries < 1000000; ++tries) {
        E_out = F.spectrum == 1 ? maxwell_spectrum(F.p0, seed) : watt_spectrum(F.p0, F.p1, seed);
        if (fpi::le(E_out, E_in - F.u)) break;
      }
      if (fpi::lt(E_out, dm.e_max_neutron)) break;
    }
    double uo[3] = {u_in[0], u_in[1], u_in[2]};
    rotate_angle(uo[0], uo[1], uo[2], mu, seed);
    const unsigned long long idx = atomicAdd(&dq.cnt->n_fission, 1ull);
    if (idx >= static_cast<unsigned long long>(dq.fbank_cap)) {
      atomicExch(&dq.cnt->fbank_full, 1);
      return;
    }
    DFissionSite& site = dq.fbank[idx];
    site.r[0] = db.rx[s];
    site.r[1] = db.ry[s];
    site.r[2] = db.rz[s];
    site.u[0] = uo[0];
    site.u[1] = uo[1];
    site.u[2] = uo[2];
    site.E = E_out;
    site.time = dm.track_time ? db.time[s] : 0.0;
    site.parent = db.id[s];
    site.progeny = db.n_progeny[s]++;
  }
}

// src/particle.cpp:331-415 + src/physics.cpp:43-168, 494-518, 638-752
__device__ int ev_collision(long long s, EvStats& st)
{
  st.coll += 1;
  // fields read and written one by one where they are used: loading the
  // slot's whole records up front and storing them back at the end measured
  // 50 % slower for this kernel (170 against 113 ms per 10^7-history batch)
  double E = db.E[s];
  double wgt = db.wgt[s];
  const double E_in = E, wgt_in = wgt;
  unsigned long long seed = db.seed[s];
  int mat = db.material[s];
  double mt = db.macro_t[s];
  // collision estimate of k-effective (src/particle.cpp:333-337)
  if (dm.eigen) db.k_col[s] += wgt * db.macro_nf[s] / mt;
  // sample_nuclide: CDF over atom_density * micro total in material order
  double cutoff = prn(seed) * mt;
  int a = 0, b = 0;
  if (mat >= 0 && mat < dm.n_mat) {
    a = s_tabs.mat_off[mat];
    b = s_tabs.mat_off[mat + 1];
  }
  int i_log = log_union_index(E);
  int chosen = -1;
  double m_tot = 0, m_abs = 0;
  // the sampled nuclide's fission and nu-fission (eigenvalue runs; FP32
  // tables carry nu-fission only, whose sign is the fission cross section's)
  double m_fis = 0, m_nf = 0;
  const bool eig = dm.eigen != 0;
  if (!dm.xs_fp32) {
    double prob = 0.0;
    for (int k = a; k < b; ++k) {
      int nuc = s_tabs.mat_nuc[k];
      st.coll_nuc += 1;
      Micro m = micro_xs64(nuc, i_log, E, eig);
      prob += s_tabs.mat_dens[k] * m.total;
      if (fpi::le(cutoff, prob)) {
        chosen = nuc;
        m_tot = m.total;
        m_abs = m.absorption;
        m_fis = m.fission;
        m_nf = m.nu_fission;
        break;
      }
    }
  } else {
    float prob = 0.0f;
    for (int k = a; k < b; ++k) {
      int nuc = s_tabs.mat_nuc[k];
      st.coll_nuc += 1;
      float t, ab, f32, nf = 0.0f;
      int ig;
      micro_xs32(nuc, i_log, E, t, ab, ig, f32, eig ? &nf : nullptr);
      prob += s_tabs.mat_dens32[k] * t;
      if (fpi::le(cutoff, fpi::to_double(prob))) {
        chosen = nuc;
        m_tot = fpi::to_double(t);
        m_abs = fpi::to_double(ab);
        m_nf = fpi::to_double(nf);
        m_fis = m_nf;
        break;
      }
    }
  }
  double u[3] = {db.ux[s], db.uy[s], db.uz[s]};
  if (chosen < 0) {
    set_error(ERR_NO_NUCLIDE);
    wgt = 0.0;
  } else {
    // fission sites (src/physics.cpp:107-127; sample_fission returns the only
    // fission reaction without a random number)
    if (eig && fpi::pos(m_fis)) create_fission_sites(s, chosen, wgt, E, u, m_nf, m_tot, seed);
    // absorption (analog) src/physics.cpp:638-672, with the absorption
    // estimate of k-effective
    if (fpi::pos(m_abs)) {
      if (fpi::lt(prn(seed) * m_tot, m_abs)) {
        if (eig) db.k_abs[s] += wgt * m_nf / m_abs;
        wgt = 0.0;
      }
    }
    if (!fpi::zero(wgt)) {
      // scatter src/physics.cpp:674-752: the reaction cutoff is drawn; the
      // nuclides of this path have elastic scattering as their only
      // scattering reaction, so the elastic branch is taken
      double c2 = prn(seed) * (m_tot - m_abs);
      (void)c2;
      elastic_scatter(chosen, E, u, seed);
      if (dm.ww_on) {
        double r[3] = {db.rx[s], db.ry[s], db.rz[s]};
        apply_weight_windows(s, wgt, seed, r, u, E, SURFACE_NONE);
      }
      if (fpi::lt(E, dm.energy_cutoff)) wgt = 0.0;
    }
  }
  if (dm.n_tally_collision > 0 && chosen >= 0) {
    const long long cap = db.cap;
    LevelCells lc;
    lc.n = db.n_coord[s];
#pragma unroll
    for (int l = 0; l < MAXL; ++l) lc.c[l] = l < lc.n ? db.cell[l * cap + s] : C_NONE;
    const double r[3] = {db.rx[s], db.ry[s], db.rz[s]};
    score_collision(r, E_in, wgt_in, mt, db.macro_a[s], lc, mat);
  }
  db.E[s] = E;
  db.wgt[s] = wgt;
  db.seed[s] = seed;
  set_direction(s, u[0], u[1], u[2]);
  db.surface[s] = SURFACE_NONE;
  db.material_last[s] = C_NONE;
  db.n_collision[s] += 1;
  long long pid;
  if (traced_slot(s, pid)) {
    TraceRec* rec = trace_slot(pid);
    if (rec) {
      rec->kind = 2;
      rec->surface_or_nuclide = chosen;
      rec->wgt = wgt;
    }
    dq.trace_n[pid - dq.trace_first] += 1;
  }
  return revive_or_free(s, wgt) ? NEXT_XS : NEXT_DEAD;
}

__device__ __forceinline__ void flush_stats(const EvStats& st, int set)
{
  unsigned long long* c = dq.cnt->stat[set];
  warp_count(c + 0, st.xs_ev);
  warp_count(c + 1, st.calc);
  warp_count(c + 2, st.nuc);
  warp_count(c + 3, st.seg);
  warp_count(c + 4, st.coll_nuc);
  warp_count(c + 5, st.surf);
  warp_count(c + 6, st.coll);
}

// ----------------------------------------------------------- queue kernels
// Minimum resident blocks per SM for the event kernels (register budget
// 65536 / (256 x minB) per thread).
#ifndef OMC_MINB_ADV
#define OMC_MINB_ADV 2
#endif
#ifndef OMC_MINB_SURF
#define OMC_MINB_SURF 2
#endif
#ifndef OMC_ADV_BLOCKS_PER_SM
#define OMC_ADV_BLOCKS_PER_SM 32
#endif
#ifndef OMC_MINB_COLL
#define OMC_MINB_COLL 2
#endif
// All kernels of an iteration leave at once while the loop is in its tail
// phase (dq.cnt->tail), where k_tail runs the remaining histories instead.

__global__ void __launch_bounds__(256) k_xs()
{
  if (dq.cnt->tail) return;  // the same for every thread of the grid
  tables_enter();
  const int n = dq.cnt->n_q;
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
    int i = base + threadIdx.x;
    EvStats st {};
    if (i < n) ev_xs(dq.q_in[i], st);
    flush_stats(st, 0);
  }
}

// with_xs: the cross-section event runs in the same thread right before the
// advance (every calculate_xs event is followed by an advance event,
// src/event.cpp:95-98), sparing one pass over the queue and the macroscopic
// XS round trip through HBM.  with_surf: a particle that reaches a boundary
// crosses it in the same thread (the surface event always follows such an
// advance, src/event.cpp:119-124); its latency-bound lookups then overlap
// the FP64 work of the other warps instead of running as a separate pass.
// Per-history results do not depend on either fusion.
// defer: track-length tallies are scored afterwards by k_score_tracks from
// the track records this kernel writes (the scoring code, the largest user
// of registers in this kernel, then stays out of it).
template<bool with_xs, bool with_surf, bool defer, bool may_time = true>
__global__ void __launch_bounds__(256, OMC_MINB_ADV) k_advance()
{
  if (dq.cnt->tail) return;
  tables_enter();
  const int n = dq.cnt->n_q;
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
    int i = base + threadIdx.x;
    bool valid = i < n;
    long long s = valid ? dq.q_in[i] : 0;
    EvStats st {};
    BankHot h {};
    if (valid) h = db.hot[s];
    if (with_xs && valid) ev_xs(s, st, &h);
    int nx = valid ? ev_advance<with_surf, defer, may_time>(s, st, i, &h) : NEXT_DEAD;
    if (!with_surf) warp_append(dq.q_surf, &dq.cnt->n_surf, static_cast<int>(s), nx == NEXT_SURF);
    warp_append(dq.q_coll, &dq.cnt->n_coll, static_cast<int>(s), nx == NEXT_COLL);
    append_next(static_cast<int>(s), nx == NEXT_XS);
    flush_stats(st, 0);
  }
}

// Track-length tallies of this iteration's advance events
// (src/tallies/tally_scoring.cpp:2416-2541, the same score_tracklength as the
// inline path) from the records k_advance wrote at each event's queue
// position.  The end point is recomputed with the advance's own expression
// r0 + d u, so the mesh walk sees the same points; only the order of the
// FP64 atomic additions differs, which atomics leave open anyway.
__global__ void __launch_bounds__(256) k_score_tracks()
{
  if (dq.cnt->tail) return;
  const DTracks& T = dq.trk;
  const int n = dq.cnt->n_q;
  const int stride = gridDim.x * blockDim.x;
  const bool recip = dm.xs_fp32 != 0;
  for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const int i = base + threadIdx.x;
    EvStats st {};
    const double w = i < n ? T.w[i] : 0.0;
    if (!fpi::zero(w)) {
      const double d = T.d[i];
      const double r0[3] = {T.r0x[i], T.r0y[i], T.r0z[i]};
      const double u[3] = {T.ux[i], T.uy[i], T.uz[i]};
      double inv_u[3] = {0.0, 0.0, 0.0};
      if (recip) {
        inv_u[0] = T.iux[i];
        inv_u[1] = T.iuy[i];
        inv_u[2] = T.iuz[i];
      }
      // the end point for the FP64 walk (the FP32 one walks from the distance)
      double r1[3] = {0.0, 0.0, 0.0};
      if (!recip) {
        r1[0] = r0[0] + d * u[0];
        r1[1] = r0[1] + d * u[1];
        r1[2] = r0[2] + d * u[2];
      }
      LevelCells lc;
      lc.n = 0;
#pragma unroll
      for (int l = 0; l < MAXL; ++l) {
        lc.c[l] = dm.trk_cells ? T.cell[l * db.cap + i] : C_NONE;
        if (lc.c[l] != C_NONE) lc.n = l + 1;
      }
      const double mt = dm.trk_xs ? T.mt[i] : 0.0;
      const double ma = dm.trk_xs ? T.ma[i] : 0.0;
      const int mat = dm.trk_mat ? T.mat[i] : C_NONE;
      st.seg += score_tracklength(r0, r1, u, T.E[i], w, d, mt, ma, lc, mat, recip ? inv_u : nullptr);
    }
    flush_stats(st, 0);
  }
}

__global__ void __launch_bounds__(256, OMC_MINB_SURF) k_surface()
{
  if (dq.cnt->tail) return;
  tables_enter();
  const int n = dq.cnt->n_surf;
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
    int i = base + threadIdx.x;
    bool valid = i < n;
    long long s = valid ? dq.q_surf[i] : 0;
    EvStats st {};
    int nx = valid ? ev_surface(s, st) : NEXT_DEAD;
    append_next(static_cast<int>(s), nx == NEXT_XS);
    flush_stats(st, 0);
  }
}

__global__ void __launch_bounds__(256, OMC_MINB_COLL) k_collision()
{
  if (dq.cnt->tail) return;
  tables_enter();
  const int n = dq.cnt->n_coll;
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
    int i = base + threadIdx.x;
    bool valid = i < n;
    long long s = valid ? dq.q_coll[i] : 0;
    EvStats st {};
    int nx = valid ? ev_collision(s, st) : NEXT_DEAD;
    append_next(static_cast<int>(s), nx == NEXT_XS);
    flush_stats(st, 0);
  }
}

// Tail phase: once every source particle of the batch has started and few
// histories remain, each thread carries one history through up to
// max_events events (src/simulation.cpp:804-821, history-based loop) instead
// of paying one kernel launch per event.  Histories that reach the limit go
// back to the queue.  The per-history physics is the same event functions.
__global__ void __launch_bounds__(128, 2) k_tail(int max_events)
{
  if (!dq.cnt->tail) return;
  tables_enter();
  const int n = dq.cnt->n_q;
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
    int i = base + threadIdx.x;
    bool valid = i < n;
    long long s = valid ? dq.q_in[i] : 0;
    EvStats st {};
    int nx = valid ? NEXT_XS : NEXT_DEAD;
    for (int e = 0; e < max_events && nx == NEXT_XS; ++e) {
      BankHot h = db.hot[s];
      ev_xs(s, st, &h);
      nx = ev_advance<true>(s, st, 0, &h);
      if (nx == NEXT_COLL) nx = ev_collision(s, st);
    }
    __syncwarp();
    append_next(static_cast<int>(s), nx == NEXT_XS);
    flush_stats(st, 1);
    warp_count(&dq.cnt->n_events, st.xs_ev);
  }
}

// Free slots take waiting split particles first (split-to-slots mode), then
// new source particles.
// History-based loop (src/simulation.cpp:804-831, the reference's default
// when settings.event_based is false): each thread owns one slot and
// carries a history from birth through every banked secondary to its end
// with the same event functions, then claims the next source index.
__global__ void __launch_bounds__(128, 2) k_history()
{
  tables_enter();
  const long long s = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  EvStats st {};
  if (s < db.cap) {
    for (;;) {
      const long long idx = static_cast<long long>(
        atomicAdd(reinterpret_cast<unsigned long long*>(&dq.cnt->next_source), 1ull));
      if (idx > dm.n_particles || dq.cnt->error != 0) break;
      initialize_history(s, idx);
      int nx = NEXT_XS;
      // every particle dies within max_events events (revive_or_free)
      for (long long e = 0; nx == NEXT_XS && e < (1LL << 40); ++e) {
        BankHot h = db.hot[s];
        ev_xs(s, st, &h);
        nx = ev_advance<true>(s, st, 0, &h);
        if (nx == NEXT_COLL) nx = ev_collision(s, st);
      }
    }
  }
  __syncwarp();
  flush_stats(st, 1);
  warp_count(&dq.cnt->n_events, st.xs_ev);
}

__global__ void k_refill_plan()
{
  DCounters* c = dq.cnt;
  int ks = 0;
  c->refill_split_base = c->split_head;
  if (dq.split && c->split_tail > c->split_head && c->error == 0) {
    const unsigned long long avail = c->split_tail - c->split_head;
    ks = avail < static_cast<unsigned long long>(c->n_free) ? static_cast<int>(avail) : c->n_free;
    c->split_head += static_cast<unsigned long long>(ks);
  }
  c->refill_split = ks;
  long long remaining = dm.n_particles - c->next_source + 1;
  if (remaining < 0) remaining = 0;
  long long room = c->n_free - ks;
  long long k = room < remaining ? room : remaining;
  c->refill_k = ks + static_cast<int>(k);
  c->refill_free_base = c->n_free - c->refill_k;
  c->refill_src = c->next_source;
  c->n_free -= c->refill_k;
  c->next_source += k;
  c->n_refill += static_cast<unsigned long long>(k);
  c->n_surf = 0;
  c->n_coll = 0;
}

__global__ void __launch_bounds__(256) k_refill()
{
  tables_enter();
  const int k = dq.cnt->refill_k;
  const int fb = dq.cnt->refill_free_base;
  const long long src = dq.cnt->refill_src;
  const int ks = dq.cnt->refill_split;
  const unsigned long long sb = dq.cnt->refill_split_base;
  const unsigned long long scap = static_cast<unsigned long long>(dq.cnt->split_cap);
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < k; base += stride) {
    int j = base + threadIdx.x;
    bool valid = j < k;
    int s = valid ? dq.free_list[fb + j] : 0;
    if (valid) {
      if (j < ks) start_split_site(s, dq.split[(sb + j) % scap]);
      else initialize_history(s, src + (j - ks));
    }
    append_next(s, valid);
  }
}

// Counting sort of the next cross-section queue by (material, energy octave,
// and the half of the octave when the keys fit the histogram):
// each block histograms a contiguous chunk in shared memory, one global
// atomic per (block, key) reserves its output range, and the block scatters
// its chunk into that range.
__device__ __forceinline__ int sort_key(int s)
{
  int mat = db.material[s] + 1;
  long long bits = __double_as_longlong(db.E[s]);
  int ex = static_cast<int>((bits >> 52) & 0x7ff) - 1023 + 32;
  ex = ex < 0 ? 0 : (ex > 63 ? 63 : ex);
  // sub-octave: the leading mantissa bits (the energy's position within its
  // octave) when the key count allows
  const int sb = dq.sort_sub_bits;
  const int sub = static_cast<int>((bits >> (52 - sb)) & ((1LL << sb) - 1));
  return (((mat * 64 + ex) << sb) | sub);
}

constexpr int SORT_MAX_KEYS = 2048;

__global__ void __launch_bounds__(512) k_sort_hist()
{
  __shared__ int h[SORT_MAX_KEYS];
  const int nk = dq.sort_keys;
  const int n = dq.cnt->n_next;
  const int chunk = (n + gridDim.x - 1) / gridDim.x;
  const int lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
  for (int k = threadIdx.x; k < nk; k += blockDim.x) h[k] = 0;
  __syncthreads();
  for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) atomicAdd(&h[dq.key_tmp[i]], 1);
  __syncthreads();
  for (int k = threadIdx.x; k < nk; k += blockDim.x)
    if (h[k]) atomicAdd(&dq.hist[k], h[k]);
}

__global__ void k_sort_scan()
{
  // single block: exclusive scan of hist into cursor, hist cleared
  __shared__ int carry;
  __shared__ int wsum[32];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int nk = dq.sort_keys;
  for (int base = 0; base < nk; base += blockDim.x) {
    int i = base + threadIdx.x;
    int v = i < nk ? dq.hist[i] : 0;
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
      int t = lane < (blockDim.x >> 5) ? wsum[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      wsum[lane] = t;
    }
    __syncthreads();
    int incl = x + (w > 0 ? wsum[w - 1] : 0) + carry;
    if (i < nk) {
      dq.cursor[i] = incl - v;
      dq.hist[i] = 0;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = incl;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(512) k_sort_scatter()
{
  __shared__ int h[SORT_MAX_KEYS];
  const int nk = dq.sort_keys;
  const int n = dq.cnt->n_next;
  const int chunk = (n + gridDim.x - 1) / gridDim.x;
  const int lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
  for (int k = threadIdx.x; k < nk; k += blockDim.x) h[k] = 0;
  __syncthreads();
  for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) atomicAdd(&h[dq.key_tmp[i]], 1);
  __syncthreads();
  for (int k = threadIdx.x; k < nk; k += blockDim.x)
    if (h[k]) h[k] = atomicAdd(&dq.cursor[k], h[k]);
  __syncthreads();
  for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
    int s = dq.q_tmp[i];
    int pos = atomicAdd(&h[dq.key_tmp[i]], 1);
    dq.q_in[pos] = s;
  }
}

__global__ void k_copy_queue()
{
  const int n = dq.cnt->n_next;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    dq.q_in[i] = dq.q_tmp[i];
}

__device__ bool finish_iter_common()
{
  DCounters* c = dq.cnt;
  if (!c->tail) c->n_events += static_cast<unsigned long long>(c->n_q);
  c->n_q = c->n_next;
  c->n_next = 0;
  c->iter += 1;
  const bool split_waiting = c->split_tail > c->split_head;
  bool more = c->n_q > 0 || c->next_source <= dm.n_particles || split_waiting;
  // enter the tail phase once every source particle (and split particle)
  // has started and the queue is short enough that per-event launches would
  // dominate
  c->tail = (c->next_source > dm.n_particles && !split_waiting && c->n_q > 0 &&
             c->n_q <= c->tail_threshold) ? 1 : 0;
  if (c->error != 0) more = false;
  if (c->iter >= c->max_iter) {
    if (more) c->error |= ERR_ITERATIONS;
    more = false;
  }
  c->more = more ? 1 : 0;
  return more;
}

__global__ void k_finish_iter(cudaGraphConditionalHandle handle)
{
  bool more = finish_iter_common();
  cudaGraphSetConditional(handle, more ? 1u : 0u);
}

// same epilogue for the profiled (graph-free) batch loop
__global__ void k_finish_iter_host() { finish_iter_common(); }

// Macroscopic cross sections at (material index, E) pairs through the same
// lookup the event kernels run (Material::calculate_neutron_xs,
// src/material.cpp:829-901), for checking the tables against the oracle.
__global__ void __launch_bounds__(256) k_material_xs(long long n, const int* mat, const double* E, double* tot,
  double* abs_, unsigned* hash)
{
  tables_enter();
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int m = mat[i];
    double t = 0.0, a = 0.0;
    uint32_t h = 0xffffffffu;
    if (m >= 0 && m < dm.n_mat) h = material_xs(m, E[i], t, a);
    tot[i] = t;
    abs_[i] = a;
    hash[i] = h;
  }
}

// Tally::accumulate (src/tallies/tally.cpp:821-880)
__global__ void k_accumulate(double* value, double* sum, double* sum_sq, long long n, double norm)
{
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    double val = value[i] * norm;
    value[i] = 0.0;
    sum[i] += val;
    sum_sq[i] += val * val;
  }
}

// ======================================================= host-side driver
#define CK(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) {                                                              \
      throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e_) +      \
                               " at " + __FILE__ + ":" + std::to_string(__LINE__));       \
    }                                                                                     \
  } while (0)

template<class T>
T* dev_upload(const std::vector<T>& v, std::vector<void*>& owned)
{
  if (v.empty()) return nullptr;
  T* p = nullptr;
  CK(cudaMalloc(&p, v.size() * sizeof(T)));
  CK(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  owned.push_back(p);
  return p;
}

template<class T>
T* dev_alloc(size_t n, std::vector<void*>& owned)
{
  if (n == 0) n = 1;
  T* p = nullptr;
  CK(cudaMalloc(&p, n * sizeof(T)));
  CK(cudaMemset(p, 0, n * sizeof(T)));
  owned.push_back(p);
  return p;
}

struct GpuSim {
  std::vector<void*> owned;
  DModel model {};
  DBank bank {};
  DQueues queues {};
  DCounters* cnt = nullptr;
  double *d_value = nullptr, *d_sum = nullptr, *d_sumsq = nullptr;
  long long n_values = 0;
  std::vector<long long> tally_off;
  cudaStream_t stream = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
  int blocks = 1216;
  int blocks_coll = 1216;  // grid of the collision kernel
  int blocks_adv = 4864;   // grid of the advance kernel
  int blocks_trk = 304;    // grid of the track-length scoring kernel
  int sort = 1;
  int fuse = 3;  // bit 0: cross-section event, bit 1: surface crossing, inside the advance kernel
  int split_slots = 0;  // split particles start in free slots with their own seeds
  int history = 0;      // history-based loop (settings.event_based false)
  int defer = 0;        // track-length tallies scored by k_score_tracks from track records
  long long tail_threshold = 1 << 15;  // measured best on the 17x17 lattice (2^17: +1 %, 2^19: +10 %)
  int tail_max_events = 1 << 16;
  // dynamic shared memory of the event kernels: the staged tables (option
  // stage_tables), or 0.  Off by default: the tables are a few KB and stay
  // in L1, and the per-block copy cost 1.4 % of the lattice batch.
  unsigned smem = 0;
  bool tallies_dirty = true;
  float last_batch_ms = 0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // weight windows on device (one set)
  double *d_ww_lower = nullptr, *d_ww_upper = nullptr, *d_ww_e = nullptr;
  long long ww_size = 0;
  unsigned long long* d_group_max = nullptr;  // MAGIC update: per-group maxima
  int n_group_max = 0;
  // eigenvalue run: fission-bank permutation (sorted position -> append
  // position), per-history offsets, comb indices
  int *d_perm = nullptr, *d_offset = nullptr, *d_comb = nullptr;

  ~GpuSim()
  {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
    for (void* p : owned) cudaFree(p);
  }
};

static void build_model(GpuSim& G, const HModel& m, const GpuOptions& opt)
{
  auto& own = G.owned;
  DModel& d = G.model;
  // geometry
  std::vector<DSurface> surf(m.surfaces.size());
  for (size_t k = 0; k < surf.size(); ++k) {
    for (int j = 0; j < 4; ++j) surf[k].c[j] = m.surfaces[k].c[j];
    surf[k].type = m.surfaces[k].type;
    surf[k].bc = m.surfaces[k].bc;
    // squared radius, rounded once as the device expressions would round it
    const double r = surf[k].type >= 3 && surf[k].type <= 5 ? surf[k].c[2] : surf[k].c[3];
    surf[k].rr = surf[k].type >= 3 ? r * r : 0.0;
  }
  std::vector<DCell> cells(m.cells.size());
  std::vector<int> tok;
  for (size_t k = 0; k < cells.size(); ++k) {
    const HCell& c = m.cells[k];
    for (int j = 0; j < 3; ++j) cells[k].tr[j] = c.tr[j];
    cells[k].universe = c.universe;
    cells[k].fill_type = c.fill_type;
    cells[k].fill = c.fill;
    cells[k].tok_off = static_cast<int>(tok.size());
    cells[k].tok_len = static_cast<int>(c.expr.size());
    cells[k].simple = c.simple ? 1 : 0;
    tok.insert(tok.end(), c.expr.begin(), c.expr.end());
  }
  std::vector<int> univ_off {0}, univ_cells;
  for (const auto& u : m.universes) {
    univ_cells.insert(univ_cells.end(), u.begin(), u.end());
    univ_off.push_back(static_cast<int>(univ_cells.size()));
  }
  std::vector<DLattice> lats(m.lattices.size());
  std::vector<int> lat_univ;
  for (size_t k = 0; k < lats.size(); ++k) {
    const HLattice& l = m.lattices[k];
    for (int j = 0; j < 3; ++j) {
      lats[k].ll[j] = l.ll[j];
      lats[k].pitch[j] = l.pitch[j];
      lats[k].half[j] = 0.5 * l.pitch[j];
      lats[k].n[j] = l.n[j];
    }
    lats[k].is3d = l.is3d;
    lats[k].outer = l.outer;
    lats[k].univ_off = static_cast<int>(lat_univ.size());
    lat_univ.insert(lat_univ.end(), l.univ.begin(), l.univ.end());
  }
  d.surf = dev_upload(surf, own);
  d.cell = dev_upload(cells, own);
  d.tok = dev_upload(tok, own);
  d.univ_off = dev_upload(univ_off, own);
  d.univ_cells = dev_upload(univ_cells, own);
  d.lat = dev_upload(lats, own);
  d.lat_univ = dev_upload(lat_univ, own);
  d.n_surf = static_cast<int>(surf.size());
  d.n_cell = static_cast<int>(cells.size());
  d.n_univ = static_cast<int>(m.universes.size());
  d.n_lat = static_cast<int>(lats.size());
  d.root_univ = m.root_universe;
  d.n_coord_levels = m.n_coord_levels;
  if (m.n_coord_levels > MAXL) throw std::runtime_error("geometry nests deeper than the supported coordinate levels");

  // nuclear data: energies FP64, rows (total, absorption, elastic, 0); the
  // FP32 rows carry 1 / (e[k+1] - e[k]) in their last slot (0 at the last
  // point and at duplicate points, whose interval is never interpolated)
  std::vector<long long> nuc_off {0};
  std::vector<double> energy, awr, kT;
  std::vector<XsRow64> xs64;
  std::vector<float4> xs32;
  std::vector<int> grid_index;
  std::vector<DFission> fis;
  for (const auto& n : m.nuclides) {
    energy.insert(energy.end(), n.energy.begin(), n.energy.end());
    for (size_t k = 0; k < n.energy.size(); ++k) {
      xs64.push_back(XsRow64 {n.total[k], n.absorption[k], n.fission[k], n.nu_fission[k]});
      const double de = k + 1 < n.energy.size() ? n.energy[k + 1] - n.energy[k] : 0.0;
      xs32.push_back(make_float4(static_cast<float>(n.total[k]), static_cast<float>(n.absorption[k]),
        static_cast<float>(n.nu_fission[k]), de > 0.0 ? static_cast<float>(1.0 / de) : 0.0f));
    }
    fis.push_back(DFission {n.nu_c[0], n.nu_c[1], n.sp[0], n.sp[1], n.u, n.spectrum, 0});
    nuc_off.push_back(static_cast<long long>(energy.size()));
    grid_index.insert(grid_index.end(), n.grid_index.begin(), n.grid_index.end());
    awr.push_back(n.awr);
    kT.push_back(n.kT);
  }
  d.xs_fp32 = opt.xs_fp32 ? 1 : 0;
  d.nuc_off = dev_upload(nuc_off, own);
  d.energy = dev_upload(energy, own);
  d.xs64 = d.xs_fp32 ? nullptr : dev_upload(xs64, own);
  d.xs32 = d.xs_fp32 ? dev_upload(xs32, own) : nullptr;
  d.grid_index = dev_upload(grid_index, own);
  d.awr = dev_upload(awr, own);
  d.kT = dev_upload(kT, own);
  d.fis = dev_upload(fis, own);
  d.eigen = m.eigenvalue ? 1 : 0;
  d.keff = 1.0;  // simulation::keff before the first generation
  d.e_max_neutron = m.energy_max;
  std::vector<int> mat_off {0}, mat_nuc, mat_id;
  std::vector<double> mat_dens;
  std::vector<float> mat_dens32;
  for (const auto& mt : m.materials) {
    mat_nuc.insert(mat_nuc.end(), mt.nuclide.begin(), mt.nuclide.end());
    mat_dens.insert(mat_dens.end(), mt.atom_density.begin(), mt.atom_density.end());
    for (double v : mt.atom_density) mat_dens32.push_back(static_cast<float>(v));
    mat_off.push_back(static_cast<int>(mat_nuc.size()));
    mat_id.push_back(mt.id);
  }
  d.mat_off = dev_upload(mat_off, own);
  d.mat_nuc = dev_upload(mat_nuc, own);
  d.mat_dens = dev_upload(mat_dens, own);
  d.mat_dens32 = dev_upload(mat_dens32, own);
  d.mat_id = dev_upload(mat_id, own);
  // shared-memory layout of the per-event tables (tables_enter): each table
  // starts on a 16-byte boundary; staged only when all of them fit
  {
    const size_t bytes[STG_N] = {surf.size() * sizeof(DSurface), cells.size() * sizeof(DCell),
                                 tok.size() * sizeof(int), univ_off.size() * sizeof(int),
                                 univ_cells.size() * sizeof(int), mat_off.size() * sizeof(int),
                                 mat_nuc.size() * sizeof(int), mat_dens.size() * sizeof(double),
                                 mat_dens32.size() * sizeof(float)};
    size_t off = 0;
    for (int k = 0; k < STG_N; ++k) {
      d.stage_off[k] = static_cast<int>(off);
      d.stage_words[k] = static_cast<int>(bytes[k] / 4);
      off += (bytes[k] + 15) / 16 * 16;
    }
    d.stage_bytes = (opt.stage_tables && off <= OMC_STAGE_MAX_BYTES) ? static_cast<int>(off) : 0;
    G.smem = static_cast<unsigned>(d.stage_bytes);
  }
  std::vector<int> cell_id;
  for (const auto& c : m.cells) cell_id.push_back(c.id);
  d.cell_id = dev_upload(cell_id, own);
  d.n_nuc = static_cast<int>(m.nuclides.size());
  d.n_mat = static_cast<int>(m.materials.size());
  d.M = m.n_log_bins;
  d.e_min = m.energy_min;
  d.e_max = m.energy_max;
  d.log_spacing = m.log_spacing;
  d.log_emin32 = static_cast<float>(std::log(m.energy_min));
  d.inv_spacing32 = static_cast<float>(1.0 / m.log_spacing);

  // source
  const HSource& src = m.source;
  d.sp_type = src.sp_type;
  d.an_type = src.an_type;
  d.en_type = src.en_type;
  d.dom_type = src.dom_type;
  for (size_t k = 0; k < src.sp.size() && k < 6; ++k) d.sp[k] = src.sp[k];
  for (int k = 0; k < 3; ++k) d.uref[k] = src.uref[k];
  if (src.en_type == 1) {
    d.en_x[0] = src.en[0];
    d.n_en = 1;
  } else {
    size_t n = src.en.size() / 2;
    if (n < 1 || n > 8) throw std::runtime_error("discrete source energies: 1 to 8 values are supported");
    d.n_en = static_cast<int>(n);
    // alias table, src/distribution.cpp:23-80 (Vose)
    std::vector<double> prob(src.en.begin() + n, src.en.end());
    double integral = 0.0;
    for (double p : prob) integral += p;
    for (double& p : prob) p /= integral;
    std::vector<size_t> large, small;
    std::vector<int> alias(n, 0);
    for (size_t i = 0; i < n; i++) {
      prob[i] *= n;
      if (prob[i] > 1.0) large.push_back(i);
      else small.push_back(i);
    }
    while (!large.empty() && !small.empty()) {
      int j = static_cast<int>(small.back());
      int k = static_cast<int>(large.back());
      small.pop_back();
      prob[k] += prob[j] - 1.0;
      alias[j] = k;
      if (prob[k] < 1.0) {
        small.push_back(k);
        large.pop_back();
      }
    }
    for (size_t i = 0; i < n; ++i) {
      d.en_x[i] = src.en[i];
      d.en_prob[i] = prob[i];
      d.en_alias[i] = alias[i];
    }
  }
  d.n_dom = static_cast<int>(src.dom_ids.size());
  d.dom_ids = dev_upload(src.dom_ids, own);

  // meshes, filters, tallies
  std::vector<DMesh> meshes(m.meshes.size());
  for (size_t k = 0; k < meshes.size(); ++k) {
    for (int j = 0; j < 3; ++j) {
      meshes[k].ll[j] = m.meshes[k].ll[j];
      meshes[k].width[j] = m.meshes[k].width[j];
      meshes[k].inv_width32[j] = m.meshes[k].width[j] > 0.0 ? static_cast<float>(1.0 / m.meshes[k].width[j]) : 0.0f;
      meshes[k].width32[j] = static_cast<float>(m.meshes[k].width[j]);
      meshes[k].shape[j] = m.meshes[k].shape[j];
    }
    meshes[k].ndim = m.meshes[k].ndim;
  }
  std::vector<DFilter> filts(m.filters.size());
  std::vector<double> ebins;
  std::vector<int> fids;
  for (size_t k = 0; k < filts.size(); ++k) {
    filts[k].type = m.filters[k].type;
    filts[k].mesh = m.filters[k].mesh;
    filts[k].nbins = m.filters[k].nbins;
    filts[k].e_off = static_cast<int>(ebins.size());
    ebins.insert(ebins.end(), m.filters[k].bins.begin(), m.filters[k].bins.end());
    filts[k].i_off = static_cast<int>(fids.size());
    fids.insert(fids.end(), m.filters[k].ids.begin(), m.filters[k].ids.end());
  }
  std::vector<DTally> tallies(m.tallies.size());
  long long off = 0;
  G.tally_off.clear();
  for (size_t k = 0; k < tallies.size(); ++k) {
    const HTally& t = m.tallies[k];
    tallies[k].value_off = off;
    tallies[k].estimator = t.estimator;
    tallies[k].nfilt = static_cast<int>(t.filters.size());
    tallies[k].nscore = static_cast<int>(t.scores.size());
    if (tallies[k].nscore > 4) throw std::runtime_error("at most four scores per tally are supported");
    for (int j = 0; j < tallies[k].nfilt; ++j) {
      tallies[k].filt[j] = t.filters[j];
      tallies[k].stride[j] = t.strides[j];
    }
    for (int j = 0; j < tallies[k].nscore; ++j) tallies[k].score[j] = t.scores[j];
    G.tally_off.push_back(off);
    off += t.n_filter_bins * static_cast<long long>(t.scores.size());
  }
  G.tally_off.push_back(off);
  G.n_values = off;
  d.mesh = dev_upload(meshes, own);
  d.filt = dev_upload(filts, own);
  d.ebins = dev_upload(ebins, own);
  d.fids = dev_upload(fids, own);
  d.tally = dev_upload(tallies, own);
  d.n_tally = static_cast<int>(tallies.size());
  d.n_tally_tracklength = d.n_tally_collision = 0;
  for (const auto& t : tallies) (t.estimator == 1 ? d.n_tally_collision : d.n_tally_tracklength) += 1;
  d.trk_xs = d.trk_cells = d.trk_mat = 0;
  for (const auto& t : tallies) {
    if (t.estimator != 0) continue;
    for (int j = 0; j < t.nscore; ++j)
      if (t.score[j] != 0) d.trk_xs = 1;
    for (int j = 0; j < t.nfilt; ++j) {
      if (filts[t.filt[j]].type == 3) d.trk_cells = 1;
      if (filts[t.filt[j]].type == 4) d.trk_mat = 1;
    }
  }
  G.d_value = dev_alloc<double>(off, own);
  G.d_sum = dev_alloc<double>(off, own);
  G.d_sumsq = dev_alloc<double>(off, own);
  d.value = G.d_value;

  // weight windows (first set)
  d.ww_on = 0;
  if (!m.weight_windows.empty()) {
    const HWeightWindows& w = m.weight_windows[0];
    d.ww_mesh = w.mesh;
    d.ww_ne = static_cast<int>(w.ebounds.size()) - 1;
    G.d_ww_e = dev_upload(w.ebounds, own);
    G.d_ww_lower = dev_upload(w.lower, own);
    G.d_ww_upper = dev_upload(w.upper, own);
    G.ww_size = static_cast<long long>(w.lower.size());
    d.ww_e = G.d_ww_e;
    d.ww_lower = G.d_ww_lower;
    d.ww_upper = G.d_ww_upper;
    d.ww_surv = w.survival_ratio;
    d.ww_mlb = w.max_lb_ratio;
    d.ww_cut = w.weight_cutoff;
    d.ww_max_split = w.max_split;
    d.ww_on = m.ww_on ? 1 : 0;
  }
  d.max_history_splits = m.max_history_splits;
  d.energy_cutoff = m.energy_cutoff;
  d.time_cutoff = m.time_cutoff;
  d.track_time = m.time_cutoff < INFTY ? 1 : 0;
  d.max_events = m.max_particle_events;
  d.n_particles = m.n_particles;
  d.master_seed = m.seed;
  d.stride = m.stride;
}

static void build_bank(GpuSim& G, long long cap, long long sec_cap)
{
  auto& own = G.owned;
  DBank& b = G.bank;
  b.cap = cap;
  BankDir* dir = dev_alloc<BankDir>(cap, own);
  BankHot* hot = dev_alloc<BankHot>(cap, own);
  BankMisc* misc = dev_alloc<BankMisc>(cap, own);
  BankPos* pos = dev_alloc<BankPos>(cap * MAXL, own);
  BankIdx* idx = dev_alloc<BankIdx>(cap * MAXL, own);
  b.pos = pos;
  b.idx = idx;
  b.dir = dir;
  b.hot = hot;
  b.misc = misc;
  b.id = dev_alloc<long long>(cap, own);
  b.n_coord = {&misc->n_coord};
  b.surface = {&misc->surface};
  b.material = {&misc->material};
  b.material_last = {&misc->material_last};
  b.n_event = dev_alloc<int>(cap, own);
  b.n_collision = dev_alloc<int>(cap, own);
  b.seed = {&hot->seed};
  b.wgt = {&hot->wgt};
  b.macro_t = {&hot->macro_t};
  b.macro_a = {&hot->macro_a};
  b.ux = {&dir->ux};
  b.uy = {&dir->uy};
  b.uz = {&dir->uz};
  b.E = {&dir->E};
  b.rx = {&pos->x};
  b.ry = {&pos->y};
  b.rz = {&pos->z};
  b.cell = {&idx->cell};
  b.univ = {&idx->univ};
  b.latt = {&idx->latt};
  b.lix = {&idx->lix};
  b.liy = {&idx->liy};
  b.liz = {&idx->liz};
  b.wgt_born = dev_alloc<double>(cap, own);
  b.wgt_ww_born = dev_alloc<double>(cap, own);
  b.ww_factor = dev_alloc<double>(cap, own);
  b.cell_last0 = dev_alloc<int>(cap, own);
  b.cell_born = dev_alloc<int>(cap, own);
  b.time = G.model.track_time ? dev_alloc<double>(cap, own) : nullptr;
  b.macro_nf = b.k_col = b.k_abs = b.k_tra = nullptr;
  b.n_progeny = nullptr;
  if (G.model.eigen) {
    b.macro_nf = dev_alloc<double>(cap, own);
    b.k_col = dev_alloc<double>(cap, own);
    b.k_abs = dev_alloc<double>(cap, own);
    b.k_tra = dev_alloc<double>(cap, own);
    b.n_progeny = dev_alloc<int>(cap, own);
  }
  b.bsurf = dev_alloc<int>(cap, own);
  b.blevel = dev_alloc<int>(cap, own);
  b.btrans = dev_alloc<int>(cap, own);
  b.n_split = dev_alloc<int>(cap, own);
  b.sec_top = dev_alloc<int>(cap, own);
  b.sec_free = dev_alloc<int>(cap, own);
  b.n_total = dev_alloc<int>(cap, own);
  DQueues& q = G.queues;
  q.q_in = dev_alloc<int>(cap, own);
  q.q_surf = dev_alloc<int>(cap, own);
  q.q_coll = dev_alloc<int>(cap, own);
  q.q_tmp = dev_alloc<int>(cap, own);
  q.key_tmp = nullptr;
  q.free_list = dev_alloc<int>(cap, own);
  // (material, energy octave) keys, with 1 sub-octave bit when they fit
  // the shared-memory histogram
  q.sort_sub_bits = (G.model.n_mat + 1) * 64 * 2 <= SORT_MAX_KEYS ? 1 : 0;
  q.sort_keys = (G.model.n_mat + 1) * 64 << q.sort_sub_bits;
  if (q.sort_keys > SORT_MAX_KEYS) G.sort = 0;
  if (G.sort) q.key_tmp = dev_alloc<int>(cap, own);
  q.hist = dev_alloc<int>(q.sort_keys, own);
  q.cursor = dev_alloc<int>(q.sort_keys, own);
  q.sec = dev_alloc<DSecondary>(G.split_slots ? 1 : sec_cap, own);
  q.split = G.split_slots ? dev_alloc<DSplitSite>(sec_cap, own) : nullptr;
  // batch source bank (64 B per history) up to 2^27 histories per batch;
  // larger batches sample their sites at refill time
  q.src_bank = nullptr;
  q.src_time = nullptr;
  q.src_n = 0;
  if (G.model.n_particles > 0 && G.model.n_particles <= (1LL << 27)) {
    q.src_bank = dev_alloc<SourceSite>(G.model.n_particles, own);
    q.src_n = G.model.n_particles;
    if (G.model.eigen && G.model.track_time) q.src_time = dev_alloc<double>(G.model.n_particles, own);
  }
  q.trk = DTracks {};
  if (G.defer) {
    DTracks& T = q.trk;
    T.r0x = dev_alloc<double>(cap, own);
    T.r0y = dev_alloc<double>(cap, own);
    T.r0z = dev_alloc<double>(cap, own);
    T.ux = dev_alloc<double>(cap, own);
    T.uy = dev_alloc<double>(cap, own);
    T.uz = dev_alloc<double>(cap, own);
    if (G.model.xs_fp32) {
      T.iux = dev_alloc<double>(cap, own);
      T.iuy = dev_alloc<double>(cap, own);
      T.iuz = dev_alloc<double>(cap, own);
    }
    T.d = dev_alloc<double>(cap, own);
    T.w = dev_alloc<double>(cap, own);
    T.E = dev_alloc<double>(cap, own);
    if (G.model.trk_xs) {
      T.mt = dev_alloc<double>(cap, own);
      T.ma = dev_alloc<double>(cap, own);
    }
    if (G.model.trk_mat) T.mat = dev_alloc<int>(cap, own);
    if (G.model.trk_cells) T.cell = dev_alloc<int>(cap * MAXL, own);
  }
  // eigenvalue run: fission bank of 3 sites per history (the reference's
  // fission_bank capacity, src/simulation.cpp:323-330), the per-history
  // progeny counts, and the permutation / comb index arrays of the bank's
  // sort and resampling
  q.fbank = nullptr;
  q.fbank_cap = 0;
  q.progeny = nullptr;
  q.src_from_bank = 0;
  if (G.model.eigen) {
    if (q.src_n != G.model.n_particles) throw std::runtime_error("eigenvalue runs need at most 2^27 particles per batch");
    q.fbank_cap = 3 * G.model.n_particles;
    q.fbank = dev_alloc<DFissionSite>(q.fbank_cap, own);
    q.progeny = dev_alloc<int>(G.model.n_particles, own);
    G.d_perm = dev_alloc<int>(q.fbank_cap, own);
    G.d_offset = dev_alloc<int>(G.model.n_particles, own);
    G.d_comb = dev_alloc<int>(G.model.n_particles, own);
  }
  G.cnt = dev_alloc<DCounters>(1, own);
  q.cnt = G.cnt;
  q.trace = nullptr;
  q.trace_n = nullptr;
  q.trace_hist = 0;
  q.trace_cap = 0;
  q.batch = 1;
  q.history = G.history;
  DCounters c {};
  c.sec_cap = G.split_slots ? 1 : static_cast<int>(sec_cap);
  c.split_cap = G.split_slots ? static_cast<int>(sec_cap) : 0;
  c.max_iter = 1 << 20;
  c.tail_threshold = static_cast<int>(G.tail_threshold);
  CK(cudaMemcpy(G.cnt, &c, sizeof(c), cudaMemcpyHostToDevice));
}

static void upload_constants(GpuSim& G)
{
  CK(cudaMemcpyToSymbol(dm, &G.model, sizeof(DModel)));
  CK(cudaMemcpyToSymbol(db, &G.bank, sizeof(DBank)));
  CK(cudaMemcpyToSymbol(dq, &G.queues, sizeof(DQueues)));
}

// The advance kernel of the fusion and tally options.  Scoring inside the
// advance is built only for the fully fused form (gpu_create checks); the
// deferred forms also serve models without track-length tallies, where no
// record is written.
static void launch_advance(const GpuSim& G, cudaStream_t S)
{
  const int nb = G.blocks_adv, nt = 256;
  if (!G.defer && G.model.n_tally_tracklength > 0) k_advance<true, true, false><<<nb, nt, G.smem, S>>>();
  else if (G.fuse == 3 && !G.model.track_time) k_advance<true, true, true, false><<<nb, nt, G.smem, S>>>();
  else if (G.fuse == 3) k_advance<true, true, true><<<nb, nt, G.smem, S>>>();
  else if (G.fuse == 1) k_advance<true, false, true><<<nb, nt, G.smem, S>>>();
  else k_advance<false, false, true><<<nb, nt, G.smem, S>>>();
}

static void build_graph(GpuSim& G)
{
  if (G.exec) {
    cudaGraphExecDestroy(G.exec);
    G.exec = nullptr;
  }
  if (G.graph) {
    cudaGraphDestroy(G.graph);
    G.graph = nullptr;
  }
  cudaGraph_t graph;
  CK(cudaGraphCreate(&graph, 0));
  cudaGraphConditionalHandle handle;
  CK(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault));
  const int nb = G.blocks, nt = 256;
  // prologue
  CK(cudaStreamBeginCaptureToGraph(G.stream, graph, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  k_batch_init<<<nb, nt, 0, G.stream>>>(0);
  if (G.queues.src_n > 0) k_source_bank<<<nb, nt, G.smem, G.stream>>>();
  CK(cudaStreamEndCapture(G.stream, &graph));
  size_t n_nodes = 0;
  CK(cudaGraphGetNodes(graph, nullptr, &n_nodes));
  std::vector<cudaGraphNode_t> nodes(n_nodes);
  CK(cudaGraphGetNodes(graph, nodes.data(), &n_nodes));
  // conditional while node
  cudaGraphNodeParams cp {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = handle;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t cond;
  CK(cudaGraphAddNode(&cond, graph, nodes.data(), nullptr, n_nodes, &cp));
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  CK(cudaStreamBeginCaptureToGraph(G.stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  if (!(G.fuse & 1)) k_xs<<<nb, nt, G.smem, G.stream>>>();
  launch_advance(G, G.stream);
  if (G.defer) k_score_tracks<<<G.blocks_trk, nt, 0, G.stream>>>();
  if (!(G.fuse & 2)) k_surface<<<nb, nt, G.smem, G.stream>>>();
  k_collision<<<G.blocks_coll, nt, G.smem, G.stream>>>();
  k_tail<<<nb * 2, 128, G.smem, G.stream>>>(G.tail_max_events);
  k_refill_plan<<<1, 1, 0, G.stream>>>();
  k_refill<<<nb, nt, 0, G.stream>>>();
  if (G.sort) {
    k_sort_hist<<<nb, nt, 0, G.stream>>>();
    k_sort_scan<<<1, 1024, 0, G.stream>>>();
    k_sort_scatter<<<nb, nt, 0, G.stream>>>();
  } else {
    k_copy_queue<<<nb, nt, 0, G.stream>>>();
  }
  k_finish_iter<<<1, 1, 0, G.stream>>>(handle);
  CK(cudaStreamEndCapture(G.stream, &body));
  CK(cudaGraphInstantiate(&G.exec, graph, 0));
  G.graph = graph;
}

GpuSim* gpu_create(const HModel& m, const GpuOptions& opt)
{
  auto* G = new GpuSim();
  try {
    CK(cudaSetDevice(0));
    CK(cudaStreamCreateWithFlags(&G->stream, cudaStreamNonBlocking));
    CK(cudaEventCreate(&G->ev0));
    CK(cudaEventCreate(&G->ev1));
    G->sort = opt.sort ? 1 : 0;
    G->fuse = opt.fuse & 3;
    if (G->fuse == 2) G->fuse = 3;  // the surface fusion builds on the cross-section fusion
    if (opt.tail_threshold >= 0) G->tail_threshold = opt.tail_threshold;
    G->history = m.event_based ? 0 : 1;
    G->split_slots = (!G->history && opt.split_slots && (m.ww_on || !m.weight_windows.empty())) ? 1 : 0;
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
    // grids (256 threads, grid-stride loops) measured on the 17x17 lattice
    // at 2^21 slots: the advance kernel 325 ms per batch with 8 blocks per
    // SM, 305 with 16, 298 with 32, 311 with 64 or 128; the scoring kernel
    // 59.5 with 8, 57.3 with 4, 55.8 with 2 (its resident count)
    G->blocks = sms * 8;
    G->blocks_coll = sms * 8;
    G->blocks_adv = sms * OMC_ADV_BLOCKS_PER_SM;
    G->blocks_trk = sms * 2;
    build_model(*G, m, opt);
    G->defer = (!G->history && opt.defer_tally && G->model.n_tally_tracklength > 0) ? 1 : 0;
    if (!G->history && !opt.defer_tally && G->model.n_tally_tracklength > 0 && G->fuse != 3)
      throw std::runtime_error("track-length tallies scored inside the advance need the fused advance (fuse 3)");
    // 3 x 2^20 slots by default: on the 17x17 lattice (10^7 histories per
    // batch) a batch took 521 ms with 2^19 slots, 492 with 2^20, 487 with
    // 2^21 and 483 with 3 x 2^20 (8 blocks per SM for every kernel), and 449
    // with 2^21 against 441 with 3 x 2^20 at the final grids: each
    // iteration's fixed costs are shared by more events, while the FP64
    // pipe, not the bank's DRAM traffic, bounds the advance kernel
    long long cap = opt.in_flight > 0 ? opt.in_flight : 3LL << 20;
    if (cap > m.n_particles) cap = m.n_particles;
    if (cap < 1) cap = 1;
    long long sec_cap = opt.secondary_cap;
    if (sec_cap <= 0) sec_cap = m.ww_on || !m.weight_windows.empty() ? std::max(cap * 64, 1LL << 22) : 1024;
    if (sec_cap > (1LL << 31) - 1) sec_cap = (1LL << 31) - 1;
    build_bank(*G, cap, sec_cap);
    upload_constants(*G);
    build_graph(*G);
    CK(cudaStreamSynchronize(G->stream));
  } catch (...) {
    delete G;
    throw;
  }
  return G;
}

void gpu_destroy(GpuSim* G) { delete G; }

void gpu_set_trace(GpuSim* G, long long n_hist, int cap, int batch, long long first)
{
  if (n_hist <= 0) {
    G->queues.trace = nullptr;
    G->queues.trace_n = nullptr;
    G->queues.trace_hist = 0;
  } else {
    G->queues.trace = dev_alloc<TraceRec>(static_cast<size_t>(n_hist) * cap, G->owned);
    G->queues.trace_n = dev_alloc<int>(n_hist, G->owned);
    G->queues.trace_hist = n_hist;
    G->queues.trace_cap = cap;
    G->queues.trace_batch = batch;
    G->queues.trace_first = first;
  }
  CK(cudaMemcpyToSymbol(dq, &G->queues, sizeof(DQueues)));
}

void gpu_get_trace(GpuSim* G, void* rec, int* counts)
{
  long long n = G->queues.trace_hist;
  if (n <= 0) return;
  CK(cudaMemcpy(rec, G->queues.trace, sizeof(TraceRec) * n * G->queues.trace_cap, cudaMemcpyDeviceToHost));
  CK(cudaMemcpy(counts, G->queues.trace_n, sizeof(int) * n, cudaMemcpyDeviceToHost));
}

static void fill_stats(const DCounters& c, BatchStats& st)
{
  st.error = c.error;
  st.n_lost = c.n_lost;
  st.lost_id = c.lost_id;
  st.n_done = c.n_done;
  st.iterations = c.iter;
  st.total_weight = c.total_weight;
  st.leakage = c.leakage;
  st.n_events = c.n_events;
  st.n_secondaries = c.n_sec;
  st.longest_events = static_cast<long long>(c.longest >> 34);
  st.longest_id = static_cast<long long>(c.longest & ((1ULL << 34) - 1));
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 7; ++b) st.stat[a][b] = c.stat[a][b];
}

static void accumulate_batch(GpuSim* G, HModel& m)
{
  double norm = m.source.strength / (static_cast<double>(m.n_particles) * 1);
  if (G->n_values > 0) {
    k_accumulate<<<G->blocks, 256, 0, G->stream>>>(G->d_value, G->d_sum, G->d_sumsq, G->n_values, norm);
    CK(cudaGetLastError());
  }
  for (auto& t : m.tallies) t.n_realizations += 1;
  G->tallies_dirty = true;
}

// An inactive batch's tally scores are dropped (the reference does not
// score inactive tallies, src/simulation.cpp:387-396).
static void discard_batch(GpuSim* G)
{
  if (G->n_values > 0) CK(cudaMemsetAsync(G->d_value, 0, sizeof(double) * G->n_values, G->stream));
}

static void launch_history_batch(GpuSim* G, int batch)
{
  const int nb = G->blocks, nt = 256;
  k_batch_init<<<nb, nt, 0, G->stream>>>(batch);
  if (G->queues.src_n > 0) k_source_bank<<<nb, nt, G->smem, G->stream>>>();
  const long long threads = G->bank.cap;
  k_history<<<static_cast<unsigned>((threads + 127) / 128), 128, G->smem, G->stream>>>();
  CK(cudaGetLastError());
}

BatchStats gpu_run_batch(GpuSim* G, HModel& m, int batch, bool accumulate)
{
  G->queues.batch = batch;
  CK(cudaMemcpyToSymbolAsync(dq, &G->queues, sizeof(DQueues), 0, cudaMemcpyHostToDevice, G->stream));
  CK(cudaEventRecord(G->ev0, G->stream));
  if (G->queues.history) launch_history_batch(G, batch);
  else CK(cudaGraphLaunch(G->exec, G->stream));
  CK(cudaEventRecord(G->ev1, G->stream));
  BatchStats st {};
  DCounters c {};
  CK(cudaMemcpyAsync(&c, G->cnt, sizeof(c), cudaMemcpyDeviceToHost, G->stream));
  CK(cudaStreamSynchronize(G->stream));
  CK(cudaEventElapsedTime(&st.ms, G->ev0, G->ev1));
  fill_stats(c, st);
  if (accumulate) accumulate_batch(G, m);
  else discard_batch(G);
  CK(cudaStreamSynchronize(G->stream));
  return st;
}

BatchStats gpu_run_batch_profiled(GpuSim* G, HModel& m, int batch, bool accumulate)
{
  if (G->queues.history) {
    BatchStats st = gpu_run_batch(G, m, batch, accumulate);
    st.kernel_ms[4] = st.ms;  // the whole batch is one history-based kernel
    return st;
  }
  G->queues.batch = batch;
  CK(cudaMemcpyToSymbolAsync(dq, &G->queues, sizeof(DQueues), 0, cudaMemcpyHostToDevice, G->stream));
  const int nb = G->blocks, nt = 256;
  const int n_ev = 16;
  cudaEvent_t ev[n_ev];
  for (auto& e : ev) CK(cudaEventCreate(&e));
  BatchStats st {};
  double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  auto span = [&](int a, int b) {
    float ms;
    CK(cudaEventElapsedTime(&ms, ev[a], ev[b]));
    return static_cast<double>(ms);
  };
  cudaStream_t S = G->stream;
  // OPENMC_GB300_LAUNCH_LOG=<file> appends one CSV line per iteration with
  // the events each queue kernel processed and its duration, so that a
  // kernel profiler's n-th advance launch (counted over the process) can be
  // matched with the work it did.
  static long long advance_launches = 0;
  static FILE* launch_log = nullptr;
  static bool launch_log_checked = false;
  if (!launch_log_checked) {
    launch_log_checked = true;
    if (const char* f = std::getenv("OPENMC_GB300_LAUNCH_LOG")) {
      launch_log = std::fopen(f, "a");
      if (launch_log)
        std::fprintf(launch_log,
          "advance_launch,batch,iteration,xs_events,xs_calc,xs_nuclide_lookups,mesh_segments,"
          "collision_nuclide_lookups,surface,collision,advance_ms,surface_ms,collision_ms,tally_ms\n");
    }
  }
  CK(cudaEventRecord(ev[0], S));
  k_batch_init<<<nb, nt, 0, S>>>(batch);
  if (G->queues.src_n > 0) k_source_bank<<<nb, nt, G->smem, S>>>();
  CK(cudaEventRecord(ev[1], S));
  CK(cudaStreamSynchronize(S));
  acc[7] += span(0, 1);
  DCounters c {};
  unsigned long long prev[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int it = 0; it < (1 << 20); ++it) {
    CK(cudaEventRecord(ev[2], S));
    if (!(G->fuse & 1)) k_xs<<<nb, nt, G->smem, S>>>();
    CK(cudaEventRecord(ev[3], S));
    launch_advance(*G, S);
    CK(cudaEventRecord(ev[12], S));
    if (G->defer) k_score_tracks<<<G->blocks_trk, nt, 0, S>>>();
    CK(cudaEventRecord(ev[4], S));
    if (!(G->fuse & 2)) k_surface<<<nb, nt, G->smem, S>>>();
    CK(cudaEventRecord(ev[5], S));
    k_collision<<<G->blocks_coll, nt, G->smem, S>>>();
    CK(cudaEventRecord(ev[6], S));
    k_tail<<<nb * 2, 128, G->smem, S>>>(G->tail_max_events);
    CK(cudaEventRecord(ev[11], S));
    k_refill_plan<<<1, 1, 0, S>>>();
    CK(cudaEventRecord(ev[7], S));
    k_refill<<<nb, nt, 0, S>>>();
    CK(cudaEventRecord(ev[8], S));
    if (G->sort) {
      k_sort_hist<<<nb, nt, 0, S>>>();
      k_sort_scan<<<1, 1024, 0, S>>>();
      k_sort_scatter<<<nb, nt, 0, S>>>();
    } else {
      k_copy_queue<<<nb, nt, 0, S>>>();
    }
    CK(cudaEventRecord(ev[9], S));
    k_finish_iter_host<<<1, 1, 0, S>>>();
    CK(cudaEventRecord(ev[10], S));
    CK(cudaMemcpyAsync(&c, G->cnt, sizeof(c), cudaMemcpyDeviceToHost, S));
    CK(cudaStreamSynchronize(S));
    acc[0] += span(2, 3);
    acc[1] += span(3, 12);
    acc[8] += span(12, 4);
    acc[2] += span(4, 5);
    acc[3] += span(5, 6);
    acc[4] += span(6, 11);
    acc[7] += span(11, 7);
    acc[5] += span(7, 8);
    acc[6] += span(8, 9);
    acc[7] += span(9, 10);
    if (launch_log) {
      std::fprintf(launch_log, "%lld,%d,%d", advance_launches, batch, it);
      for (int b = 0; b < 7; ++b) {
        std::fprintf(launch_log, ",%llu", c.stat[0][b] - prev[b]);
        prev[b] = c.stat[0][b];
      }
      std::fprintf(launch_log, ",%.6f,%.6f,%.6f,%.6f\n", span(3, 12), span(4, 5), span(5, 6), span(12, 4));
    }
    ++advance_launches;
    if (!c.more) break;
  }
  if (launch_log) std::fflush(launch_log);
  double total = 0;
  for (int k = 0; k < 9; ++k) {
    st.kernel_ms[k] = static_cast<float>(acc[k]);
    total += acc[k];
  }
  st.ms = static_cast<float>(total);
  fill_stats(c, st);
  for (auto& e : ev) cudaEventDestroy(e);
  if (accumulate) accumulate_batch(G, m);
  else discard_batch(G);
  CK(cudaStreamSynchronize(S));
  return st;
}

void gpu_fetch_tallies(GpuSim* G, HModel& m)
{
  if (!G->tallies_dirty) return;
  std::vector<double> sum(G->n_values), sq(G->n_values), val(G->n_values);
  if (G->n_values > 0) {
    CK(cudaMemcpy(sum.data(), G->d_sum, sizeof(double) * G->n_values, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(sq.data(), G->d_sumsq, sizeof(double) * G->n_values, cudaMemcpyDeviceToHost));
    CK(cudaMemcpy(val.data(), G->d_value, sizeof(double) * G->n_values, cudaMemcpyDeviceToHost));
  }
  for (size_t t = 0; t < m.tallies.size(); ++t) {
    long long o = G->tally_off[t];
    long long n = G->tally_off[t + 1] - o;
    auto& r = m.tallies[t].results;
    for (long long k = 0; k < n; ++k) {
      r[3 * k] = val[o + k];
      r[3 * k + 1] = sum[o + k];
      r[3 * k + 2] = sq[o + k];
    }
  }
  G->tallies_dirty = false;
}

void gpu_reset_tallies(GpuSim* G, HModel& m)
{
  if (G->n_values > 0) {
    CK(cudaMemset(G->d_value, 0, sizeof(double) * G->n_values));
    CK(cudaMemset(G->d_sum, 0, sizeof(double) * G->n_values));
    CK(cudaMemset(G->d_sumsq, 0, sizeof(double) * G->n_values));
  }
  for (auto& t : m.tallies) {
    t.n_realizations = 0;
    std::fill(t.results.begin(), t.results.end(), 0.0);
  }
  G->tallies_dirty = false;
}

void gpu_set_ww_bounds(GpuSim* G, const double* lower, const double* upper, long long n)
{
  if (n != G->ww_size) throw std::runtime_error("weight-window bounds have the wrong size");
  CK(cudaMemcpy(G->d_ww_lower, lower, sizeof(double) * n, cudaMemcpyHostToDevice));
  CK(cudaMemcpy(G->d_ww_upper, upper, sizeof(double) * n, cudaMemcpyHostToDevice));
}

// src/weight_windows.cpp:640-673: mean (or 1 / relative error) per window
// bin over the element volume, kept in lower; the relative error in upper;
// the positive maximum of each energy group through an integer atomic max
// on the bit pattern (positive doubles order like their bits).
__global__ void k_magic_values(MagicArgs a, const double* sum, const double* sum_sq, double* lower, double* upper,
                               unsigned long long* group_max)
{
  const long long n_bins = a.e_bins * a.mesh_bins;
  for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < n_bins;
       k += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int e = static_cast<int>(k / a.mesh_bins);
    const long long mb = k - e * a.mesh_bins;
    long long fb = mb * a.stride_mesh;
    if (a.stride_energy >= 0) fb += e * a.stride_energy;
    const long long i = fb * a.n_scores + a.score;
    const double s = sum[i];
    double nb = s / a.n;
    double rel;
    if (s > 0.0) {
      const double mean_val = nb;
      const double variance = (sum_sq[i] / a.n - mean_val * mean_val) / (a.n - 1);
      rel = sqrt(variance) / mean_val;
    } else {
      rel = 1.7976931348623157e308;
    }
    if (a.rel_err) nb = 1.0 / rel;
    nb /= a.volume;
    lower[k] = nb;
    upper[k] = rel;
    if (nb > 0.0) atomicMax(group_max + e, static_cast<unsigned long long>(__double_as_longlong(nb)));
  }
}

// src/weight_windows.cpp:675-700, 734-753: per-group normalisation by
// 1 / (2 max), -1 where the bin is unscored or noisier than the threshold,
// upper = ratio x lower.
__global__ void k_magic_finish(MagicArgs a, const double* sum, double* lower, double* upper,
                               const unsigned long long* group_max)
{
  const long long n_bins = a.e_bins * a.mesh_bins;
  for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < n_bins;
       k += static_cast<long long>(gridDim.x) * blockDim.x) {
    const int e = static_cast<int>(k / a.mesh_bins);
    const long long mb = k - e * a.mesh_bins;
    long long fb = mb * a.stride_mesh;
    if (a.stride_energy >= 0) fb += e * a.stride_energy;
    const double s = sum[fb * a.n_scores + a.score];
    double nb = lower[k];
    const double rel = upper[k];
    const double gm = __longlong_as_double(static_cast<long long>(group_max[e]));
    if (gm > 0.0) nb *= 1.0 / (2.0 * gm);
    if (s <= 0.0) nb = -1.0;
    else if (rel > a.threshold) nb = -1.0;
    lower[k] = nb;
    upper[k] = a.ratio * nb;
  }
}

void gpu_update_magic(GpuSim* G, const MagicArgs& a, double* lower, double* upper)
{
  const long long n = a.e_bins * a.mesh_bins;
  if (n != G->ww_size || !G->d_ww_lower) throw std::runtime_error("weight-window bounds have the wrong size");
  if (a.tally < 0 || a.tally + 1 >= static_cast<int>(G->tally_off.size()))
    throw std::runtime_error("tally index out of range");
  if (G->n_group_max < a.e_bins) {
    G->d_group_max = dev_alloc<unsigned long long>(a.e_bins, G->owned);
    G->n_group_max = a.e_bins;
  }
  const long long off = G->tally_off[a.tally];
  CK(cudaMemsetAsync(G->d_group_max, 0, sizeof(unsigned long long) * a.e_bins, G->stream));
  const int nb = G->blocks, nt = 256;
  k_magic_values<<<nb, nt, 0, G->stream>>>(a, G->d_sum + off, G->d_sumsq + off, G->d_ww_lower, G->d_ww_upper,
                                           G->d_group_max);
  k_magic_finish<<<nb, nt, 0, G->stream>>>(a, G->d_sum + off, G->d_ww_lower, G->d_ww_upper, G->d_group_max);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(lower, G->d_ww_lower, sizeof(double) * n, cudaMemcpyDeviceToHost, G->stream));
  CK(cudaMemcpyAsync(upper, G->d_ww_upper, sizeof(double) * n, cudaMemcpyDeviceToHost, G->stream));
  CK(cudaStreamSynchronize(G->stream));
}

// ------------------------------------------------ eigenvalue generations
// src/bank.cpp:83-88: exclusive scan of the per-history progeny counts (one
// block; n is at most 2^27)
__global__ void __launch_bounds__(1024) k_eig_scan(const int* progeny, int* offset, long long n)
{
  __shared__ int wsum[32];
  __shared__ long long carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (long long base = 0; base < n; base += blockDim.x) {
    const long long i = base + threadIdx.x;
    const int v = i < n ? progeny[i] : 0;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
      int t = lane < static_cast<int>(blockDim.x >> 5) ? wsum[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      wsum[lane] = t;
    }
    __syncthreads();
    const long long incl = x + (w > 0 ? wsum[w - 1] : 0) + carry;
    if (i < n) offset[i] = static_cast<int>(incl - v);
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = incl;
    __syncthreads();
  }
}

// src/bank.cpp:111-125: the sorted position of each appended site is its
// parent's offset plus its progeny number; perm maps sorted -> appended
__global__ void k_eig_place(const DFissionSite* bank, long long n_sites, const int* offset, int* perm)
{
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n_sites;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const DFissionSite& site = bank[i];
    const long long pos = static_cast<long long>(offset[site.parent - 1]) + site.progeny;
    if (pos < 0 || pos >= n_sites) {
      set_error(ERR_BANK);  // progeny counts and bank disagree
      continue;
    }
    perm[pos] = static_cast<int>(i);
  }
}

// The combed sites (sorted positions comb[k]) become the source sites of
// generation `batch` (src/eigenvalue.cpp:351-356 copy into the source
// bank), each with the tracking seed of its history id (initialize_history,
// src/simulation.cpp:613-616)
__global__ void k_eig_gather(const DFissionSite* bank, const int* perm, const int* comb, long long n, int batch,
                             SourceSite* src)
{
  for (long long k = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; k < n;
       k += static_cast<long long>(gridDim.x) * blockDim.x) {
    const DFissionSite& site = bank[perm[comb[k]]];
    SourceSite out;
    for (int j = 0; j < 3; ++j) {
      out.r[j] = site.r[j];
      out.u[j] = site.u[j];
    }
    out.E = site.E;
    if (dq.src_time) dq.src_time[k] = site.time;
    const long long id = static_cast<long long>(batch - 1) * n + k + 1;
    out.tseed = future_seed(static_cast<unsigned long long>(id) * dm.stride,
                            static_cast<unsigned long long>(dm.master_seed + 0));
    src[k] = out;
  }
}

GenerationStats gpu_finish_generation(GpuSim* G, int batch)
{
  GenerationStats out;
  if (!G->model.eigen) return out;
  DCounters c {};
  CK(cudaMemcpyAsync(&c, G->cnt, sizeof(c), cudaMemcpyDeviceToHost, G->stream));
  CK(cudaStreamSynchronize(G->stream));
  if (c.fbank_full) throw std::runtime_error("The shared fission bank is full.");
  out.fission_sites = static_cast<long long>(c.n_fission);
  out.k_col = c.k_col;
  out.k_abs = c.k_abs;
  out.k_tra = c.k_tra;
  out.total_weight = c.total_weight;
  if (out.fission_sites == 0) throw std::runtime_error("No fission sites banked on MPI rank 0");
  const long long n = G->model.n_particles;
  k_eig_scan<<<1, 1024, 0, G->stream>>>(G->queues.progeny, G->d_offset, n);
  k_eig_place<<<G->blocks, 256, 0, G->stream>>>(G->queues.fbank, out.fission_sites, G->d_offset, G->d_perm);
  // src/eigenvalue.cpp:135-174 uniform combing on one rank, the teeth
  // positions accumulated in the reference's order
  unsigned long long seed = future_seed(static_cast<unsigned long long>(batch) * G->model.stride,
                                        static_cast<unsigned long long>(G->model.master_seed + 0));
  const long long total = out.fission_sites;
  const double teeth_distance = static_cast<double>(total) / n;
  const double teeth_offset = std::ldexp(static_cast<double>(prn_word(seed)), -64) * teeth_distance;
  const long long tooth_start = static_cast<long long>(std::ceil((0 - teeth_offset) / teeth_distance));
  const long long tooth_end = static_cast<long long>(std::floor((total - teeth_offset) / teeth_distance)) + 1;
  std::vector<int> comb;
  comb.reserve(n);
  double tooth = tooth_start * teeth_distance + teeth_offset;
  for (long long i = tooth_start; i < tooth_end && static_cast<long long>(comb.size()) < n; i++) {
    const long long idx = static_cast<long long>(std::floor(tooth));
    if (idx < 0 || idx >= total) throw std::runtime_error("comb tooth outside the fission bank");
    comb.push_back(static_cast<int>(idx));
    tooth += teeth_distance;
  }
  if (static_cast<long long>(comb.size()) < n) throw std::runtime_error("the comb selected fewer sites than particles");
  CK(cudaMemcpyAsync(G->d_comb, comb.data(), sizeof(int) * n, cudaMemcpyHostToDevice, G->stream));
  k_eig_gather<<<G->blocks, 256, 0, G->stream>>>(G->queues.fbank, G->d_perm, G->d_comb, n, batch + 1,
                                                 G->queues.src_bank);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(&c, G->cnt, sizeof(c), cudaMemcpyDeviceToHost, G->stream));
  CK(cudaStreamSynchronize(G->stream));
  if (c.error & ERR_BANK) throw std::runtime_error("Mismatch detected between sum of all particle progeny and shared fission bank size.");
  G->queues.src_from_bank = 1;
  return out;
}

void gpu_set_keff(GpuSim* G, double keff)
{
  G->model.keff = keff;
  CK(cudaMemcpyToSymbol(dm, &G->model, sizeof(DModel)));
}

void gpu_set_ww_on(GpuSim* G, bool on)
{
  if (on && !G->d_ww_lower) throw std::runtime_error("no weight windows are defined");
  G->model.ww_on = on ? 1 : 0;
  CK(cudaMemcpyToSymbol(dm, &G->model, sizeof(DModel)));
}

long long gpu_capacity(GpuSim* G) { return G->bank.cap; }

void gpu_material_xs(GpuSim* G, long long n, const int* mat, const double* E, double* total, double* absorption,
                     unsigned* grid_hash)
{
  if (n <= 0) return;
  struct Scratch {
    int* mat = nullptr;
    double *E = nullptr, *t = nullptr, *a = nullptr;
    unsigned* h = nullptr;
    ~Scratch()
    {
      cudaFree(mat);
      cudaFree(E);
      cudaFree(t);
      cudaFree(a);
      cudaFree(h);
    }
  } d;
  CK(cudaMalloc(&d.mat, n * sizeof(int)));
  CK(cudaMalloc(&d.E, n * sizeof(double)));
  CK(cudaMalloc(&d.t, n * sizeof(double)));
  CK(cudaMalloc(&d.a, n * sizeof(double)));
  CK(cudaMalloc(&d.h, n * sizeof(unsigned)));
  CK(cudaMemcpyAsync(d.mat, mat, n * sizeof(int), cudaMemcpyHostToDevice, G->stream));
  CK(cudaMemcpyAsync(d.E, E, n * sizeof(double), cudaMemcpyHostToDevice, G->stream));
  const long long blocks = std::min<long long>((n + 255) / 256, G->blocks);
  k_material_xs<<<static_cast<unsigned>(blocks), 256, G->smem, G->stream>>>(n, d.mat, d.E, d.t, d.a, d.h);
  CK(cudaGetLastError());
  CK(cudaMemcpyAsync(total, d.t, n * sizeof(double), cudaMemcpyDeviceToHost, G->stream));
  CK(cudaMemcpyAsync(absorption, d.a, n * sizeof(double), cudaMemcpyDeviceToHost, G->stream));
  CK(cudaMemcpyAsync(grid_hash, d.h, n * sizeof(unsigned), cudaMemcpyDeviceToHost, G->stream));
  CK(cudaStreamSynchronize(G->stream));
}

}  // namespace OMC_NS
}  // namespace omc
