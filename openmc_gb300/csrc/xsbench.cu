// Macroscopic cross-section lookup kernel on flat 5-channel tables
// (68 nuclides x 11,303 points x 5 channels, 12 materials; the lookup
// microbenchmark shape).  Each lookup restates Material::calculate_neutron_xs
// (src/material.cpp:829-901) with the per-nuclide hash window, bounded
// binary search, duplicate-point bump and linear interpolation of
// Nuclide::calculate_xs (src/nuclide.cpp:724-775) applied to all 5 row
// columns.
//
// Layout in HBM: energies FP64 [n_nuc][G]; rows [n_nuc][G][5] in FP64 or FP32;
// hash windows int32 [n_nuc][M+1]; material nuclide lists with FP64 (or FP32)
// atom densities.  Lookups are counting-sorted by (material, energy octave)
// so that a warp walks one material's nuclide list in lockstep and its grid
// reads land on neighbouring rows.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_runtime.h>

namespace xsb {

struct Tables {
  int n_nuc, G, M, n_mat, fp32;
  double e_min, e_max, log_spacing;
  float log_emin32, inv_spacing32;
  double* energy;
  double* xs64;
  float* xs32;
  int* grid_index;
  int* mat_off;
  int* mat_nuc;
  double* mat_dens;
  float* mat_dens32;
  // sort scratch (allocated at creation for a maximum lookup count)
  long long max_n;
  int* keys_hist;
  int* keys_cursor;
  int* perm;
  int n_keys;
  cudaStream_t stream;
  cudaEvent_t ev[4];
  float last_ms_sort, last_ms_lookup;
};

__device__ __forceinline__ int lb_index(const double* a, int lo, int hi, double v)
{
  if (a[lo] == v) return 0;
  long long key = __double_as_longlong(v);
  int first = lo, count = hi - lo;
  while (count > 0) {
    int step = count >> 1;
    int it = first + step;
    if (__double_as_longlong(__ldg(a + it)) < key) {
      first = it + 1;
      count -= step + 1;
    } else {
      count = step;
    }
  }
  return first - lo - 1;
}

// Sort key of a lookup: material x 64 + binary exponent of E (clamped to
// 64 octaves).  A material index outside [0, n_mat) gets key 0, so that the
// histogram and cursor arrays (n_mat x 64 entries) are never indexed out of
// range; k_lookup then writes NaN for that lookup.
__device__ __forceinline__ int key_of(int mat, double E, int n_mat)
{
  if (mat < 0 || mat >= n_mat) return 0;
  long long bits = __double_as_longlong(E);
  int ex = static_cast<int>((bits >> 52) & 0x7ff) - 1023 + 32;
  ex = ex < 0 ? 0 : (ex > 63 ? 63 : ex);
  return mat * 64 + ex;
}

__global__ void k_hist(const int* mat, const double* E, long long n, int n_mat, int* hist)
{
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    atomicAdd(&hist[key_of(mat[i], E[i], n_mat)], 1);
}

__global__ void k_scan(int* hist, int* cursor, int nk)
{
  __shared__ int carry;
  __shared__ int wsum[32];
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nk; base += blockDim.x) {
    int i = base + threadIdx.x;
    int v = i < nk ? hist[i] : 0;
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
      cursor[i] = incl - v;
      hist[i] = 0;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = incl;
    __syncthreads();
  }
}

__global__ void k_scatter(const int* mat, const double* E, long long n, int n_mat, int* cursor, int* perm)
{
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    int pos = atomicAdd(&cursor[key_of(mat[i], E[i], n_mat)], 1);
    perm[pos] = static_cast<int>(i);
  }
}

template<bool FP32>
__global__ void __launch_bounds__(256) k_lookup(Tables T, const int* __restrict__ mat, const double* __restrict__ Ein,
  const int* __restrict__ perm, long long n, double* __restrict__ out, int* __restrict__ grid_hash)
{
  for (long long j = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; j < n;
       j += static_cast<long long>(gridDim.x) * blockDim.x) {
    int k = perm ? __ldg(perm + j) : static_cast<int>(j);
    int m = __ldg(mat + k);
    double E = __ldg(Ein + k);
    if (m < 0 || m >= T.n_mat) {
      // material index out of range: no table is read; NaN results and hash 0
      double* o = out + static_cast<long long>(k) * 5;
#pragma unroll
      for (int c = 0; c < 5; ++c) o[c] = __longlong_as_double(0x7ff8000000000000LL);
      if (grid_hash) grid_hash[k] = 0;
      continue;
    }
    // hash bin: FP32 pre-test, FP64 expression within 1/64 bin of a bin
    // edge (the same exact scheme as the transport kernels)
    int i_log;
    {
      const float q = (logf(static_cast<float>(E)) - T.log_emin32) * T.inv_spacing32;
      const float fl = floorf(q), fr = q - fl;
      if (fr > 0.015625f && fr < 0.984375f && fabsf(q) < 1.0e7f) i_log = static_cast<int>(fl);
      else i_log = static_cast<int>(log(E / T.e_min) / T.log_spacing);
    }
    i_log = i_log < 0 ? 0 : (i_log > T.M - 1 ? T.M - 1 : i_log);
    double macro[5] = {0, 0, 0, 0, 0};
    float macro32[5] = {0, 0, 0, 0, 0};
    uint32_t h = 0;
    int a = __ldg(T.mat_off + m), b = __ldg(T.mat_off + m + 1);
    for (int q = a; q < b; ++q) {
      int nuc = __ldg(T.mat_nuc + q);
      const double* e = T.energy + static_cast<long long>(nuc) * T.G;
      int i_grid;
      if (E < __ldg(e)) {
        i_grid = 0;
      } else if (E > __ldg(e + T.G - 1)) {
        i_grid = T.G - 2;
      } else {
        const int* gi = T.grid_index + static_cast<long long>(nuc) * (T.M + 1);
        int i_low = __ldg(gi + i_log);
        int i_high = __ldg(gi + i_log + 1) + 1;
        i_grid = i_low + lb_index(e, i_low, i_high, E);
      }
      double e0 = __ldg(e + i_grid), e1 = __ldg(e + i_grid + 1);
      if (e0 == e1) {
        ++i_grid;
        e0 = e1;
        e1 = __ldg(e + i_grid + 1);
      }
      h = h * 31u + static_cast<uint32_t>(i_grid);
      long long row = (static_cast<long long>(nuc) * T.G + i_grid) * 5;
      if (FP32) {
        const float* x = T.xs32 + row;
        const float f32 = static_cast<float>(E - e0) / static_cast<float>(e1 - e0);
        float d = __ldg(T.mat_dens32 + q);
#pragma unroll
        for (int c = 0; c < 5; ++c) {
          float a = __ldg(x + c), b = __ldg(x + 5 + c);
          macro32[c] += d * (a + f32 * (b - a));
        }
      } else {
        const double f = (E - e0) / (e1 - e0);
        const double* x = T.xs64 + row;
        double d = __ldg(T.mat_dens + q);
#pragma unroll
        for (int c = 0; c < 5; ++c) macro[c] += d * ((1.0 - f) * __ldg(x + c) + f * __ldg(x + 5 + c));
      }
    }
    double* o = out + static_cast<long long>(k) * 5;
#pragma unroll
    for (int c = 0; c < 5; ++c) o[c] = FP32 ? static_cast<double>(macro32[c]) : macro[c];
    if (grid_hash) grid_hash[k] = static_cast<int>(h);
  }
}

#define CK(call)                                                                              \
  do {                                                                                        \
    cudaError_t e_ = (call);                                                                  \
    if (e_ != cudaSuccess)                                                                    \
      throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e_) + " line " + \
                               std::to_string(__LINE__));                                     \
  } while (0)

}  // namespace xsb

// ---------------------------------------------------------------------------
// Scratch for openmc_gb300_xs_lookup_noalloc: a fixed-size array in device
// global memory that the library owns for its whole lifetime (every GPU that
// loads the library holds these ~16 MiB until the process exits).  Layout:
// [NOALLOC_MAX_KEYS histogram | NOALLOC_MAX_KEYS cursors | NOALLOC_MAX_LOOKUPS
// permutation], all int32.
constexpr long long NOALLOC_MAX_LOOKUPS = 1LL << 22;  // 4,194,304 lookups per call
constexpr int NOALLOC_MAX_KEYS = 4096;                // materials x 64 energy octaves
static __device__ __align__(256) int g_noalloc_scratch[2 * NOALLOC_MAX_KEYS + NOALLOC_MAX_LOOKUPS];

__global__ void k_zero_ints(int* p, int n)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) p[i] = 0;
}

extern "C" char openmc_err_msg[256];
extern "C" int OPENMC_E_ALLOCATE;
extern "C" int OPENMC_E_INVALID_ARGUMENT;
extern "C" int OPENMC_E_OUT_OF_BOUNDS;

using namespace xsb;

extern "C" {

// Build device tables.  energy [n_nuc][G], xs [n_nuc][G][5] (host, FP64);
// the hash windows follow Nuclide::init_grid (src/nuclide.cpp:502-533) over
// [max of grid minima, min of grid maxima].  max_lookups sizes the sort
// scratch.  Returns 0 and a handle, or an OPENMC_E_* code.
int openmc_gb300_xs_tables_create(int n_nuc, int G, const double* energy, const double* xs, int n_mat,
  const int32_t* mat_off, const int32_t* mat_nuc, const double* mat_dens, int n_log_bins, int fp32,
  int64_t max_lookups, void** handle)
{
  Tables* T = nullptr;
  try {
    if (n_nuc <= 0 || G < 2 || n_mat <= 0 || n_log_bins < 1)
      throw std::invalid_argument("invalid table dimensions");
    T = new Tables();
    std::memset(T, 0, sizeof(Tables));
    T->n_nuc = n_nuc;
    T->G = G;
    T->M = n_log_bins;
    T->n_mat = n_mat;
    T->fp32 = fp32 ? 1 : 0;
    double emin = 0.0, emax = 1.7976931348623157e308;
    for (int i = 0; i < n_nuc; ++i) {
      emin = std::max(emin, energy[static_cast<size_t>(i) * G]);
      emax = std::min(emax, energy[static_cast<size_t>(i) * G + G - 1]);
    }
    T->e_min = emin;
    T->e_max = emax;
    std::vector<int> gidx(static_cast<size_t>(n_nuc) * (n_log_bins + 1));
    const int M = n_log_bins;
    double spacing = std::log(emax / emin) / M;
    double stop = M * spacing;
    double step = stop / M;
    for (int i = 0; i < n_nuc; ++i) {
      const double* e = energy + static_cast<size_t>(i) * G;
      int j = 0;
      for (int k = 0; k <= M; ++k) {
        double umesh = (k == M) ? stop : 0.0 + step * k;
        while (std::log(e[j + 1] / emin) <= umesh) {
          if (j + 2 == G) break;
          ++j;
        }
        gidx[static_cast<size_t>(i) * (M + 1) + k] = j;
      }
    }
    T->log_spacing = std::log(emax / emin) / M;
    T->log_emin32 = static_cast<float>(std::log(emin));
    T->inv_spacing32 = static_cast<float>(1.0 / T->log_spacing);
    size_t ne = static_cast<size_t>(n_nuc) * G;
    CK(cudaMalloc(&T->energy, ne * 8));
    CK(cudaMemcpy(T->energy, energy, ne * 8, cudaMemcpyHostToDevice));
    if (T->fp32) {
      std::vector<float> x32(ne * 5);
      for (size_t k = 0; k < ne * 5; ++k) x32[k] = static_cast<float>(xs[k]);
      CK(cudaMalloc(&T->xs32, ne * 5 * 4));
      CK(cudaMemcpy(T->xs32, x32.data(), ne * 5 * 4, cudaMemcpyHostToDevice));
    } else {
      CK(cudaMalloc(&T->xs64, ne * 5 * 8));
      CK(cudaMemcpy(T->xs64, xs, ne * 5 * 8, cudaMemcpyHostToDevice));
    }
    CK(cudaMalloc(&T->grid_index, gidx.size() * 4));
    CK(cudaMemcpy(T->grid_index, gidx.data(), gidx.size() * 4, cudaMemcpyHostToDevice));
    int nm = mat_off[n_mat];
    CK(cudaMalloc(&T->mat_off, (n_mat + 1) * 4));
    CK(cudaMemcpy(T->mat_off, mat_off, (n_mat + 1) * 4, cudaMemcpyHostToDevice));
    CK(cudaMalloc(&T->mat_nuc, nm * 4));
    CK(cudaMemcpy(T->mat_nuc, mat_nuc, nm * 4, cudaMemcpyHostToDevice));
    CK(cudaMalloc(&T->mat_dens, nm * 8));
    CK(cudaMemcpy(T->mat_dens, mat_dens, nm * 8, cudaMemcpyHostToDevice));
    std::vector<float> d32(mat_dens, mat_dens + nm);
    CK(cudaMalloc(&T->mat_dens32, nm * 4));
    CK(cudaMemcpy(T->mat_dens32, d32.data(), nm * 4, cudaMemcpyHostToDevice));
    T->n_keys = n_mat * 64;
    T->max_n = max_lookups;
    CK(cudaMalloc(&T->keys_hist, T->n_keys * 4));
    CK(cudaMemset(T->keys_hist, 0, T->n_keys * 4));
    CK(cudaMalloc(&T->keys_cursor, T->n_keys * 4));
    if (max_lookups > 0) CK(cudaMalloc(&T->perm, max_lookups * 4));
    CK(cudaStreamCreateWithFlags(&T->stream, cudaStreamNonBlocking));
    for (auto& e : T->ev) CK(cudaEventCreate(&e));
    *handle = T;
    return 0;
  } catch (const std::exception& e) {
    std::snprintf(openmc_err_msg, sizeof(openmc_err_msg), "%s", e.what());
    delete T;
    return OPENMC_E_ALLOCATE;
  }
}

int openmc_gb300_xs_tables_free(void* handle)
{
  auto* T = static_cast<Tables*>(handle);
  if (!T) return 0;
  cudaFree(T->energy);
  cudaFree(T->xs64);
  cudaFree(T->xs32);
  cudaFree(T->grid_index);
  cudaFree(T->mat_off);
  cudaFree(T->mat_nuc);
  cudaFree(T->mat_dens);
  cudaFree(T->mat_dens32);
  cudaFree(T->keys_hist);
  cudaFree(T->keys_cursor);
  cudaFree(T->perm);
  for (auto& e : T->ev) cudaEventDestroy(e);
  cudaStreamDestroy(T->stream);
  delete T;
  return 0;
}

// Lookups with inputs already in device memory: d_mat[n], d_E[n] -> d_out[n][5]
// (macroscopic total, elastic, absorption, aux1, aux2 for the microbenchmark
// tables) and optional d_grid_hash[n] (h = 31 h + grid index over the
// material's nuclides).  sort != 0 counting-sorts the lookups first.
// Asynchronous on the library's stream; times are kept for the next call of
// openmc_gb300_xs_last_times.
int openmc_gb300_xs_lookup_device(void* handle, int64_t n, const int32_t* d_mat, const double* d_E, double* d_out,
  int32_t* d_grid_hash, int sort)
{
  auto* T = static_cast<Tables*>(handle);
  try {
    if (!T || n < 0) throw std::invalid_argument("invalid lookup arguments");
    if (n == 0) return 0;
    int dev = 0, sms = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int blocks = sms * 8;
    const int* perm = nullptr;
    CK(cudaEventRecord(T->ev[0], T->stream));
    if (sort) {
      if (n > T->max_n) throw std::invalid_argument("more lookups than the sort scratch holds");
      k_hist<<<blocks, 256, 0, T->stream>>>(d_mat, d_E, n, T->n_mat, T->keys_hist);
      k_scan<<<1, 1024, 0, T->stream>>>(T->keys_hist, T->keys_cursor, T->n_keys);
      k_scatter<<<blocks, 256, 0, T->stream>>>(d_mat, d_E, n, T->n_mat, T->keys_cursor, T->perm);
      perm = T->perm;
    }
    CK(cudaEventRecord(T->ev[1], T->stream));
    if (T->fp32) k_lookup<true><<<blocks, 256, 0, T->stream>>>(*T, d_mat, d_E, perm, n, d_out, d_grid_hash);
    else k_lookup<false><<<blocks, 256, 0, T->stream>>>(*T, d_mat, d_E, perm, n, d_out, d_grid_hash);
    CK(cudaEventRecord(T->ev[2], T->stream));
    CK(cudaGetLastError());
    return 0;
  } catch (const std::exception& e) {
    std::snprintf(openmc_err_msg, sizeof(openmc_err_msg), "%s", e.what());
    return OPENMC_E_INVALID_ARGUMENT;
  }
}

// Same lookups from host buffers (copies in, computes, copies out; blocking).
int openmc_gb300_xs_lookup(void* handle, int64_t n, const int32_t* mat, const double* E, double* out,
  int32_t* grid_hash, int sort)
{
  auto* T = static_cast<Tables*>(handle);
  int32_t* dm = nullptr;
  double *dE = nullptr, *dout = nullptr;
  int32_t* dh = nullptr;
  try {
    if (!T || n < 0) throw std::invalid_argument("invalid lookup arguments");
    if (n == 0) return 0;
    for (int64_t i = 0; i < n; ++i)
      if (mat[i] < 0 || mat[i] >= T->n_mat) {
        std::snprintf(openmc_err_msg, sizeof(openmc_err_msg),
                      "lookup %lld: material index %d outside [0, %d)", static_cast<long long>(i), mat[i], T->n_mat);
        return OPENMC_E_OUT_OF_BOUNDS;
      }
    CK(cudaMallocAsync(&dm, n * 4, T->stream));
    CK(cudaMallocAsync(&dE, n * 8, T->stream));
    CK(cudaMallocAsync(&dout, n * 40, T->stream));
    if (grid_hash) CK(cudaMallocAsync(&dh, n * 4, T->stream));
    CK(cudaMemcpyAsync(dm, mat, n * 4, cudaMemcpyHostToDevice, T->stream));
    CK(cudaMemcpyAsync(dE, E, n * 8, cudaMemcpyHostToDevice, T->stream));
    int rc = openmc_gb300_xs_lookup_device(handle, n, dm, dE, dout, dh, sort);
    if (rc) throw std::runtime_error(openmc_err_msg);
    CK(cudaMemcpyAsync(out, dout, n * 40, cudaMemcpyDeviceToHost, T->stream));
    if (grid_hash) CK(cudaMemcpyAsync(grid_hash, dh, n * 4, cudaMemcpyDeviceToHost, T->stream));
    cudaFreeAsync(dm, T->stream);
    cudaFreeAsync(dE, T->stream);
    cudaFreeAsync(dout, T->stream);
    if (dh) cudaFreeAsync(dh, T->stream);
    CK(cudaStreamSynchronize(T->stream));
    return 0;
  } catch (const std::exception& e) {
    std::snprintf(openmc_err_msg, sizeof(openmc_err_msg), "%s", e.what());
    return OPENMC_E_INVALID_ARGUMENT;
  }
}

int openmc_gb300_xs_stream(void* handle, void** stream)
{
  *stream = static_cast<Tables*>(handle)->stream;
  return 0;
}

// milliseconds of the last device lookup call: [sort, lookup]
int openmc_gb300_xs_last_times(void* handle, float* ms)
{
  auto* T = static_cast<Tables*>(handle);
  cudaEventSynchronize(T->ev[2]);
  cudaEventElapsedTime(&ms[0], T->ev[0], T->ev[1]);
  cudaEventElapsedTime(&ms[1], T->ev[1], T->ev[2]);
  return 0;
}

// No counterpart in the reference.  The same sorted macroscopic-XS lookups as
// openmc_gb300_xs_lookup_device, for callers that cannot allocate device
// memory at the time of the call: code running under a memory budget or a
// pool it does not own, or an embedding host whose allocator must not be
// re-entered from a solver callback.  The call allocates nothing: the sort
// scratch is the library's static device array g_noalloc_scratch.
//
// - n must not exceed 4,194,304 lookups and the tables at most 64 materials
//   (4,096 sort keys); larger requests return OPENMC_E_INVALID_ARGUMENT.
// - The first call on a device looks up the array's device address with
//   cudaGetSymbolAddress (with that device current) and caches it; make that
//   first call before any stream capture on the device.
// - All calls share the one array: calls whose work overlaps on the GPU
//   (different streams, or other host threads) race and give wrong results.
//   The histogram part is cleared at the start of every call; the rest is
//   fully rewritten by each call.
// - Inputs and outputs are device pointers; the work is queued on `stream`
//   (a cudaStream_t, null for the legacy default stream) and the call returns
//   without waiting for it.
int openmc_gb300_xs_lookup_noalloc(void* handle, int64_t n, const int32_t* d_mat, const double* d_E, double* d_out,
  int32_t* d_grid_hash, void* stream)
{
  static std::mutex lock;
  static int* scratch_of_device[128] = {nullptr};
  auto* T = static_cast<Tables*>(handle);
  try {
    if (!T || n < 0) throw std::invalid_argument("invalid lookup arguments");
    if (n > NOALLOC_MAX_LOOKUPS)
      throw std::invalid_argument("openmc_gb300_xs_lookup_noalloc: " + std::to_string(n) +
                                  " lookups exceed the static scratch limit of 4194304 per call");
    if (T->n_keys > NOALLOC_MAX_KEYS)
      throw std::invalid_argument("openmc_gb300_xs_lookup_noalloc: tables with more than 64 materials "
                                  "exceed the static sort scratch");
    if (n == 0) return 0;
    int dev = 0;
    CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 128) throw std::invalid_argument("device index out of range");
    int* base;
    {
      std::lock_guard<std::mutex> g(lock);
      if (!scratch_of_device[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
          throw std::runtime_error(std::string("cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
        scratch_of_device[dev] = static_cast<int*>(p);
      }
      base = scratch_of_device[dev];
    }
    int* hist = base;
    int* cursor = base + NOALLOC_MAX_KEYS;
    int* perm = base + 2 * NOALLOC_MAX_KEYS;
    cudaStream_t S = static_cast<cudaStream_t>(stream);
    int sms = 0;
    CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int blocks = sms * 8;
    k_zero_ints<<<(T->n_keys + 255) / 256, 256, 0, S>>>(hist, T->n_keys);
    k_hist<<<blocks, 256, 0, S>>>(d_mat, d_E, n, T->n_mat, hist);
    k_scan<<<1, 1024, 0, S>>>(hist, cursor, T->n_keys);
    k_scatter<<<blocks, 256, 0, S>>>(d_mat, d_E, n, T->n_mat, cursor, perm);
    if (T->fp32) k_lookup<true><<<blocks, 256, 0, S>>>(*T, d_mat, d_E, perm, n, d_out, d_grid_hash);
    else k_lookup<false><<<blocks, 256, 0, S>>>(*T, d_mat, d_E, perm, n, d_out, d_grid_hash);
    CK(cudaGetLastError());
    return 0;
  } catch (const std::exception& e) {
    std::snprintf(openmc_err_msg, sizeof(openmc_err_msg), "%s", e.what());
    return OPENMC_E_INVALID_ARGUMENT;
  }
}

}  // extern "C"
