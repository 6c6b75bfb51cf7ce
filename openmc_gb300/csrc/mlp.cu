// Importance MLP for learned weight windows: (x, y, z, log E) -> log flux,
// 4 -> 128 -> 128 -> 128 -> 1 with SiLU, BF16 weights and activations in the
// matrix products, FP32 accumulation, FP32 master weights and Adam.
// No counterpart in the reference; its output feeds the weight-window bounds
// consumed by apply_weight_windows (src/weight_windows.cpp:56-146).
//
// The three hidden-layer products of every training step -- forward
// (Z = H W^T), input gradient (dH = dZ W) and weight gradient (dW = dZ^T H) --
// run on the 5th-generation tensor cores: one CTA of 128 threads owns a
// 128-row tile of D = A B^T (A: rows x K, B: N x K, both K-major BF16), stages
// 64-wide K chunks of A and B into shared memory in the canonical no-swizzle
// core-matrix layout (8 rows x 16 bytes per core matrix), and one elected
// thread issues tcgen05.mma.cta_group::1.kind::f16 (M = 128, N = 16..128,
// K = 16 per instruction) into an FP32 accumulator in tensor memory.
// tcgen05.commit signals an mbarrier when the products are done; the four
// warps read their 32 accumulator rows back with tcgen05.ld and apply the
// epilogue (bias + SiLU, SiLU derivative, or split-K accumulation).
// Every mbarrier wait is bounded: on timeout the kernel records an error,
// releases its tensor memory and returns.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace mlp {

constexpr int TILE_M = 128;  // rows of D per CTA (tcgen05 M)
constexpr int KC = 64;       // K elements staged per chunk
constexpr int HID = 128;     // hidden width
constexpr int IN_PAD = 16;   // input features padded to one K step

// ------------------------------------------------------------------ PTX
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor (tcgen05): start address >> 4 in bits
// 0-13, leading-dimension byte offset >> 4 in bits 16-29 (distance between
// core matrices along K for K-major operands), stride-dimension byte offset
// >> 4 in bits 32-45 (distance between 8-row groups), the fixed value 0b001
// in bits 46-48, base offset 0, no swizzle (bits 61-63 = 0).
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
  uint64_t d = 0;
  d |= static_cast<uint64_t>((addr >> 4) & 0x3FFF);
  d |= static_cast<uint64_t>((lbo >> 4) & 0x3FFF) << 16;
  d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFF) << 32;
  d |= 1ull << 46;
  return d;
}

// Instruction descriptor for kind::f16: FP32 accumulator (bits 4-5 = 1),
// BF16 A and B (bits 7-9 = 1, 10-12 = 1), both K-major (bits 15, 16 = 0),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N)
{
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
         (static_cast<uint32_t>(M >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t* smem_dst, uint32_t ncols)
{
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(smem_dst)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
  uint32_t accumulate)
{
  asm volatile(
    "{\n\t.reg .pred p;\n\t"
    "setp.ne.b32 p, %4, 0;\n\t"
    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
    "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
    : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* mbar)
{
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                 smem_u32(mbar))
               : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* mbar, uint32_t count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(mbar)), "r"(count) : "memory");
}

// Waits for the mbarrier phase with the given parity; gives up after
// max_tries polls and returns false.
__device__ __forceinline__ bool mbar_wait(uint64_t* mbar, uint32_t parity, uint32_t max_tries)
{
  uint32_t addr = smem_u32(mbar);
  for (uint32_t i = 0; i < max_tries; ++i) {
    uint32_t done;
    asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(addr), "r"(parity)
      : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void fence_async_shared()
{
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

// 32 consecutive FP32 accumulator columns of this thread's row
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v)
{
  uint32_t r[32];
  asm volatile(
    "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
    "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
    "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
      "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
      "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
    : "r"(taddr)
    : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 32; ++k) v[k] = __uint_as_float(r[k]);
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float silu_grad(float z)
{
  float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

enum Epi { EPI_FORWARD = 0, EPI_DINPUT = 1, EPI_DWEIGHT = 2 };

struct GemmArgs {
  const __nv_bfloat16* A;  // rows x K (row stride lda)
  const __nv_bfloat16* B;  // N x K (row stride ldb)
  int lda, ldb;
  int rows;      // valid rows of D (multiple of 128 after padding)
  int N;         // 16 or 128
  int K;         // reduction length handled by each CTA (multiple of 16)
  int k_split;   // EPI_DWEIGHT: K range per CTA; CTA c reduces [c k_split, (c+1) k_split)
  // epilogue operands
  const float* bias;      // EPI_FORWARD: [N]
  float* Z;               // EPI_FORWARD: pre-activation out [rows][N]
  __nv_bfloat16* H;       // EPI_FORWARD: silu(Z) out [rows][N]
  const float* Zprev;     // EPI_DINPUT: pre-activation of the layer below [rows][N]
  __nv_bfloat16* dZprev;  // EPI_DINPUT: dH * silu'(Zprev) out [rows][N]
  __nv_bfloat16* HT;      // EPI_FORWARD / EPI_DINPUT: optional transposed copy [N][ldT]
  int ldT;
  float* dW;              // EPI_DWEIGHT: partial blockIdx.x of [128][N]
  int* error;
};

// Issues asynchronous 16-byte copies (cp.async, zero-filled past k_end) of
// a tile of `nrows` rows x KC elements (row r of the source at
// src + r * ld + k0) into shared memory in core-matrix order
// [row/8][k/8][row%8][k%8]; the caller commits and waits for the group.
__device__ __forceinline__ void stage_tile_async(__nv_bfloat16* dst, const __nv_bfloat16* src, int ld, int nrows,
  int k0, int k_end)
{
  constexpr int groups = KC / 8;  // 8-element (16-byte) groups per row
  for (int idx = threadIdx.x; idx < nrows * groups; idx += blockDim.x) {
    const int r = idx / groups, g = idx % groups;
    const int k = k0 + g * 8;
    const bool in = k + 8 <= k_end;
    const __nv_bfloat16* from = in ? src + static_cast<long long>(r) * ld + k : src;
    __nv_bfloat16* out = dst + ((r / 8) * groups + g) * 64 + (r % 8) * 8;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(out)), "l"(from),
                 "r"(in ? 16 : 0)
                 : "memory");
  }
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// Copies a tile of `nrows` rows x KC elements (row r of the source at
// src + r * ld + k0) into shared memory in core-matrix order
// [row/8][k/8][row%8][k%8]; elements past k_end are zero.
__device__ __forceinline__ void stage_tile(__nv_bfloat16* dst, const __nv_bfloat16* src, int ld, int nrows, int k0,
  int k_end, int kc)
{
  const int groups = kc / 8;  // 8-element (16-byte) groups per row
  for (int idx = threadIdx.x; idx < nrows * groups; idx += blockDim.x) {
    int r = idx / groups, g = idx % groups;
    int k = k0 + g * 8;
    uint4 v = make_uint4(0, 0, 0, 0);
    if (k + 8 <= k_end) v = *reinterpret_cast<const uint4*>(src + static_cast<long long>(r) * ld + k);
    __nv_bfloat16* out = dst + ((r / 8) * groups + g) * 64 + (r % 8) * 8;
    *reinterpret_cast<uint4*>(out) = v;
  }
}

// ------------------------------------------------------------------ GEMM
constexpr int MAX_N = 144;                    // 128 outputs + ones row (bias gradient) + padding
constexpr int A_TILE_BYTES = TILE_M * KC * 2;  // 16 KB
constexpr int B_TILE_BYTES = MAX_N * KC * 2;   // 18 KB
constexpr int GEMM_SMEM = 2 * (A_TILE_BYTES + B_TILE_BYTES) + 1024;
constexpr uint32_t WAIT_TRIES = 1u << 22;
constexpr int ERR_TIMEOUT = 1;

// D = A B^T for one 128-row tile (EPI_FORWARD, EPI_DINPUT: tile blockIdx.x
// of the rows; K = the whole reduction) or for one K range of the weight
// gradient (EPI_DWEIGHT: the 128 output neurons x N inputs, reduced over
// rows [blockIdx.x k_split, ...), written to partial blockIdx.x).
// Two shared-memory stages: the 128 threads stage chunk c while the tensor
// core multiplies chunk c-1; an mbarrier per stage, signalled by
// tcgen05.commit, says when a stage may be overwritten.
template <int EPI>
__global__ void __launch_bounds__(128, 1) k_gemm(GemmArgs g)
{
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __nv_bfloat16* sA[2] = {reinterpret_cast<__nv_bfloat16*>(base),
                          reinterpret_cast<__nv_bfloat16*>(base + A_TILE_BYTES)};
  __nv_bfloat16* sB[2] = {reinterpret_cast<__nv_bfloat16*>(base + 2 * A_TILE_BYTES),
                          reinterpret_cast<__nv_bfloat16*>(base + 2 * A_TILE_BYTES + B_TILE_BYTES)};
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t tmem_s;

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const uint32_t ncols = g.N <= 128 ? 128u : 256u;
  if (warp == 0) tmem_alloc(&tmem_s, ncols);
  if (threadIdx.x == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_s;

  long long row0 = 0;
  int k_begin = 0, k_end = g.K;
  const __nv_bfloat16* A = g.A;
  if (EPI == EPI_DWEIGHT) {
    k_begin = blockIdx.x * g.k_split;
    k_end = min(g.K, k_begin + g.k_split);
  } else {
    row0 = static_cast<long long>(blockIdx.x) * TILE_M;
    A = g.A + row0 * g.lda;
  }
  const int n_chunks = k_end > k_begin ? (k_end - k_begin + KC - 1) / KC : 0;
  const uint32_t idesc = instr_desc(TILE_M, g.N);
  bool ok = true;
  // Two-stage pipeline: the copies of chunk c + 1 are in flight while the
  // tensor core multiplies chunk c; a stage is refilled once the MMAs that
  // read it have committed to its mbarrier.
  if (n_chunks > 0) {
    stage_tile_async(sA[0], A, g.lda, TILE_M, k_begin, k_end);
    stage_tile_async(sB[0], g.B, g.ldb, g.N, k_begin, k_end);
    cp_async_commit();
  }
  for (int c = 0; c < n_chunks && ok; ++c) {
    const int s = c & 1;
    if (c + 1 < n_chunks) {
      const int s1 = (c + 1) & 1;
      // stage s1 was last read by the MMAs of chunk c - 1
      if (c >= 1) ok = mbar_wait(&mbar[s1], ((c - 1) >> 1) & 1, WAIT_TRIES);
      ok = __syncthreads_and(ok);
      if (!ok) break;
      const int k1 = k_begin + (c + 1) * KC;
      stage_tile_async(sA[s1], A, g.lda, TILE_M, k1, k_end);
      stage_tile_async(sB[s1], g.B, g.ldb, g.N, k1, k_end);
      cp_async_commit();
      cp_async_wait<1>();  // this thread's copies of chunk c have landed
    } else {
      cp_async_wait<0>();
    }
    fence_async_shared();
    __syncthreads();
    if (threadIdx.x == 0) {
      tc_fence_after();
      const int k0 = k_begin + c * KC;
      const int nk = min(KC, k_end - k0);
      const uint32_t a0 = smem_u32(sA[s]), b0 = smem_u32(sB[s]);
      for (int j = 0; j * 16 < nk; ++j) {
        // K step j: two core matrices (2 x 128 B) further along K
        uint64_t ad = smem_desc(a0 + j * 256, 128, 1024);
        uint64_t bd = smem_desc(b0 + j * 256, 128, 1024);
        mma_bf16(tmem, ad, bd, idesc, (c > 0 || j > 0) ? 1u : 0u);
      }
      mma_commit(&mbar[s]);
    }
  }
  cp_async_wait<0>();
  if (n_chunks > 0) {
    const int last = n_chunks - 1;
    bool done = mbar_wait(&mbar[last & 1], (last >> 1) & 1, WAIT_TRIES);
    ok = __syncthreads_and(ok && done);
  }
  if (!ok) {
    if (threadIdx.x == 0) atomicOr(g.error, ERR_TIMEOUT);
  } else {
    tc_fence_after();
    // Epilogue.  tcgen05.ld gives each thread one row (32 columns at a
    // time); rows are written through a per-warp 32 x 33 shared-memory
    // transpose so that each global store covers consecutive columns of one
    // row, while the transposed copies (HT) are written from the row layout,
    // where consecutive lanes hold consecutive rows.  The stage buffers are
    // free: every MMA has completed.
    float* st = reinterpret_cast<float*>(base) + warp * (32 * 33);
    const uint32_t t_row = tmem + (static_cast<uint32_t>(32 * warp) << 16);
    const long long r0w = row0 + 32 * warp;  // first row of this warp
    float v[32];
    for (int cb = 0; cb < g.N; cb += 32) {
      if (n_chunks > 0) tmem_ld32(t_row + cb, v);
      else for (int k = 0; k < 32; ++k) v[k] = 0.0f;
      if (EPI == EPI_FORWARD) {
        if (g.HT) {
#pragma unroll
          for (int k = 0; k < 32; ++k)
            g.HT[static_cast<long long>(cb + k) * g.ldT + r0w + lane] =
              __float2bfloat16_rn(silu(v[k] + g.bias[cb + k]));
        }
      }
#pragma unroll
      for (int k = 0; k < 32; ++k) st[lane * 33 + k] = v[k];
      __syncwarp();
      const int col = cb + lane;
      if (EPI == EPI_FORWARD) {
        const float b = g.bias[col];
        for (int rr = 0; rr < 32; ++rr) {
          const long long r = r0w + rr;
          const float z = st[rr * 33 + lane] + b;
          g.Z[r * g.N + col] = z;
          g.H[r * g.N + col] = __float2bfloat16_rn(silu(z));
        }
      } else if (EPI == EPI_DINPUT) {
        // all 32 pre-activations of this column first, so that the loads
        // are in flight together
        float zp[32];
#pragma unroll
        for (int rr = 0; rr < 32; ++rr) zp[rr] = __ldg(g.Zprev + (r0w + rr) * g.N + col);
#pragma unroll
        for (int rr = 0; rr < 32; ++rr) {
          const long long r = r0w + rr;
          const float d = st[rr * 33 + lane] * silu_grad(zp[rr]);
          const __nv_bfloat16 db16 = __float2bfloat16_rn(d);
          g.dZprev[r * g.N + col] = db16;
          st[rr * 33 + lane] = __bfloat162float(db16);
        }
        __syncwarp();
        if (g.HT) {
#pragma unroll
          for (int k = 0; k < 32; ++k)
            g.HT[static_cast<long long>(cb + k) * g.ldT + r0w + lane] = __float2bfloat16_rn(st[lane * 33 + k]);
        }
      } else {
        float* out = g.dW + static_cast<long long>(blockIdx.x) * TILE_M * g.N;
        if (col < g.N)
          for (int rr = 0; rr < 32; ++rr) out[(32 * warp + rr) * static_cast<long long>(g.N) + col] = st[rr * 33 + lane];
      }
      __syncwarp();
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, ncols);
  }
}

// ------------------------------------------------------------------ output layer
// y = H3 . w4 + b4 in FP32 (one thread per row), the weighted squared-error
// loss against the target, and the start of the backward pass:
// dZ3 = (dL/dy) w4 * silu'(Z3).  Per-block partial sums of dL/dw4 (128),
// dL/db4 and the loss go to partial[block][130] in a fixed order.
// Block 0 advances the optimizer step counter.
__global__ void __launch_bounds__(128) k_head(const __nv_bfloat16* __restrict__ H3, const float* __restrict__ Z3,
  const float* __restrict__ w4, const float* __restrict__ b4, const float* __restrict__ target,
  const float* __restrict__ weight, int n_real, int R_pad, float inv_n, __nv_bfloat16* dZ3, __nv_bfloat16* dZ3T,
  float* partial, float* y_out, int* step)
{
  __shared__ float sw[HID], sdy[TILE_M], sl[TILE_M];
  const int t = threadIdx.x;
  const long long row0 = static_cast<long long>(blockIdx.x) * TILE_M;
  const long long r = row0 + t;
  sw[t] = w4[t];
  __syncthreads();
  const __nv_bfloat16* h = H3 + r * HID;
  float y = b4[0];
  for (int k = 0; k < HID; k += 8) {
    uint4 q = *reinterpret_cast<const uint4*>(h + k);
    const __nv_bfloat16* e = reinterpret_cast<const __nv_bfloat16*>(&q);
#pragma unroll
    for (int j = 0; j < 8; ++j) y = fmaf(__bfloat162float(e[j]), sw[k + j], y);
  }
  if (y_out && r < n_real) y_out[r] = y;
  if (!dZ3) return;
  float dy = 0.0f, loss = 0.0f;
  if (r < n_real) {
    const float wt = weight ? weight[r] : 1.0f;
    const float e = y - target[r];
    loss = wt * e * e * inv_n;
    dy = 2.0f * wt * e * inv_n;
  }
  const float* z = Z3 + r * HID;
  for (int k = 0; k < HID; k += 8) {
    __align__(16) __nv_bfloat16 d[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) d[j] = __float2bfloat16_rn(dy * sw[k + j] * silu_grad(z[k + j]));
    *reinterpret_cast<uint4*>(dZ3 + r * HID + k) = *reinterpret_cast<const uint4*>(d);
#pragma unroll
    for (int j = 0; j < 8; ++j) dZ3T[static_cast<long long>(k + j) * R_pad + r] = d[j];
  }
  sdy[t] = dy;
  sl[t] = loss;
  __syncthreads();
  float acc = 0.0f;
  for (int rr = 0; rr < TILE_M; ++rr) acc = fmaf(sdy[rr], __bfloat162float(H3[(row0 + rr) * HID + t]), acc);
  float* out = partial + static_cast<long long>(blockIdx.x) * 130;
  out[t] = acc;
  if (t == 0) {
    float sd = 0.0f, ss = 0.0f;
    for (int rr = 0; rr < TILE_M; ++rr) {
      sd += sdy[rr];
      ss += sl[rr];
    }
    out[128] = sd;
    out[129] = ss;
    if (blockIdx.x == 0) step[0] += 1;
  }
}

// ------------------------------------------------------------------ parameters
// Flat FP32 parameter vector: W1[128][4], b1[128], W2[128][128], b2[128],
// W3[128][128], b3[128], w4[128], b4.
constexpr int P_W1 = 0, P_B1 = 512, P_W2 = 640, P_B2 = P_W2 + 16384, P_W3 = P_B2 + 128, P_B3 = P_W3 + 16384,
              P_W4 = P_B3 + 128, P_B4 = P_W4 + 128, N_PARAMS = P_B4 + 1;
constexpr int G1_N = 16, G_N = 144;  // row widths of the weight-gradient partials

struct AdamArgs {
  float* P;
  float* m;
  float* v;
  const float* G1;  // [splits][128][16]: cols 0-3 dW1, col 4 db1
  const float* G2;  // [splits][128][144]: cols 0-127 dW2, col 128 db2
  const float* G3;
  const float* GH;  // [head_blocks][130]: dw4, db4, loss
  int splits, head_blocks;
  float lr, beta1, beta2, eps;
  const int* step;
  int update;       // 0: gradients only
  float* grad_out;  // optional flat gradient [N_PARAMS]
  float* loss_out;  // optional loss of this step (indexed by step - 1)
  __nv_bfloat16 *W1, *W2, *W2T, *W3, *W3T;  // BF16 operand copies
};

__device__ __forceinline__ float sum_partials(const float* G, int splits, long long stride, long long off)
{
  float s = 0.0f;
  for (int k = 0; k < splits; ++k) s += G[k * stride + off];
  return s;
}

// One thread per parameter: sums the gradient partials in a fixed order,
// applies Adam (bias-corrected first and second moments) and rewrites the
// BF16 operand copies (W and its transpose for the input-gradient product).
__global__ void k_adam(AdamArgs a)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= N_PARAMS) return;
  const long long s1 = 128LL * G1_N, s2 = 128LL * G_N;
  float g;
  if (p < P_B1) g = sum_partials(a.G1, a.splits, s1, (p / 4) * G1_N + p % 4);
  else if (p < P_W2) g = sum_partials(a.G1, a.splits, s1, (p - P_B1) * G1_N + 4);
  else if (p < P_B2) g = sum_partials(a.G2, a.splits, s2, ((p - P_W2) / 128) * G_N + (p - P_W2) % 128);
  else if (p < P_W3) g = sum_partials(a.G2, a.splits, s2, (p - P_B2) * G_N + 128);
  else if (p < P_B3) g = sum_partials(a.G3, a.splits, s2, ((p - P_W3) / 128) * G_N + (p - P_W3) % 128);
  else if (p < P_W4) g = sum_partials(a.G3, a.splits, s2, (p - P_B3) * G_N + 128);
  else if (p < P_B4) g = sum_partials(a.GH, a.head_blocks, 130, p - P_W4);
  else g = sum_partials(a.GH, a.head_blocks, 130, 128);
  if (a.grad_out) a.grad_out[p] = g;
  const int t = a.step[0];
  if (p == 0 && a.loss_out && t > 0) a.loss_out[t - 1] = sum_partials(a.GH, a.head_blocks, 130, 129);
  float w = a.P[p];
  if (a.update) {
    float m = a.beta1 * a.m[p] + (1.0f - a.beta1) * g;
    float v = a.beta2 * a.v[p] + (1.0f - a.beta2) * g * g;
    a.m[p] = m;
    a.v[p] = v;
    const float mh = m / (1.0f - powf(a.beta1, static_cast<float>(t)));
    const float vh = v / (1.0f - powf(a.beta2, static_cast<float>(t)));
    w -= a.lr * mh / (sqrtf(vh) + a.eps);
    a.P[p] = w;
  }
  const __nv_bfloat16 wb = __float2bfloat16_rn(w);
  if (p < P_B1) {
    a.W1[(p / 4) * IN_PAD + p % 4] = wb;
  } else if (p >= P_W2 && p < P_B2) {
    const int o = (p - P_W2) / 128, i = (p - P_W2) % 128;
    a.W2[o * HID + i] = wb;
    a.W2T[i * HID + o] = wb;
  } else if (p >= P_W3 && p < P_B3) {
    const int o = (p - P_W3) / 128, i = (p - P_W3) % 128;
    a.W3[o * HID + i] = wb;
    a.W3T[i * HID + o] = wb;
  }
}

// ------------------------------------------------------------------ input staging
// Writes the BF16 input tile X0[R][16] (features 0-3, zero padding), its
// transpose X0T[16][R] (row 4 = 1 so that column 4 of the first weight
// gradient is the bias gradient), and the constant rows 128-143 of the
// transposed hidden activations (row 128 = 1 for the same reason).
__global__ void k_prepare(const float* __restrict__ x4, long long n, long long R, __nv_bfloat16* X0,
  __nv_bfloat16* X0T, __nv_bfloat16* H1T, __nv_bfloat16* H2T)
{
  const __nv_bfloat16 one = __float2bfloat16_rn(1.0f), zero = __float2bfloat16_rn(0.0f);
  for (long long r = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; r < R;
       r += static_cast<long long>(gridDim.x) * blockDim.x) {
    for (int i = 0; i < IN_PAD; ++i) {
      __nv_bfloat16 v = (i < 4 && r < n) ? __float2bfloat16_rn(x4[r * 4 + i]) : zero;
      X0[r * IN_PAD + i] = v;
      X0T[i * R + r] = (i == 4) ? one : v;
    }
    if (H1T) {
      for (int i = HID; i < MAX_N; ++i) {
        H1T[i * R + r] = (i == HID) ? one : zero;
        H2T[i * R + r] = (i == HID) ? one : zero;
      }
    }
  }
}

// ------------------------------------------------------------------ fused training step
// One persistent kernel for the whole forward and backward pass: each CTA
// (one per SM, 16 warps) walks 128-row tiles and keeps every activation of a
// tile on chip.  Shared memory holds the two hidden weight matrices for the
// whole launch and four 128 x 128 BF16 activation tiles (H1, H2, dZ3, dZ2;
// dZ1 reuses H2's), all in the K-major core-matrix layout by feature:
// element (r, f) at byte ((r/8) 16 + f/8) 128 + (r%8) 16 + (f%8) 2.  The
// products that need a transposed operand (input gradients dZ W: B = W^T;
// weight gradients dZ^T H: A = dZ^T, B = H^T) read the same tiles through
// MN-major descriptors, so no tile is ever written twice.  (The 128-byte
// swizzled layout, which would also serve both readings, measured 2-3 %
// slower in the products.)  Tensor memory
// (512 columns) holds Z2 / dH1 (columns 0-127), Z3 / dH2 and the per-tile
// column sums (128-255), and the dW3 and dW2 accumulators (256-383,
// 384-511), which run over all of the CTA's tiles.  Bias gradients and dW1
// come from N = 16 products against the input tile [x0..x3, 1, 0...]
// (column 4 = 1 gives the column sums); dw4, db4 and the loss are reduced
// over rows with shuffles.  Each CTA writes one partial per gradient in the
// layouts k_adam sums (G1, G2, G3, GH).  Layer 1 (K = 4) runs on the CUDA
// cores.  BF16 rounding happens where the layer-by-layer kernels round:
// inputs, weights, activations and pre-activation gradients.
constexpr int F_THREADS = 512;
constexpr int F_COLS = HID * TILE_M / F_THREADS;  // columns of a row per thread (32)
constexpr int F_GROUPS = HID / F_COLS;           // threads per row (4)
constexpr int TILE_BYTES = TILE_M * HID * 2;   // 32 KB
constexpr int X0_BYTES = TILE_M * IN_PAD * 2;  // 4 KB
constexpr int F_W2 = 0, F_W3 = F_W2 + TILE_BYTES, F_H1 = F_W3 + TILE_BYTES, F_H2 = F_H1 + TILE_BYTES,
              F_DZ3 = F_H2 + TILE_BYTES, F_DZ2 = F_DZ3 + TILE_BYTES, F_X0 = F_DZ2 + TILE_BYTES,
              F_PAR = F_X0 + X0_BYTES,                  // float4 W1[128]; float b1[128], b2[128]; float2 (b3, w4)[128]
              F_RED = F_PAR + (4 * HID + 4 * HID) * 4,  // floats: red[4][128], ypart[4][128], misc[16]
              F_END = F_RED + (4 * HID + F_GROUPS * HID + 16) * 4;
// An MN-major descriptor read spans at most 7 x 4096 + 15 x 2048 + 255 bytes
// past its tile's start under either assignment of the two descriptor
// strides; the allocation covers that from the last tile, so no stride
// reading can leave the CTA's shared memory.
constexpr int F_SPAN = 7 * 4096 + 15 * 2048 + 256;
constexpr int F_SMEM = (F_END > F_DZ2 + F_SPAN ? F_END : F_DZ2 + F_SPAN) + 1024;
static_assert(F_SMEM <= 232448, "fused kernel shared memory");
constexpr uint32_t T_R0 = 0, T_R1 = 128, T_DW3 = 256, T_DW2 = 384;

struct FusedArgs {
  const float* x4;      // [n][4]
  const float* target;  // [n] (train)
  const float* weight;  // [n] (train)
  long long n;
  int tiles;
  int train;
  float inv_n;
  const __nv_bfloat16* W1;  // BF16 operand copies: [128][16], [128][128], [128][128]
  const __nv_bfloat16* W2;
  const __nv_bfloat16* W3;
  const float* P;  // FP32 parameters (biases, w4, b4)
  float* y_out;    // predictions [n] (forward only)
  float* G1;       // per-CTA partials [grid][128][16], [grid][128][144] x 2, [grid][130]
  float* G2;
  float* G3;
  float* GH;
  int* step;
  int* error;
};

// byte offset of element (r, f) of a 128 x 128 tile
__device__ __forceinline__ uint32_t tile_off(int r, int f)
{
  return static_cast<uint32_t>((((r >> 3) * 16 + (f >> 3)) << 7) + ((r & 7) << 4) + ((f & 7) << 1));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ float bf16_round(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }

// Logistic function 1 / (1 + e^-z) = 1 / (1 + 2^(-z log2 e)) from the
// approximate base-2 exponential and reciprocal of the special-function
// unit (each within a few units in the last place of FP32; the results are
// rounded to BF16).
// Large negative z gives 1 / inf = 0, large positive z gives 1.
// Two columns at a time: the FP32 arithmetic of the epilogues runs as packed
// two-wide operations (fma / add / mul .f32x2), the special-function steps
// per column.
__device__ __forceinline__ float ex2_approx(float x)
{
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ float rcp_approx(float x)
{
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ float2 sigm2(float2 z)
{
  const float2 m = __fmul2_rn(z, make_float2(-1.4426950408889634f, -1.4426950408889634f));
  const float2 d = __fadd2_rn(make_float2(ex2_approx(m.x), ex2_approx(m.y)), make_float2(1.0f, 1.0f));
  return make_float2(rcp_approx(d.x), rcp_approx(d.y));
}

// SiLU derivative from z and s = sigmoid(z): s (1 + z (1 - s))
__device__ __forceinline__ float2 silu_grad2(float2 z, float2 s)
{
  const float2 one = make_float2(1.0f, 1.0f);
  const float2 oms = __ffma2_rn(s, make_float2(-1.0f, -1.0f), one);
  return __fmul2_rn(s, __ffma2_rn(z, oms, one));
}

// 16 consecutive FP32 accumulator columns of this thread's row
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v)
{
  uint32_t r[16];
  asm volatile(
    "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
    "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
    : "r"(taddr)
    : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int k = 0; k < 16; ++k) v[k] = __uint_as_float(r[k]);
}

// Issues a load of 16 consecutive FP32 accumulator columns without waiting
// (tmem_wait16 / tmem_wait8 complete it)
__device__ __forceinline__ void tmem_ld16_issue(uint32_t taddr, uint32_t (&r)[16])
{
  asm volatile(
    "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
    "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
      "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
    : "r"(taddr)
    : "memory");
}

// Waits for this thread's outstanding tensor-memory loads.  The destination
// registers of the loads pass through the instruction, so no use of them
// can be placed before it.
__device__ __forceinline__ void tmem_wait16(uint32_t* r)
{
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                 "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                 "+r"(r[15])
               :
               : "memory");
}

// 8 consecutive FP32 accumulator columns of this thread's row, not waited for
__device__ __forceinline__ void tmem_ld8_issue(uint32_t taddr, uint32_t* r)
{
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr)
               : "memory");
}

__device__ __forceinline__ void tmem_wait8(uint32_t* r)
{
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7])
               :
               : "memory");
}

// 8 consecutive floats of a 16-byte aligned shared-memory array
__device__ __forceinline__ void load_f32x8(const float* p, float* v)
{
  const float4 a = reinterpret_cast<const float4*>(p)[0], b = reinterpret_cast<const float4*>(p)[1];
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
  v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}

// Sums 32 values over the 32 lanes of a warp, one column per lane: on
// return lane l holds the sum over all lanes of v[l] (31 shuffles, fixed
// order).  v is overwritten.
__device__ __forceinline__ float lane_column_sums(float (&v)[32], int lane)
{
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) {
    const bool hi = (lane & m) != 0;
#pragma unroll
    for (int i = 0; i < m; ++i) {
      const float send = hi ? v[i] : v[i + m];
      const float keep = hi ? v[i + m] : v[i];
      v[i] = keep + __shfl_xor_sync(0xffffffffu, send, m);
    }
  }
  return v[0];
}

// An operand of one product: the tile's shared-memory address, whether it is
// read MN-major, the bytes its descriptor advances per K step of 16, and
// the descriptor's leading (K direction) / stride (M or N direction) byte
// offsets between core matrices.
struct Operand {
  uint32_t addr;
  bool mn;
  uint32_t kstep, lbo, sbo;
};

// 128 x 128 tile by feature, read with K = features (K-major) or K = rows
// (MN-major: the 8 features of a core-matrix row are the M or N index)
__device__ __forceinline__ Operand big_tile(uint32_t addr, bool mn)
{
  return mn ? Operand{addr, true, 4096u, 2048u, 128u} : Operand{addr, false, 256u, 128u, 2048u};
}

// 128 x 16 input tile read MN-major (N = the 16 input columns, K = rows)
__device__ __forceinline__ Operand x0_tile(uint32_t addr) { return Operand{addr, true, 512u, 256u, 128u}; }

__device__ __forceinline__ uint64_t op_desc(const Operand& o, int j)
{
  return smem_desc(o.addr + j * o.kstep, o.lbo, o.sbo);
}

// D (+)= A B^T over K = 128 in 8 steps of 16 (issued by one thread; an
// issue is accepted about as fast as the tensor core retires products)
__device__ __forceinline__ void issue_product(uint32_t d, const Operand& a, const Operand& b, int n, bool accumulate)
{
  const uint32_t idesc = instr_desc(TILE_M, n) | (a.mn ? 1u << 15 : 0u) | (b.mn ? 1u << 16 : 0u);
#pragma unroll 1
  for (int j = 0; j < HID / 16; ++j) mma_bf16(d, op_desc(a, j), op_desc(b, j), idesc, (accumulate || j > 0) ? 1u : 0u);
}

__global__ void __launch_bounds__(F_THREADS, 1) k_fused(FusedArgs a)
{
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  // layer-1 weights (BF16 values) by neuron pair p = (2p, 2p + 1):
  // sW1[2p] = (W1[2p][0], W1[2p+1][0], W1[2p][1], W1[2p+1][1]), sW1[2p+1] the same for inputs 2, 3
  float4* sW1 = reinterpret_cast<float4*>(base + F_PAR);
  float* sb1 = reinterpret_cast<float*>(sW1 + HID);
  float* sb2 = sb1 + HID;
  float4* sb3w4 = reinterpret_cast<float4*>(sb2 + HID);  // pair p: (b3[2p], b3[2p+1], w4[2p], w4[2p+1])
  float* s_red = reinterpret_cast<float*>(base + F_RED);
  float* s_ypart = s_red + 4 * HID;
  float* s_misc = s_ypart + F_GROUPS * HID;
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_s;

  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  // A warp reaches tensor-memory lanes 32 (warp mod 4) .. + 31: quarter
  // q = warp mod 4, column group h = warp / 4.  Thread 0 also issues the
  // products.
  const int q = warp & 3, h = warp >> 2;
  const int r = 32 * q + lane;  // row of the tile (tensor-memory lane) this thread works on
  const int c0 = F_COLS * h;    // its columns [c0, c0 + F_COLS)
  const bool issuer = t == 0;
  const uint32_t sbase = smem_u32(base);

  if (warp == 0) tmem_alloc(&tmem_s, 512);
  if (t == 0) {
    mbar_init(&mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // weights into the K-major layout (16-byte groups of 8 inputs), layer-1
  // weights and the biases as FP32
  for (int i = t; i < 2 * HID * (HID / 8); i += F_THREADS) {
    const int w = i / (HID * (HID / 8)), k = i % (HID * (HID / 8));
    const int o = k / (HID / 8), g = k % (HID / 8);
    const __nv_bfloat16* src = (w ? a.W3 : a.W2) + o * HID + g * 8;
    *reinterpret_cast<uint4*>(base + (w ? F_W3 : F_W2) + tile_off(o, g * 8)) = *reinterpret_cast<const uint4*>(src);
  }
  for (int o = t; o < HID; o += F_THREADS) {
    const int p = o >> 1, u = o & 1;
    float* w = reinterpret_cast<float*>(sW1 + 2 * p);
    for (int i = 0; i < 4; ++i) w[(i >> 1) * 4 + (i & 1) * 2 + u] = __bfloat162float(a.W1[o * IN_PAD + i]);
    sb1[o] = a.P[P_B1 + o];
    sb2[o] = a.P[P_B2 + o];
    float* bw = reinterpret_cast<float*>(sb3w4 + p);
    bw[u] = a.P[P_B3 + o];
    bw[2 + u] = a.P[P_W4 + o];
  }
  const float b4 = a.P[P_B4];
  fence_async_shared();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_s;
  const uint32_t t_row = tmem + (static_cast<uint32_t>(32 * q) << 16);

  float acc_dw4 = 0.0f, acc_db3 = 0.0f, acc_db2 = 0.0f, acc_db1 = 0.0f, acc_db4 = 0.0f, acc_loss = 0.0f;
  float acc_dw1[4] = {0.0f, 0.0f, 0.0f, 0.0f};
  uint32_t phase = 0;
  bool ok = true, first = true;

  auto wait_products = [&]() {
    const bool done = mbar_wait(&mbar, phase & 1u, WAIT_TRIES);
    ++phase;
    ok = ok && done;
    tc_fence_after();
  };
  // all threads: shared-memory tiles written, tensor-memory reads done
  auto tiles_ready = [&]() -> bool {
    fence_async_shared();
    tc_fence_before();
    const bool all = __syncthreads_and(ok);
    tc_fence_after();
    return all;
  };
  // pre-activations of layer 1 for neurons o, o + 1 (o even) with biases b
  auto z1_of = [&](const float2 (&xx)[4], int o, float2 b) {
    const float4 wa = sW1[o], wb = sW1[o + 1];
    float2 z = __ffma2_rn(xx[0], make_float2(wa.x, wa.y), b);
    z = __ffma2_rn(xx[1], make_float2(wa.z, wa.w), z);
    z = __ffma2_rn(xx[2], make_float2(wb.x, wb.y), z);
    return __ffma2_rn(xx[3], make_float2(wb.z, wb.w), z);
  };

  // inputs of this thread's row, loaded one tile ahead
  auto load_x = [&](int tile) {
    const long long row = static_cast<long long>(tile) * TILE_M + r;
    return (tile < a.tiles && row < a.n) ? __ldg(reinterpret_cast<const float4*>(a.x4 + row * 4))
                                         : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  };
  float4 x_next = load_x(blockIdx.x);

  for (int tile = blockIdx.x; tile < a.tiles; tile += gridDim.x) {
    const long long rg = static_cast<long long>(tile) * TILE_M + r;
    const bool real = rg < a.n;
    // target and weight are used after the forward pass
    float tgt = 0.0f, wt = 0.0f;
    if (a.train && real) {
      tgt = __ldg(a.target + rg);
      wt = __ldg(a.weight + rg);
    }
    // ---- layer 1 on the CUDA cores: H1 = silu(X0 W1^T + b1)
    const float x[4] = {bf16_round(x_next.x), bf16_round(x_next.y), bf16_round(x_next.z), bf16_round(x_next.w)};
    const float2 xx[4] = {make_float2(x[0], x[0]), make_float2(x[1], x[1]), make_float2(x[2], x[2]),
                          make_float2(x[3], x[3])};
    x_next = load_x(tile + gridDim.x);
    if (h == 0) {
      *reinterpret_cast<uint4*>(base + F_X0 + ((r >> 3) * 2 << 7) + ((r & 7) << 4)) =
        make_uint4(pack_bf16(x[0], x[1]), pack_bf16(x[2], x[3]), pack_bf16(1.0f, 0.0f), 0u);
      *reinterpret_cast<uint4*>(base + F_X0 + (((r >> 3) * 2 + 1) << 7) + ((r & 7) << 4)) = make_uint4(0u, 0u, 0u, 0u);
    }
    {
#pragma unroll
      for (int g = 0; g < F_COLS / 8; ++g) {
        uint32_t pk[4];
        float b[8];
        load_f32x8(sb1 + c0 + 8 * g, b);
#pragma unroll
        for (int e = 0; e < 8; e += 2) {
          const float2 z = z1_of(xx, c0 + 8 * g + e, make_float2(b[e], b[e + 1]));
          const float2 hv = __fmul2_rn(z, sigm2(z));
          pk[e / 2] = pack_bf16(hv.x, hv.y);
        }
        *reinterpret_cast<uint4*>(base + F_H1 + tile_off(r, c0 + 8 * g)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
    if (!tiles_ready()) break;
    if (issuer) {
      issue_product(tmem + T_R0, big_tile(sbase + F_H1, false), big_tile(sbase + F_W2, false), HID, false);
      mma_commit(&mbar);
    }
    wait_products();
    // ---- layer 2 epilogue: H2 = silu(Z2 + b2)
    {
      float v[32];
      tmem_ld32(t_row + T_R0 + c0, v);
#pragma unroll
      for (int g = 0; g < 4; ++g) {
        uint32_t pk[4];
        float b[8];
        load_f32x8(sb2 + c0 + 8 * g, b);
#pragma unroll
        for (int e = 0; e < 8; e += 2) {
          const int k = 8 * g + e;
          const float2 z = __fadd2_rn(make_float2(v[k], v[k + 1]), make_float2(b[e], b[e + 1]));
          const float2 hv = __fmul2_rn(z, sigm2(z));
          pk[e / 2] = pack_bf16(hv.x, hv.y);
        }
        *reinterpret_cast<uint4*>(base + F_H2 + tile_off(r, c0 + 8 * g)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
    if (!tiles_ready()) break;
    if (issuer) {
      issue_product(tmem + T_R1, big_tile(sbase + F_H2, false), big_tile(sbase + F_W3, false), HID, false);
      mma_commit(&mbar);
    }
    wait_products();
    // ---- layer 3 epilogue and the output layer: H3 = silu(Z3 + b3),
    // y = H3 . w4 + b4; g3 = w4 silu'(Z3) is kept for dZ3 = dy g3
    float2 g3[16];
    uint32_t h3[16];
    float ypart = 0.0f;
    {
      float2 yp = make_float2(0.0f, 0.0f);
#pragma unroll
      for (int half = 0; half < 32; half += 16) {
        float v[16];
        tmem_ld16(t_row + T_R1 + c0 + half, v);
#pragma unroll
        for (int k = 0; k < 16; k += 2) {
          const int kk = half + k;
          const float4 bw = sb3w4[(c0 + kk) >> 1];  // b3, w4 of neurons c0 + kk, c0 + kk + 1
          const float2 w4 = make_float2(bw.z, bw.w);
          const float2 z = __fadd2_rn(make_float2(v[k], v[k + 1]), make_float2(bw.x, bw.y));
          const float2 sg = sigm2(z);
          const float2 hv = __fmul2_rn(z, sg);
          h3[kk / 2] = pack_bf16(hv.x, hv.y);
          const __nv_bfloat162 hp = *reinterpret_cast<const __nv_bfloat162*>(&h3[kk / 2]);
          yp = __ffma2_rn(make_float2(__low2float(hp), __high2float(hp)), w4, yp);
          g3[kk / 2] = __fmul2_rn(w4, silu_grad2(z, sg));
        }
      }
      ypart = yp.x + yp.y;
    }
    s_ypart[h * HID + r] = ypart;
    __syncthreads();
    const float y = b4 + (((s_ypart[r] + s_ypart[HID + r]) + s_ypart[2 * HID + r]) + s_ypart[3 * HID + r]);
    if (!a.train) {
      if (h == 0 && real) a.y_out[rg] = y;
      tc_fence_before();
      __syncthreads();
      continue;
    }
    float dy = 0.0f, loss = 0.0f;
    if (real) {
      const float e = y - tgt;
      loss = wt * e * e * a.inv_n;
      dy = 2.0f * wt * e * a.inv_n;
    }
    // dZ3 = bf16(dy g3) into its tile; dw4 = sum over rows of dy H3
    const float2 dy2 = make_float2(dy, dy);
    {
#pragma unroll
    for (int g = 0; g < 4; ++g) {
      uint32_t pk[4];
#pragma unroll
      for (int e = 0; e < 8; e += 2) {
        const float2 d = __fmul2_rn(dy2, g3[(8 * g + e) / 2]);
        pk[e / 2] = pack_bf16(d.x, d.y);
      }
      *reinterpret_cast<uint4*>(base + F_DZ3 + tile_off(r, c0 + 8 * g)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    }
    {
      float v[32];
#pragma unroll
      for (int k = 0; k < 32; k += 2) {
        const __nv_bfloat162 p = *reinterpret_cast<const __nv_bfloat162*>(&h3[k / 2]);
        const float2 d = __fmul2_rn(dy2, make_float2(__low2float(p), __high2float(p)));
        v[k] = d.x;
        v[k + 1] = d.y;
      }
      s_red[q * HID + c0 + lane] = lane_column_sums(v, lane);
    }
    }
    if (h == 0) {
      float sd = dy, sl = loss;
#pragma unroll
      for (int m = 16; m >= 1; m >>= 1) {
        sd += __shfl_xor_sync(0xffffffffu, sd, m);
        sl += __shfl_xor_sync(0xffffffffu, sl, m);
      }
      if (lane == 0) {
        s_misc[q] = sd;
        s_misc[4 + q] = sl;
      }
    }
    if (!tiles_ready()) break;
    if (h == 0) acc_dw4 += ((s_red[r] + s_red[HID + r]) + s_red[2 * HID + r]) + s_red[3 * HID + r];
    if (issuer) {
      acc_db4 += ((s_misc[0] + s_misc[1]) + s_misc[2]) + s_misc[3];
      acc_loss += ((s_misc[4] + s_misc[5]) + s_misc[6]) + s_misc[7];
    }
    if (issuer) {
      // dH2 = dZ3 W3 (B = W3 read MN-major); dW3 += dZ3^T H2 runs on
      // while dZ2 is formed (it reads neither tensor-memory columns 0-255
      // nor the dZ2 tile)
      issue_product(tmem + T_R1, big_tile(sbase + F_DZ3, false), big_tile(sbase + F_W3, true), HID, false);
      mma_commit(&mbar);
      issue_product(tmem + T_DW3, big_tile(sbase + F_DZ3, true), big_tile(sbase + F_H2, true), HID, !first);
    }
    wait_products();
    // ---- dZ2 = bf16(dH2 silu'(Z2)), Z2 still in columns 0-127
    {
#pragma unroll
      for (int half = 0; half < 32; half += 16) {
        uint32_t dhr[16], zr[16];
        tmem_ld16_issue(t_row + T_R1 + c0 + half, dhr);
        tmem_ld16_issue(t_row + T_R0 + c0 + half, zr);
        tmem_wait16(dhr);
        tmem_wait16(zr);
#pragma unroll
        for (int g = 0; g < 2; ++g) {
          uint32_t pk[4];
          float b[8];
          load_f32x8(sb2 + c0 + half + 8 * g, b);
#pragma unroll
          for (int e = 0; e < 8; e += 2) {
            const int k = 8 * g + e;
            const float2 zz = __fadd2_rn(make_float2(__uint_as_float(zr[k]), __uint_as_float(zr[k + 1])),
                                         make_float2(b[e], b[e + 1]));
            const float2 d = __fmul2_rn(make_float2(__uint_as_float(dhr[k]), __uint_as_float(dhr[k + 1])),
                                        silu_grad2(zz, sigm2(zz)));
            pk[e / 2] = pack_bf16(d.x, d.y);
          }
          *reinterpret_cast<uint4*>(base + F_DZ2 + tile_off(r, c0 + half + 8 * g)) =
            make_uint4(pk[0], pk[1], pk[2], pk[3]);
        }
      }
    }
    if (!tiles_ready()) break;
    if (issuer) {
      // dH1 = dZ2 W2 (its completion also covers the dW3 product issued
      // before it); then dW2 += dZ2^T H1 and the column sums of dZ3 and dZ2
      // (db3, db2) run on while dZ1 is formed
      issue_product(tmem + T_R0, big_tile(sbase + F_DZ2, false), big_tile(sbase + F_W2, true), HID, false);
      mma_commit(&mbar);
      issue_product(tmem + T_DW2, big_tile(sbase + F_DZ2, true), big_tile(sbase + F_H1, true), HID, !first);
      issue_product(tmem + T_R1, big_tile(sbase + F_DZ3, true), x0_tile(sbase + F_X0), IN_PAD, false);
      issue_product(tmem + T_R1 + 32, big_tile(sbase + F_DZ2, true), x0_tile(sbase + F_X0), IN_PAD, false);
    }
    wait_products();
    // ---- dZ1 = bf16(dH1 silu'(Z1)) into H2's tile (dW3, its last reader,
    // completed before dH1)
    {
      float dh[32];
      tmem_ld32(t_row + T_R0 + c0, dh);
#pragma unroll
      for (int g = 0; g < 4; ++g) {
        uint32_t pk[4];
        float b[8];
        load_f32x8(sb1 + c0 + 8 * g, b);
#pragma unroll
        for (int e = 0; e < 8; e += 2) {
          const int k = 8 * g + e;
          const float2 zz = z1_of(xx, c0 + k, make_float2(b[e], b[e + 1]));
          const float2 d = __fmul2_rn(make_float2(dh[k], dh[k + 1]), silu_grad2(zz, sigm2(zz)));
          pk[e / 2] = pack_bf16(d.x, d.y);
        }
        *reinterpret_cast<uint4*>(base + F_H2 + tile_off(r, c0 + 8 * g)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
    if (!tiles_ready()) break;
    if (issuer) {
      // dW1 (columns 0-3) and db1 (column 4); the commit covers every
      // product of the tile
      issue_product(tmem + T_R1 + 64, big_tile(sbase + F_H2, true), x0_tile(sbase + F_X0), IN_PAD, false);
      mma_commit(&mbar);
    }
    wait_products();
    if (h == 0) {
      uint32_t v[24];
      tmem_ld8_issue(t_row + T_R1, v);
      tmem_ld8_issue(t_row + T_R1 + 32, v + 8);
      tmem_ld8_issue(t_row + T_R1 + 64, v + 16);
      tmem_wait16(v);
      tmem_wait8(v + 16);
      acc_db3 += __uint_as_float(v[4]);
      acc_db2 += __uint_as_float(v[12]);
#pragma unroll
      for (int i = 0; i < 4; ++i) acc_dw1[i] += __uint_as_float(v[16 + i]);
      acc_db1 += __uint_as_float(v[20]);
    }
    first = false;
    // No barrier here: every product of the tile has completed, and the next
    // tile overwrites columns 128-255 (read just above) only after two more
    // barriers.
    tc_fence_before();
  }

  if (!ok) {
    if (t == 0) atomicOr(a.error, ERR_TIMEOUT);
  } else if (a.train) {
    // this CTA's partials: tensor-memory lane = output neuron
    const int o = r;
    float* g2 = a.G2 + (static_cast<long long>(blockIdx.x) * HID + o) * G_N;
    float* g3 = a.G3 + (static_cast<long long>(blockIdx.x) * HID + o) * G_N;
    float v[32];
    tmem_ld32(t_row + T_DW3 + c0, v);
#pragma unroll
    for (int k = 0; k < 32; k += 4)
      *reinterpret_cast<float4*>(g3 + c0 + k) = make_float4(v[k], v[k + 1], v[k + 2], v[k + 3]);
    tmem_ld32(t_row + T_DW2 + c0, v);
#pragma unroll
    for (int k = 0; k < 32; k += 4)
      *reinterpret_cast<float4*>(g2 + c0 + k) = make_float4(v[k], v[k + 1], v[k + 2], v[k + 3]);
    if (h == 0) {
      g3[HID] = acc_db3;
      g2[HID] = acc_db2;
      float* g1 = a.G1 + (static_cast<long long>(blockIdx.x) * HID + o) * G1_N;
#pragma unroll
      for (int i = 0; i < 4; ++i) g1[i] = acc_dw1[i];
      g1[4] = acc_db1;
      float* gh = a.GH + static_cast<long long>(blockIdx.x) * 130;
      gh[r] = acc_dw4;
      if (t == 0) {
        gh[128] = acc_db4;
        gh[129] = acc_loss;
        if (blockIdx.x == 0) a.step[0] += 1;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_dealloc(tmem, 512);
  }
}

__global__ void k_fill_f32(float* p, long long n, float v)
{
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x)
    p[i] = v;
}

// ------------------------------------------------------------------ host
#define MLP_CK(x)                                                                                    \
  do {                                                                                               \
    cudaError_t e_ = (x);                                                                            \
    if (e_ != cudaSuccess) throw std::runtime_error(std::string("CUDA: ") + cudaGetErrorString(e_)); \
  } while (0)

struct Net {
  int device = 0;
  int n_sm = 0;
  long long cap = 0;  // rows (multiple of 128)
  long long n = 0, R = 0;
  int splits = 0, k_split = 0;
  int max_splits = 0;
  int fused_grid = 0;     // CTAs of the last fused launch (= its gradient partials)
  bool graph_fused = false;
  bool prepared = false;  // staged rows converted for the layer-by-layer kernels
  cudaStream_t stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  float graph_lr = -1.0f;
  float last_ms = 0.0f;
  // parameters, optimizer state, gradients
  float *P = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr, *loss_hist = nullptr;
  int *step = nullptr, *err = nullptr;
  long long loss_cap = 0;
  __nv_bfloat16 *W1 = nullptr, *W2 = nullptr, *W2T = nullptr, *W3 = nullptr, *W3T = nullptr;
  float *G1 = nullptr, *G2 = nullptr, *G3 = nullptr, *GH = nullptr;
  // data and activations
  float *x4 = nullptr, *target = nullptr, *weight = nullptr, *y = nullptr;
  // layer-by-layer kernels only (allocated on first use)
  __nv_bfloat16 *X0 = nullptr, *X0T = nullptr;
  float *Z1 = nullptr, *Z2 = nullptr, *Z3 = nullptr;
  __nv_bfloat16 *H1 = nullptr, *H2 = nullptr, *H3 = nullptr, *H1T = nullptr, *H2T = nullptr;
  __nv_bfloat16 *dZ1 = nullptr, *dZ2 = nullptr, *dZ3 = nullptr, *dZ1T = nullptr, *dZ2T = nullptr, *dZ3T = nullptr;
  std::vector<void*> allocs;

  template <class T>
  T* alloc(size_t count)
  {
    void* p = nullptr;
    MLP_CK(cudaMalloc(&p, count * sizeof(T) + 16));
    MLP_CK(cudaMemset(p, 0, count * sizeof(T) + 16));
    allocs.push_back(p);
    return static_cast<T*>(p);
  }

  ~Net()
  {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    for (void* p : allocs) cudaFree(p);
    if (stream) cudaStreamDestroy(stream);
  }
};

static bool g_attr_set[64] = {false};

static void set_gemm_attributes(int dev)
{
  if (dev >= 0 && dev < 64 && g_attr_set[dev]) return;
  MLP_CK(cudaFuncSetAttribute(k_gemm<EPI_FORWARD>, cudaFuncAttributeMaxDynamicSharedMemorySize, GEMM_SMEM));
  MLP_CK(cudaFuncSetAttribute(k_gemm<EPI_DINPUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, GEMM_SMEM));
  MLP_CK(cudaFuncSetAttribute(k_gemm<EPI_DWEIGHT>, cudaFuncAttributeMaxDynamicSharedMemorySize, GEMM_SMEM));
  MLP_CK(cudaFuncSetAttribute(k_fused, cudaFuncAttributeMaxDynamicSharedMemorySize, F_SMEM));
  if (dev >= 0 && dev < 64) g_attr_set[dev] = true;
}

static GemmArgs gemm_args(Net& N)
{
  GemmArgs g;
  std::memset(&g, 0, sizeof(g));
  g.error = N.err;
  return g;
}

template <int EPI>
static void launch_gemm(Net& N, const GemmArgs& g, int grid)
{
  k_gemm<EPI><<<grid, 128, GEMM_SMEM, N.stream>>>(g);
  MLP_CK(cudaGetLastError());
}

// Forward pass over the N.R staged rows; `train` also writes the transposed
// activations and runs the output layer's backward part.
static void enqueue_forward(Net& N, bool train, float* y_out)
{
  const int tiles = static_cast<int>(N.R / TILE_M);
  N.fused_grid = 0;
  const int ldT = static_cast<int>(N.R);
  GemmArgs g = gemm_args(N);
  g.A = N.X0; g.lda = IN_PAD; g.B = N.W1; g.ldb = IN_PAD; g.K = IN_PAD; g.N = HID;
  g.bias = N.P + P_B1; g.Z = N.Z1; g.H = N.H1; g.HT = train ? N.H1T : nullptr; g.ldT = ldT;
  launch_gemm<EPI_FORWARD>(N, g, tiles);
  g.A = N.H1; g.lda = HID; g.B = N.W2; g.ldb = HID; g.K = HID;
  g.bias = N.P + P_B2; g.Z = N.Z2; g.H = N.H2; g.HT = train ? N.H2T : nullptr;
  launch_gemm<EPI_FORWARD>(N, g, tiles);
  g.A = N.H2; g.B = N.W3; g.bias = N.P + P_B3; g.Z = N.Z3; g.H = N.H3; g.HT = nullptr;
  launch_gemm<EPI_FORWARD>(N, g, tiles);
  const float inv_n = N.n > 0 ? 1.0f / static_cast<float>(N.n) : 0.0f;
  k_head<<<tiles, TILE_M, 0, N.stream>>>(N.H3, N.Z3, N.P + P_W4, N.P + P_B4, N.target, N.weight,
    static_cast<int>(N.n), static_cast<int>(N.R), inv_n, train ? N.dZ3 : nullptr, N.dZ3T, N.GH, y_out, N.step);
  MLP_CK(cudaGetLastError());
}

static void enqueue_backward(Net& N)
{
  const int tiles = static_cast<int>(N.R / TILE_M);
  const int K = static_cast<int>(N.R);
  GemmArgs g = gemm_args(N);
  // dW3 = dZ3^T [H2 | 1]
  g.A = N.dZ3T; g.lda = K; g.B = N.H2T; g.ldb = K; g.K = K; g.N = G_N; g.k_split = N.k_split; g.dW = N.G3;
  launch_gemm<EPI_DWEIGHT>(N, g, N.splits);
  // dZ2 = (dZ3 W3) * silu'(Z2)
  g = gemm_args(N);
  g.A = N.dZ3; g.lda = HID; g.B = N.W3T; g.ldb = HID; g.K = HID; g.N = HID;
  g.Zprev = N.Z2; g.dZprev = N.dZ2; g.HT = N.dZ2T; g.ldT = K;
  launch_gemm<EPI_DINPUT>(N, g, tiles);
  // dW2 = dZ2^T [H1 | 1]
  g = gemm_args(N);
  g.A = N.dZ2T; g.lda = K; g.B = N.H1T; g.ldb = K; g.K = K; g.N = G_N; g.k_split = N.k_split; g.dW = N.G2;
  launch_gemm<EPI_DWEIGHT>(N, g, N.splits);
  // dZ1 = (dZ2 W2) * silu'(Z1)
  g = gemm_args(N);
  g.A = N.dZ2; g.lda = HID; g.B = N.W2T; g.ldb = HID; g.K = HID; g.N = HID;
  g.Zprev = N.Z1; g.dZprev = N.dZ1; g.HT = N.dZ1T; g.ldT = K;
  launch_gemm<EPI_DINPUT>(N, g, tiles);
  // dW1 = dZ1^T [X0 | 1]
  g = gemm_args(N);
  g.A = N.dZ1T; g.lda = K; g.B = N.X0T; g.ldb = K; g.K = K; g.N = G1_N; g.k_split = N.k_split; g.dW = N.G1;
  launch_gemm<EPI_DWEIGHT>(N, g, N.splits);
}

// Activation buffers of the layer-by-layer kernels (cap rows each), and the
// staged rows converted to their BF16 input tiles.
static void prepare_layers(Net& N)
{
  if (!N.Z1) {
    const long long R = N.cap;
    N.X0 = N.alloc<__nv_bfloat16>(R * IN_PAD);
    N.X0T = N.alloc<__nv_bfloat16>(R * IN_PAD);
    N.Z1 = N.alloc<float>(R * HID);
    N.Z2 = N.alloc<float>(R * HID);
    N.Z3 = N.alloc<float>(R * HID);
    N.H1 = N.alloc<__nv_bfloat16>(R * HID);
    N.H2 = N.alloc<__nv_bfloat16>(R * HID);
    N.H3 = N.alloc<__nv_bfloat16>(R * HID);
    N.H1T = N.alloc<__nv_bfloat16>(R * MAX_N);
    N.H2T = N.alloc<__nv_bfloat16>(R * MAX_N);
    N.dZ1 = N.alloc<__nv_bfloat16>(R * HID);
    N.dZ2 = N.alloc<__nv_bfloat16>(R * HID);
    N.dZ3 = N.alloc<__nv_bfloat16>(R * HID);
    N.dZ1T = N.alloc<__nv_bfloat16>(R * HID);
    N.dZ2T = N.alloc<__nv_bfloat16>(R * HID);
    N.dZ3T = N.alloc<__nv_bfloat16>(R * HID);
  }
  if (!N.prepared && N.R > 0) {
    k_prepare<<<152, 256, 0, N.stream>>>(N.x4, N.n, N.R, N.X0, N.X0T, N.H1T, N.H2T);
    MLP_CK(cudaGetLastError());
    N.prepared = true;
  }
}

// The fused kernel over the N.R staged rows: a training pass (gradient
// partials, one per CTA) or the forward pass into y_out.
static void enqueue_fused(Net& N, bool train, float* y_out)
{
  const int tiles = static_cast<int>(N.R / TILE_M);
  FusedArgs f;
  std::memset(&f, 0, sizeof(f));
  f.x4 = N.x4;
  f.target = N.target;
  f.weight = N.weight;
  f.n = N.n;
  f.tiles = tiles;
  f.train = train ? 1 : 0;
  f.inv_n = N.n > 0 ? 1.0f / static_cast<float>(N.n) : 0.0f;
  f.W1 = N.W1;
  f.W2 = N.W2;
  f.W3 = N.W3;
  f.P = N.P;
  f.y_out = y_out;
  f.G1 = N.G1;
  f.G2 = N.G2;
  f.G3 = N.G3;
  f.GH = N.GH;
  f.step = N.step;
  f.error = N.err;
  const int grid = std::max(1, std::min(tiles, N.n_sm));
  k_fused<<<grid, F_THREADS, F_SMEM, N.stream>>>(f);
  MLP_CK(cudaGetLastError());
  N.fused_grid = grid;
}

static AdamArgs adam_args(Net& N, int update, float lr)
{
  AdamArgs a;
  std::memset(&a, 0, sizeof(a));
  a.P = N.P; a.m = N.m; a.v = N.v;
  a.G1 = N.G1; a.G2 = N.G2; a.G3 = N.G3; a.GH = N.GH;
  if (N.fused_grid > 0) {
    a.splits = N.fused_grid;
    a.head_blocks = N.fused_grid;
  } else {
    a.splits = N.splits;
    a.head_blocks = static_cast<int>(N.R / TILE_M);
  }
  a.lr = lr; a.beta1 = 0.9f; a.beta2 = 0.999f; a.eps = 1e-8f;
  a.step = N.step; a.update = update;
  a.W1 = N.W1; a.W2 = N.W2; a.W2T = N.W2T; a.W3 = N.W3; a.W3T = N.W3T;
  return a;
}

static void enqueue_adam(Net& N, const AdamArgs& a)
{
  k_adam<<<(N_PARAMS + 255) / 256, 256, 0, N.stream>>>(a);
  MLP_CK(cudaGetLastError());
}

static void check_error(Net& N)
{
  int e = 0;
  MLP_CK(cudaMemcpyAsync(&e, N.err, sizeof(int), cudaMemcpyDeviceToHost, N.stream));
  MLP_CK(cudaStreamSynchronize(N.stream));
  if (e) {
    MLP_CK(cudaMemsetAsync(N.err, 0, sizeof(int), N.stream));
    throw std::runtime_error("tensor-core product did not complete within its wait limit");
  }
}

static void drop_graph(Net& N)
{
  if (N.exec) cudaGraphExecDestroy(N.exec);
  if (N.graph) cudaGraphDestroy(N.graph);
  N.exec = nullptr;
  N.graph = nullptr;
}

static uint64_t splitmix(uint64_t& s)
{
  uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

// LeCun-uniform weights (variance 1/fan_in), zero biases.
static std::vector<float> init_params(uint64_t seed)
{
  std::vector<float> p(N_PARAMS, 0.0f);
  uint64_t s = seed;
  auto fill = [&](int off, int count, int fan_in) {
    const double a = std::sqrt(3.0 / fan_in);
    for (int i = 0; i < count; ++i) {
      double u = static_cast<double>(splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
      p[off + i] = static_cast<float>((2.0 * u - 1.0) * a);
    }
  };
  fill(P_W1, 512, 4);
  fill(P_W2, 16384, HID);
  fill(P_W3, 16384, HID);
  fill(P_W4, HID, HID);
  return p;
}

static void upload_params(Net& N, const float* p)
{
  MLP_CK(cudaMemcpyAsync(N.P, p, sizeof(float) * N_PARAMS, cudaMemcpyHostToDevice, N.stream));
  MLP_CK(cudaMemsetAsync(N.m, 0, sizeof(float) * N_PARAMS, N.stream));
  MLP_CK(cudaMemsetAsync(N.v, 0, sizeof(float) * N_PARAMS, N.stream));
  MLP_CK(cudaMemsetAsync(N.step, 0, sizeof(int), N.stream));
  // refresh the BF16 copies without an update (no gradient partials yet: splits = 0)
  AdamArgs a = adam_args(N, 0, 0.0f);
  a.splits = 0;
  a.head_blocks = 0;
  enqueue_adam(N, a);
  MLP_CK(cudaStreamSynchronize(N.stream));
}

}  // namespace mlp

// ------------------------------------------------------------------ C API
extern "C" char openmc_err_msg[256];
extern "C" int OPENMC_E_ALLOCATE;
extern "C" int OPENMC_E_INVALID_ARGUMENT;
extern "C" int OPENMC_E_UNASSIGNED;

extern "C" {
// 1 (default): each training step and query runs the fused per-tile kernel;
// 0: the layer-by-layer kernels (activations through device memory).
int openmc_gb300_mlp_fused = 1;
}

namespace {

int fail(int code, const char* what)
{
  std::snprintf(openmc_err_msg, sizeof(openmc_err_msg), "%s", what);
  return code;
}

// One forward (+ backward when training) pass over the staged rows.
void enqueue_pass(mlp::Net& N, bool train, float* y_out)
{
  if (openmc_gb300_mlp_fused) {
    mlp::enqueue_fused(N, train, y_out);
  } else {
    mlp::prepare_layers(N);
    mlp::enqueue_forward(N, train, y_out);
    if (train) mlp::enqueue_backward(N);
  }
}

}  // namespace

extern "C" {

// Number of FP32 parameters of the importance network (33,793).
int openmc_gb300_mlp_n_params(void) { return mlp::N_PARAMS; }

// Creates a network with seeded LeCun-uniform weights on the current device,
// with room for max_rows training or query rows.
int openmc_gb300_mlp_create(int64_t max_rows, uint64_t seed, void** handle)
{
  using namespace mlp;
  if (!handle || max_rows <= 0) return fail(OPENMC_E_INVALID_ARGUMENT, "invalid network capacity");
  Net* N = nullptr;
  try {
    N = new Net();
    MLP_CK(cudaGetDevice(&N->device));
    MLP_CK(cudaDeviceGetAttribute(&N->n_sm, cudaDevAttrMultiProcessorCount, N->device));
    set_gemm_attributes(N->device);
    MLP_CK(cudaStreamCreateWithFlags(&N->stream, cudaStreamNonBlocking));
    N->cap = (max_rows + TILE_M - 1) / TILE_M * TILE_M;
    const long long R = N->cap;
    N->max_splits = 320;
    N->P = N->alloc<float>(N_PARAMS);
    N->m = N->alloc<float>(N_PARAMS);
    N->v = N->alloc<float>(N_PARAMS);
    N->grad = N->alloc<float>(N_PARAMS);
    N->loss_cap = 1 << 16;
    N->loss_hist = N->alloc<float>(N->loss_cap);
    N->step = N->alloc<int>(1);
    N->err = N->alloc<int>(1);
    N->W1 = N->alloc<__nv_bfloat16>(HID * IN_PAD);
    N->W2 = N->alloc<__nv_bfloat16>(HID * HID);
    N->W2T = N->alloc<__nv_bfloat16>(HID * HID);
    N->W3 = N->alloc<__nv_bfloat16>(HID * HID);
    N->W3T = N->alloc<__nv_bfloat16>(HID * HID);
    N->G1 = N->alloc<float>(static_cast<size_t>(N->max_splits) * HID * G1_N);
    N->G2 = N->alloc<float>(static_cast<size_t>(N->max_splits) * HID * G_N);
    N->G3 = N->alloc<float>(static_cast<size_t>(N->max_splits) * HID * G_N);
    N->GH = N->alloc<float>(static_cast<size_t>(R / TILE_M) * 130);
    N->x4 = N->alloc<float>(R * 4);
    N->target = N->alloc<float>(R);
    N->weight = N->alloc<float>(R);
    N->y = N->alloc<float>(R);
    std::vector<float> p = init_params(seed);
    upload_params(*N, p.data());
    *handle = N;
    return 0;
  } catch (const std::exception& e) {
    delete N;
    return fail(OPENMC_E_ALLOCATE, e.what());
  }
}

int openmc_gb300_mlp_free(void* handle)
{
  delete static_cast<mlp::Net*>(handle);
  return 0;
}

// Stages n training rows: x4 = n x (x, y, z, log E) features (host, FP32,
// already scaled to about [-1, 1]), target = n values of the regression
// target, weight = n per-row loss weights (NULL: all 1).
int openmc_gb300_mlp_set_data(void* handle, int64_t n, const float* x4, const float* target, const float* weight)
{
  using namespace mlp;
  Net* N = static_cast<Net*>(handle);
  if (!N || n <= 0 || !x4 || !target) return fail(OPENMC_E_INVALID_ARGUMENT, "invalid training data");
  try {
    const long long R = (n + TILE_M - 1) / TILE_M * TILE_M;
    if (R > N->cap) return fail(OPENMC_E_INVALID_ARGUMENT, "more rows than the network was created for");
    N->n = n;
    N->R = R;
    // about two weight-gradient tiles per SM, each at least 256 rows deep
    long long per = (R + 295) / 296;
    N->k_split = static_cast<int>(std::max<long long>(256, (per + KC - 1) / KC * KC));
    N->splits = static_cast<int>((R + N->k_split - 1) / N->k_split);
    if (N->splits > N->max_splits) return fail(OPENMC_E_INVALID_ARGUMENT, "too many gradient partials");
    MLP_CK(cudaMemsetAsync(N->target, 0, sizeof(float) * R, N->stream));
    MLP_CK(cudaMemcpyAsync(N->x4, x4, sizeof(float) * 4 * n, cudaMemcpyHostToDevice, N->stream));
    MLP_CK(cudaMemcpyAsync(N->target, target, sizeof(float) * n, cudaMemcpyHostToDevice, N->stream));
    if (weight) {
      MLP_CK(cudaMemsetAsync(N->weight, 0, sizeof(float) * R, N->stream));
      MLP_CK(cudaMemcpyAsync(N->weight, weight, sizeof(float) * n, cudaMemcpyHostToDevice, N->stream));
    } else {
      k_fill_f32<<<64, 256, 0, N->stream>>>(N->weight, R, 1.0f);
      MLP_CK(cudaGetLastError());
    }
    N->prepared = false;
    if (N->Z1) prepare_layers(*N);
    MLP_CK(cudaStreamSynchronize(N->stream));
    drop_graph(*N);
    return 0;
  } catch (const std::exception& e) {
    return fail(OPENMC_E_ALLOCATE, e.what());
  }
}

// Runs `steps` full-batch Adam steps (learning rate lr) on the staged rows,
// as one CUDA graph per step.  loss_history (host, may be NULL) receives the
// loss before each step's update.
int openmc_gb300_mlp_train(void* handle, int steps, double lr, float* loss_history)
{
  using namespace mlp;
  Net* N = static_cast<Net*>(handle);
  if (!N || steps < 0 || N->R == 0) return fail(OPENMC_E_INVALID_ARGUMENT, "no training data staged");
  try {
    int t0 = 0;
    MLP_CK(cudaMemcpyAsync(&t0, N->step, sizeof(int), cudaMemcpyDeviceToHost, N->stream));
    MLP_CK(cudaStreamSynchronize(N->stream));
    if (t0 + steps > N->loss_cap) return fail(OPENMC_E_INVALID_ARGUMENT, "too many optimizer steps");
    const bool fused = openmc_gb300_mlp_fused != 0;
    if (!N->exec || N->graph_lr != static_cast<float>(lr) || N->graph_fused != fused) {
      drop_graph(*N);
      if (!fused) prepare_layers(*N);  // buffers and input tiles outside the capture
      MLP_CK(cudaStreamBeginCapture(N->stream, cudaStreamCaptureModeThreadLocal));
      enqueue_pass(*N, true, nullptr);
      AdamArgs a = adam_args(*N, 1, static_cast<float>(lr));
      a.loss_out = N->loss_hist;
      enqueue_adam(*N, a);
      MLP_CK(cudaStreamEndCapture(N->stream, &N->graph));
      MLP_CK(cudaGraphInstantiate(&N->exec, N->graph, 0));
      N->graph_lr = static_cast<float>(lr);
      N->graph_fused = fused;
    }
    cudaEvent_t e0, e1;
    MLP_CK(cudaEventCreate(&e0));
    MLP_CK(cudaEventCreate(&e1));
    MLP_CK(cudaEventRecord(e0, N->stream));
    for (int s = 0; s < steps; ++s) MLP_CK(cudaGraphLaunch(N->exec, N->stream));
    MLP_CK(cudaEventRecord(e1, N->stream));
    MLP_CK(cudaEventSynchronize(e1));
    MLP_CK(cudaEventElapsedTime(&N->last_ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    check_error(*N);
    if (loss_history && steps > 0)
      MLP_CK(cudaMemcpy(loss_history, N->loss_hist + t0, sizeof(float) * steps, cudaMemcpyDeviceToHost));
    return 0;
  } catch (const std::exception& e) {
    return fail(OPENMC_E_UNASSIGNED, e.what());
  }
}

// One forward and backward pass over the staged rows without an update:
// grad (host, n_params floats) receives dLoss/dparams, loss the loss.
int openmc_gb300_mlp_gradients(void* handle, float* grad, float* loss)
{
  using namespace mlp;
  Net* N = static_cast<Net*>(handle);
  if (!N || N->R == 0 || !grad) return fail(OPENMC_E_INVALID_ARGUMENT, "no training data staged");
  try {
    int t0 = 0;
    MLP_CK(cudaMemcpyAsync(&t0, N->step, sizeof(int), cudaMemcpyDeviceToHost, N->stream));
    MLP_CK(cudaStreamSynchronize(N->stream));
    enqueue_pass(*N, true, nullptr);
    AdamArgs a = adam_args(*N, 0, 0.0f);
    a.grad_out = N->grad;
    enqueue_adam(*N, a);
    check_error(*N);
    MLP_CK(cudaMemcpy(grad, N->grad, sizeof(float) * N_PARAMS, cudaMemcpyDeviceToHost));
    if (loss) {
      const long long blocks = N->fused_grid > 0 ? N->fused_grid : N->R / TILE_M;
      std::vector<float> gh(static_cast<size_t>(blocks) * 130);
      MLP_CK(cudaMemcpy(gh.data(), N->GH, sizeof(float) * gh.size(), cudaMemcpyDeviceToHost));
      float s = 0.0f;
      for (size_t b = 0; b < gh.size() / 130; ++b) s += gh[b * 130 + 129];
      *loss = s;
    }
    // a gradient evaluation is not an optimizer step
    MLP_CK(cudaMemcpyAsync(N->step, &t0, sizeof(int), cudaMemcpyHostToDevice, N->stream));
    MLP_CK(cudaStreamSynchronize(N->stream));
    return 0;
  } catch (const std::exception& e) {
    return fail(OPENMC_E_UNASSIGNED, e.what());
  }
}

// Network output for n query rows (host x4 [n][4] -> host y [n]), in
// chunks of the network's row capacity.  Replaces the staged training rows.
int openmc_gb300_mlp_predict(void* handle, int64_t n, const float* x4, float* y)
{
  using namespace mlp;
  Net* N = static_cast<Net*>(handle);
  if (!N || n < 0 || (n > 0 && (!x4 || !y))) return fail(OPENMC_E_INVALID_ARGUMENT, "invalid query");
  try {
    drop_graph(*N);
    for (long long off = 0; off < n; off += N->cap) {
      const long long c = std::min<long long>(N->cap, n - off);
      const long long R = (c + TILE_M - 1) / TILE_M * TILE_M;
      N->n = c;
      N->R = R;
      MLP_CK(cudaMemcpyAsync(N->x4, x4 + off * 4, sizeof(float) * 4 * c, cudaMemcpyHostToDevice, N->stream));
      N->prepared = false;
      enqueue_pass(*N, false, N->y);
      check_error(*N);
      MLP_CK(cudaMemcpy(y + off, N->y, sizeof(float) * c, cudaMemcpyDeviceToHost));
    }
    N->n = 0;
    N->R = 0;
    N->prepared = false;
    return 0;
  } catch (const std::exception& e) {
    return fail(OPENMC_E_UNASSIGNED, e.what());
  }
}

int openmc_gb300_mlp_get_params(void* handle, float* params, int64_t n)
{
  using namespace mlp;
  Net* N = static_cast<Net*>(handle);
  if (!N || !params || n != N_PARAMS) return fail(OPENMC_E_INVALID_ARGUMENT, "parameter count mismatch");
  try {
    MLP_CK(cudaStreamSynchronize(N->stream));
    MLP_CK(cudaMemcpy(params, N->P, sizeof(float) * N_PARAMS, cudaMemcpyDeviceToHost));
    return 0;
  } catch (const std::exception& e) {
    return fail(OPENMC_E_UNASSIGNED, e.what());
  }
}

// Replaces the parameters and resets the optimizer state.
int openmc_gb300_mlp_set_params(void* handle, const float* params, int64_t n)
{
  using namespace mlp;
  Net* N = static_cast<Net*>(handle);
  if (!N || !params || n != N_PARAMS) return fail(OPENMC_E_INVALID_ARGUMENT, "parameter count mismatch");
  try {
    upload_params(*N, params);
    return 0;
  } catch (const std::exception& e) {
    return fail(OPENMC_E_UNASSIGNED, e.what());
  }
}

// Device milliseconds of the last openmc_gb300_mlp_train call.
int openmc_gb300_mlp_last_ms(void* handle, float* ms)
{
  mlp::Net* N = static_cast<mlp::Net*>(handle);
  if (!N || !ms) return fail(OPENMC_E_INVALID_ARGUMENT, "invalid handle");
  *ms = N->last_ms;
  return 0;
}

}  // extern "C"
