// Tensor-core (tcgen05) versions of the pointwise channel-MLP chains, in split-BF16: every GEMM operand x is carried as
// hi = bf16(x) and lo = bf16(x - hi), and each product as hi*hi + hi*lo + lo*hi on the BF16 tensor cores with FP32
// accumulation in tensor memory (relative error about 2^-16; a single BF16 product, 2^-8, moves log10 n by 1e-2).
// Activations, residuals and GroupNorm statistics stay FP32 in HBM, so every kernel has the contract of an FP32 entry
// point of pointwise_f32.cu / backward_f32.cu (or of a stage of one).
//
// CTA = 256 threads = two warpgroups over one tile of 128 voxels: thread t serves voxel row t % 128 (tensor-memory lane
// t % 128), warpgroup t / 128 the even or odd 16-column chunks of every accumulator. The split weights
// (packed on the host in the canonical K-major order) are bulk-copied (TMA) into shared memory once per persistent
// CTA. Each GEMM is issued by thread 0 and completes on an mbarrier; every wait is bounded: a timeout sets *err, all
// threads leave the tile loop together, and the CTA frees its tensor memory after one more bounded wait.
#include <math.h>

#include "common.cuh"
#include "tc.cuh"

using namespace ffno;

namespace {

constexpr int TM = 128;  // voxels per tile = MMA M
constexpr int TT = 256;  // threads per CTA (two warpgroups)
constexpr int FB = 8;    // fill: independent loads in flight per thread

__host__ __device__ constexpr uint32_t tmem_cols(int n) {
  return n <= 32 ? 32 : n <= 64 ? 64 : n <= 128 ? 128 : n <= 256 ? 256 : 512;
}

// bytes of one split matrix (hi + lo) of R x K
__host__ __device__ constexpr uint32_t mat_bytes(int R, int K) { return (uint32_t)R * K * 2 * 2; }
// bytes of one split activation tile of 128 x K
__host__ __device__ constexpr uint32_t tile_bytes(int K) { return (uint32_t)TM * K * 2 * 2; }

struct Ctx {
  uint64_t* bar;
  uint32_t phase;
  bool ok;
};

// A split matrix or tile in shared memory: hi half then lo half.
struct Split {
  uint8_t* p;
  uint32_t half;  // bytes of one half
  __device__ uint8_t* hi() const { return p; }
  __device__ uint8_t* lo() const { return p + half; }
};

__device__ __forceinline__ Split split_at(uint8_t* p, int R, int K) { return Split{p, (uint32_t)R * K * 2}; }

__device__ __forceinline__ bool load_weights(void* dst, const void* src, uint32_t bytes, Ctx& cx, int* err) {
  if (threadIdx.x == 0) {
    tc::mbar_arrive_expect_tx(cx.bar, bytes);
    uint32_t off = 0;
    while (off < bytes) {
      const uint32_t n = (bytes - off) < 65536u ? (bytes - off) : 65536u;
      tc::bulk_g2s(static_cast<uint8_t*>(dst) + off, static_cast<const uint8_t*>(src) + off, n, cx.bar);
      off += n;
    }
  }
  const bool ok = __syncthreads_and(tc::mbar_wait(cx.bar, cx.phase)) != 0;
  cx.phase ^= 1u;
  if (!ok && threadIdx.x == 0) atomicExch(err, 1);
  return ok;
}

// Issue up to two split GEMMs D_i = A_i B_i^T (thread 0) behind one commit and wait for them (all threads).
__device__ __forceinline__ bool gemms(Ctx& cx, int* err, uint32_t d0, Split a0, Split b0, int k0, int n0,
                                      uint32_t d1 = 0, Split a1 = Split{nullptr, 0}, Split b1 = Split{nullptr, 0},
                                      int k1 = 0, int n1 = 0) {
  tc::fence_async_smem();
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  if (threadIdx.x == 0) {
    tc::gemm3_128xN(d0, tc::smem_u32(a0.hi()), tc::smem_u32(a0.lo()), tc::smem_u32(b0.hi()), tc::smem_u32(b0.lo()),
                    k0, n0);
    if (a1.p)
      tc::gemm3_128xN(d1, tc::smem_u32(a1.hi()), tc::smem_u32(a1.lo()), tc::smem_u32(b1.hi()), tc::smem_u32(b1.lo()),
                      k1, n1);
    tc::mma_commit(cx.bar);
  }
  const bool ok = __syncthreads_and(tc::mbar_wait(cx.bar, cx.phase)) != 0;
  cx.phase ^= 1u;
  tc::tc_after_sync();
  if (!ok && threadIdx.x == 0) atomicExch(err, 2);
  cx.ok = ok;
  return ok;
}

__device__ __forceinline__ void finish(Ctx& cx, uint32_t tmem, uint32_t ncol) {
  if (!cx.ok) tc::mbar_wait(cx.bar, cx.phase ^ 1u);
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  if (threadIdx.x < 32) tc::tmem_free(tmem, ncol);
}

// Fill a split tile [128][KW] from FP32 sources: f(v, k) returns columns k..k+3 of voxel v (v < V); rows past the
// cube are zero. Consecutive threads fill consecutive 8-byte pieces of the canonical layout.
template <int KW, typename F>
__device__ __forceinline__ void fill_tile(Split t, long v0, long V, F f) {
  constexpr int NE = TM * KW / 4;
  for (int e0 = threadIdx.x; e0 < NE; e0 += TT * FB) {
    float4 a[FB];
#pragma unroll
    for (int u = 0; u < FB; ++u) {  // issue the loads of FB pieces before converting any of them
      const int e = e0 + u * TT;
      const int h = e & 1, r8 = (e >> 1) & 7, q = e >> 4;
      const int kb = q % (KW / 8), rb = q / (KW / 8);
      const long v = v0 + rb * 8 + r8;
      a[u] = (e < NE && v < V) ? f(v, kb * 8 + h * 4) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < FB; ++u) {
      const int e = e0 + u * TT;
      if (e >= NE) break;
      uint32_t h0, l0, h1, l1;
      tc::split_pack(a[u].x, a[u].y, h0, l0);
      tc::split_pack(a[u].z, a[u].w, h1, l1);
      *reinterpret_cast<uint2*>(t.hi() + (size_t)e * 8) = make_uint2(h0, h1);
      *reinterpret_cast<uint2*>(t.lo() + (size_t)e * 8) = make_uint2(l0, l1);
    }
  }
}

// Write 16 values of this thread's row into a split tile with K columns at columns c0..c0+15.
__device__ __forceinline__ void put16(Split t, int r, int c0, int K, const float (&v)[16]) {
  uint32_t h[8], l[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) tc::split_pack(v[2 * i], v[2 * i + 1], h[i], l[i]);
  const uint32_t o0 = tc::kmajor_offset(r, c0, K), o1 = tc::kmajor_offset(r, c0 + 8, K);
  *reinterpret_cast<uint4*>(t.hi() + o0) = make_uint4(h[0], h[1], h[2], h[3]);
  *reinterpret_cast<uint4*>(t.hi() + o1) = make_uint4(h[4], h[5], h[6], h[7]);
  *reinterpret_cast<uint4*>(t.lo() + o0) = make_uint4(l[0], l[1], l[2], l[3]);
  *reinterpret_cast<uint4*>(t.lo() + o1) = make_uint4(l[4], l[5], l[6], l[7]);
}

__device__ __forceinline__ uint32_t lane_base() { return (uint32_t)(32 * ((threadIdx.x >> 5) & 3)) << 16; }
__device__ __forceinline__ int row_of() { return threadIdx.x & (TM - 1); }
__device__ __forceinline__ int wg_of() { return threadIdx.x >> 7; }

// L2 prefetch of rows [n0, n0 + 128) of a [V][width] FP32 array, by one thread
__device__ __forceinline__ void prefetch_rows(const float* base, long n0, long V, int width) {
  if (!base || n0 >= V) return;
  const long rows = (V - n0) < TM ? (V - n0) : TM;
  tc::prefetch_l2(base + n0 * width, (uint32_t)(rows * width * 4));
}

__device__ __forceinline__ float4 ld4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

// GroupNorm apply (+ GELU) of 4 consecutive channels k..k+3 with coefs [3][C]
template <bool GELU>
__device__ __forceinline__ float4 gn4(float4 p, const float* __restrict__ cf, int C, int k) {
  float4 y;
  y.x = (p.x - __ldg(cf + k)) * __ldg(cf + C + k) + __ldg(cf + 2 * C + k);
  y.y = (p.y - __ldg(cf + k + 1)) * __ldg(cf + C + k + 1) + __ldg(cf + 2 * C + k + 1);
  y.z = (p.z - __ldg(cf + k + 2)) * __ldg(cf + C + k + 2) + __ldg(cf + 2 * C + k + 2);
  y.w = (p.w - __ldg(cf + k + 3)) * __ldg(cf + C + k + 3) + __ldg(cf + 2 * C + k + 3);
  if (GELU) {
    y.x = gelu(y.x);
    y.y = gelu(y.y);
    y.z = gelu(y.z);
    y.w = gelu(y.w);
  }
  return y;
}

__device__ __forceinline__ float gn1gelu(float p, const float* __restrict__ cf, int C, int k) {
  return gelu((p - __ldg(cf + k)) * __ldg(cf + C + k) + __ldg(cf + 2 * C + k));
}

// Per-tile depth-weighted group statistics of the tile's values, merged with Chan's update into acc (threads
// g < GMAX). Each thread holds, in v[C], the columns of the 16-column chunks of its warpgroup (chunk j belongs to
// warpgroup j % 2; a group never straddles two chunks); w is its row's weight (0 past the cube). Fixed reduction order.
template <int C>
__device__ __forceinline__ void row_group_stats(const float (&v)[C], float w, float* red, float* gm, float* wsum,
                                                GroupAcc& acc) {
  constexpr int CPG = C / GMAX;
  constexpr int NW = TT / 32;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, wg = wg_of();
  float ws = wg == 0 ? w : 0.f;
#pragma unroll
  for (int o = 16; o; o >>= 1) ws += __shfl_xor_sync(0xffffffffu, ws, o);
  float s[GMAX];
#pragma unroll
  for (int g = 0; g < GMAX; ++g) s[g] = 0.f;
#pragma unroll
  for (int c = 0; c < C; ++c)
    if (((c >> 4) & 1) == wg) s[c / CPG] += v[c];
#pragma unroll
  for (int g = 0; g < GMAX; ++g) {
    float x = w * s[g];
#pragma unroll
    for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    s[g] = x;
  }
  if (lane == 0) {
    red[warp * (GMAX + 1) + GMAX] = ws;
#pragma unroll
    for (int g = 0; g < GMAX; ++g) red[warp * (GMAX + 1) + g] = s[g];
  }
  __syncthreads();
  if (tid == 0) {
    float t = 0.f;
    for (int q = 0; q < NW; ++q) t += red[q * (GMAX + 1) + GMAX];
    *wsum = t;
  }
  if (tid < GMAX) {
    float t = 0.f, wt = 0.f;
    for (int q = 0; q < NW; ++q) {
      t += red[q * (GMAX + 1) + tid];
      wt += red[q * (GMAX + 1) + GMAX];
    }
    wt *= CPG;
    gm[tid] = wt > 0.f ? t / wt : 0.f;
  }
  __syncthreads();
#pragma unroll
  for (int g = 0; g < GMAX; ++g) s[g] = 0.f;
#pragma unroll
  for (int c = 0; c < C; ++c)
    if (((c >> 4) & 1) == wg) {
      const float d = v[c] - gm[c / CPG];
      s[c / CPG] += d * d;
    }
#pragma unroll
  for (int g = 0; g < GMAX; ++g) {
    float x = w * s[g];
#pragma unroll
    for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    s[g] = x;
  }
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int g = 0; g < GMAX; ++g) red[warp * (GMAX + 1) + g] = s[g];
  __syncthreads();
  if (tid < GMAX) {
    float t = 0.f;
    for (int q = 0; q < NW; ++q) t += red[q * (GMAX + 1) + tid];
    chan_merge(acc, (double)*wsum * CPG, (double)gm[tid], (double)t);
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------------------------------- ping-pong
// Two warpgroups of a CTA run independent tile pipelines over alternate tiles (warpgroup w takes tiles
// 2 * blockIdx.x + w, then every 2 * gridDim.x): each has its own operand tiles in shared memory, its own tensor-memory
// columns and MMA mbarrier, and synchronises with a named barrier of its 128 threads, so one warpgroup's loads and
// epilogue overlap the other's MMAs and waits. Thread t of a warpgroup serves voxel row t (tensor-memory lane t) and
// every column of it. The split weights are shared.
constexpr int WGT = 256;              // threads per pipeline
constexpr int SPL = WGT / TM;         // threads per voxel row (each takes every SPL-th 16-column chunk)
constexpr int CT = 2 * WGT;           // threads per CTA (two pipelines)

__device__ __forceinline__ void wg_sync(int wg) { asm volatile("bar.sync %0, %1;" ::"r"(1 + wg), "n"(WGT) : "memory"); }

// whether this thread's part of the row owns 16-column chunk jj
__device__ __forceinline__ bool owns(int jj, int half) { return SPL == 1 || (jj % SPL) == half; }

// Named-barrier AND over the warpgroup's predicates.
__device__ __forceinline__ bool wg_sync_and(int wg, bool p) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred pi, po;\n setp.ne.u32 pi, %1, 0;\n bar.red.and.pred po, %2, %3, pi;\n selp.u32 %0, 1, 0, po;\n}"
      : "=r"(r)
      : "r"((uint32_t)p), "r"(1 + wg), "n"(WGT)
      : "memory");
  return r != 0;
}

struct WCtx {
  uint64_t* bar;  // this warpgroup's MMA barrier
  uint32_t phase;
  bool ok;
  int wg, wtid;
};

// A split operand in shared memory for the MMA: hi and lo shared-space addresses and the row-group stride.
struct Op {
  uint32_t hi, lo, sbo;
};
__device__ __forceinline__ Op op_of(Split s, int K) {
  return Op{tc::smem_u32(s.hi()), tc::smem_u32(s.lo()), (uint32_t)K * 16u};
}
// Columns k0.. of a split operand with Ktot columns (a K-slice; k0 a multiple of 8).
__device__ __forceinline__ Op op_kslice(Split s, int Ktot, int k0) {
  const uint32_t o = (uint32_t)(k0 / 8) * 128u;
  return Op{tc::smem_u32(s.hi()) + o, tc::smem_u32(s.lo()) + o, (uint32_t)Ktot * 16u};
}

// D [128 x N] (+)= A B^T over K columns, split-BF16 (Ah Bh + Ah Bl + Al Bh); accumulates onto D when acc.
__device__ __forceinline__ void gemm3_op(uint32_t tmem_d, Op a, Op b, int K, int N, bool acc) {
  const uint32_t idesc = tc::idesc_bf16(128, N);
  const uint32_t as[3] = {a.hi, a.hi, a.lo}, bs[3] = {b.hi, b.lo, b.hi};
#pragma unroll
  for (int s = 0; s < 3; ++s)
    for (int k = 0; k < K; k += 16) {
      const uint64_t ad = tc::kmajor_desc(as[s] + (uint32_t)(k / 8) * 128u, 128u, a.sbo);
      const uint64_t bd = tc::kmajor_desc(bs[s] + (uint32_t)(k / 8) * 128u, 128u, b.sbo);
      tc::mma_bf16(tmem_d, ad, bd, idesc, (acc || s > 0 || k > 0) ? 1u : 0u);
    }
}

// Issue up to two split GEMMs (the warpgroup's thread 0) behind one commit and wait for them (the warpgroup).
__device__ __forceinline__ bool wg_gemms(WCtx& cx, int* err, uint32_t d0, Op a0, Op b0, int k0, int n0,
                                         bool acc0 = false, uint32_t d1 = 0, Op a1 = Op{0, 0, 0},
                                         Op b1 = Op{0, 0, 0}, int k1 = 0, int n1 = 0) {
  tc::fence_async_smem();
  tc::tc_before_sync();
  wg_sync(cx.wg);
  tc::tc_after_sync();
  if (cx.wtid == 0) {
    gemm3_op(d0, a0, b0, k0, n0, acc0);
    if (k1) gemm3_op(d1, a1, b1, k1, n1, false);
    tc::mma_commit(cx.bar);
  }
  const bool ok = wg_sync_and(cx.wg, tc::mbar_wait(cx.bar, cx.phase));
  cx.phase ^= 1u;
  tc::tc_after_sync();
  if (!ok && cx.wtid == 0) atomicExch(err, 2);
  cx.ok = ok;
  return ok;
}

// fill_tile for one warpgroup (wtid = thread within it)
template <int KW, typename F>
__device__ __forceinline__ void wg_fill_tile(Split t, long v0, long V, int wtid, F f) {
  constexpr int NE = TM * KW / 4;
  for (int e0 = wtid; e0 < NE; e0 += WGT * FB) {
    float4 a[FB];
#pragma unroll
    for (int u = 0; u < FB; ++u) {  // issue the loads of FB pieces before converting any of them
      const int e = e0 + u * WGT;
      const int h = e & 1, r8 = (e >> 1) & 7, q = e >> 4;
      const int kb = q % (KW / 8), rb = q / (KW / 8);
      const long v = v0 + rb * 8 + r8;
      a[u] = (e < NE && v < V) ? f(v, kb * 8 + h * 4) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < FB; ++u) {
      const int e = e0 + u * WGT;
      if (e >= NE) break;
      uint32_t h0, l0, h1, l1;
      tc::split_pack(a[u].x, a[u].y, h0, l0);
      tc::split_pack(a[u].z, a[u].w, h1, l1);
      *reinterpret_cast<uint2*>(t.hi() + (size_t)e * 8) = make_uint2(h0, h1);
      *reinterpret_cast<uint2*>(t.lo() + (size_t)e * 8) = make_uint2(l0, l1);
    }
  }
}

// Per-tile depth-weighted group statistics of one warpgroup's tile (every thread holds all C values of its row in
// v, weight w; 0 past the cube), merged with Chan's update into acc (threads wtid < GMAX). Fixed reduction order.
// red: [4][GMAX + 1] of this warpgroup.
template <int C>
__device__ __forceinline__ void wg_row_group_stats(const float (&v)[C], float w, float* red, float* gm, float* wsum,
                                                   GroupAcc& acc, int wg, int wtid) {
  constexpr int CPG = C / GMAX;
  const int lane = wtid & 31, wl = wtid >> 5, half = wtid / TM;
  float ws = half == 0 ? w : 0.f;
#pragma unroll
  for (int o = 16; o; o >>= 1) ws += __shfl_xor_sync(0xffffffffu, ws, o);
  float s[GMAX];
#pragma unroll
  for (int g = 0; g < GMAX; ++g) s[g] = 0.f;
#pragma unroll
  for (int c = 0; c < C; ++c)
    if (owns(c / 16, half)) s[c / CPG] += v[c];
#pragma unroll
  for (int g = 0; g < GMAX; ++g) {
    float x = w * s[g];
#pragma unroll
    for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    s[g] = x;
  }
  if (lane == 0) {
    red[wl * (GMAX + 1) + GMAX] = ws;
#pragma unroll
    for (int g = 0; g < GMAX; ++g) red[wl * (GMAX + 1) + g] = s[g];
  }
  wg_sync(wg);
  if (wtid == 0) {
    float t = 0.f;
    for (int q = 0; q < WGT / 32; ++q) t += red[q * (GMAX + 1) + GMAX];
    *wsum = t;
  }
  if (wtid < GMAX) {
    float t = 0.f, wt = 0.f;
    for (int q = 0; q < WGT / 32; ++q) {
      t += red[q * (GMAX + 1) + wtid];
      wt += red[q * (GMAX + 1) + GMAX];
    }
    wt *= CPG;
    gm[wtid] = wt > 0.f ? t / wt : 0.f;
  }
  wg_sync(wg);
#pragma unroll
  for (int g = 0; g < GMAX; ++g) s[g] = 0.f;
#pragma unroll
  for (int c = 0; c < C; ++c)
    if (owns(c / 16, half)) {
      const float d = v[c] - gm[c / CPG];
      s[c / CPG] += d * d;
    }
#pragma unroll
  for (int g = 0; g < GMAX; ++g) {
    float x = w * s[g];
#pragma unroll
    for (int o = 16; o; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    s[g] = x;
  }
  if (lane == 0)
#pragma unroll
    for (int g = 0; g < GMAX; ++g) red[wl * (GMAX + 1) + g] = s[g];
  wg_sync(wg);
  if (wtid < GMAX) {
    float t = 0.f;
    for (int q = 0; q < WGT / 32; ++q) t += red[q * (GMAX + 1) + wtid];
    chan_merge(acc, (double)*wsum * CPG, (double)gm[wtid], (double)t);
  }
  wg_sync(wg);
}

// The CTA's GroupNorm partial: warpgroup 1's statistics merged into warpgroup 0's (fixed order). All threads call it.
__device__ __forceinline__ void wg_write_partial(double* partials, GroupAcc acc, double* xs, int wg, int wtid) {
  if (wg == 1 && wtid < GMAX) {
    xs[3 * wtid] = acc.w;
    xs[3 * wtid + 1] = acc.mean;
    xs[3 * wtid + 2] = acc.m2;
  }
  __syncthreads();
  if (wg == 0 && wtid < GMAX) {
    chan_merge(acc, xs[3 * wtid], xs[3 * wtid + 1], xs[3 * wtid + 2]);
    double* p = partials + ((long)blockIdx.x * GMAX + wtid) * 3;
    p[0] = acc.w;
    p[1] = acc.mean;
    p[2] = acc.m2;
  }
}

// After both warpgroups left their loops: wait once more (bounded) for an MMA of a failed wait, free tensor memory.
__device__ __forceinline__ void wg_finish(const WCtx& cx, uint32_t tmem_all, uint32_t ncol_all) {
  if (!cx.ok) tc::mbar_wait(cx.bar, cx.phase ^ 1u);
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  if (threadIdx.x < 32) tc::tmem_free(tmem_all, ncol_all);
}

#define TC_PROLOGUE_WG(NCOLS)                                                            \
  __shared__ uint64_t bars[3];                                                           \
  __shared__ uint32_t tslot;                                                             \
  const int tid = threadIdx.x, wg = tid / WGT, wtid = tid % WGT, half = wtid / TM;      \
  constexpr uint32_t NCOL = tmem_cols(NCOLS);                                            \
  static_assert(2 * NCOL <= 512, "two warpgroups' accumulators exceed tensor memory");   \
  if (tid < 32) tc::tmem_alloc(&tslot, 2 * NCOL);                                        \
  if (tid == 0) {                                                                        \
    tc::mbar_init(&bars[0], 1);                                                          \
    tc::mbar_init(&bars[1], 1);                                                          \
    tc::mbar_init(&bars[2], 1);                                                          \
    tc::mbar_init_fence();                                                               \
  }                                                                                      \
  tc::tc_before_sync();                                                                  \
  __syncthreads();                                                                       \
  tc::tc_after_sync();                                                                   \
  const uint32_t tmem_all = tslot, tmem = tslot + (uint32_t)wg * NCOL;                   \
  Ctx wcx{&bars[0], 0u, true};                                                           \
  WCtx cx{&bars[1 + wg], 0u, true, wg, wtid};                                            \
  const uint32_t lb = lane_base();                                                       \
  const int row = wtid % TM;                                                             \
  const long nt = (V + TM - 1) / TM;                                                     \
  const long tstep = 2L * gridDim.x;                                                     \
  (void)row;                                                                             \
  (void)half;

#define TC_PROLOGUE(NCOLS)                    \
  __shared__ uint64_t bar;                    \
  __shared__ uint32_t tslot;                  \
  const int tid = threadIdx.x;                \
  constexpr uint32_t NCOL = tmem_cols(NCOLS); \
  if (tid < 32) tc::tmem_alloc(&tslot, NCOL); \
  if (tid == 0) {                             \
    tc::mbar_init(&bar, 1);                   \
    tc::mbar_init_fence();                    \
  }                                           \
  tc::tc_before_sync();                       \
  __syncthreads();                            \
  tc::tc_after_sync();                        \
  const uint32_t tmem = tslot;                \
  Ctx cx{&bar, 0u, true};                     \
  const uint32_t lb = lane_base();            \
  const int row = row_of(), wg = wg_of();     \
  (void)row;                                  \
  (void)wg;                                   \
  const long nt = (V + TM - 1) / TM;

// ============================================================================================== forward
// 2-layer MLP C -> 2C -> C with the residual prologue of ffno_mlp2_fwd and GroupNorm partials of the output.
// Weights: [w1 (2C x C), w2 (C x 2C)]. Per warpgroup: the input tile, then (aliased) the hidden tile.
template <int C, int MODE>
__global__ void __launch_bounds__(CT, 1) k_mlp2_tc(const float* __restrict__ in, const float* __restrict__ prev,
                                                const float* __restrict__ pc, float res, float* __restrict__ xout,
                                                long V, const uint8_t* __restrict__ wpack,
                                                const float* __restrict__ dw, float* __restrict__ pre,
                                                double* __restrict__ partials, int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(2 * C, C), B2 = mat_bytes(C, 2 * C), RB = tile_bytes(2 * C);
  Split w1 = split_at(smem, 2 * C, C), w2 = split_at(smem + B1, C, 2 * C);
  __shared__ float red[2][(WGT / 32) * (GMAX + 1)], gmean[2][GMAX], wsum[2];
  __shared__ double xs[3 * GMAX];
  TC_PROLOGUE_WG(2 * C)
  uint8_t* region = smem + B1 + B2 + wg * RB;
  Split A = split_at(region, TM, C), H = split_at(region, TM, 2 * C);
  GroupAcc acc{0.0, 0.0, 0.0};
  cx.ok = load_weights(smem, wpack, B1 + B2, wcx, err);
  for (long t = 2L * blockIdx.x + wg; cx.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (wtid == 0) {
      prefetch_rows(in, (t + tstep) * TM, V, C);
      if (MODE != 0) prefetch_rows(prev, (t + tstep) * TM, V, C);
    }
    wg_fill_tile<C>(A, v0, V, wtid, [&](long v, int k) {
      float4 a = ld4(in + v * C + k);
      if (MODE != 0) {
        const float4 y = gn4<MODE == 1>(ld4(prev + v * C + k), pc, C, k);
        a.x += res * y.x;
        a.y += res * y.y;
        a.z += res * y.z;
        a.w += res * y.w;
        *reinterpret_cast<float4*>(xout + v * C + k) = a;
      }
      return a;
    });
    if (!wg_gemms(cx, err, tmem, op_of(A, C), op_of(w1, C), C, 2 * C)) break;
#pragma unroll
    for (int jj = 0; jj < (2 * C) / 16; ++jj) {
      if (!owns(jj, half)) continue;
      const int c0 = 16 * jj;
      float v[16];
      tc::tmem_ld16(tmem + lb + c0, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = gelu(v[i]);
      put16(H, row, c0, 2 * C, v);
    }
    if (!wg_gemms(cx, err, tmem, op_of(H, 2 * C), op_of(w2, 2 * C), 2 * C, C)) break;
    float o[C];
#pragma unroll
    for (int jj = 0; jj < C / 16; ++jj) {
      if (!owns(jj, half)) continue;
      float v[16];
      tc::tmem_ld16(tmem + lb + 16 * jj, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) o[16 * jj + i] = v[i];
    }
    const long v = v0 + row;
    float w = 0.f;
    if (v < V) {
      w = __ldg(dw + v);
      float4* dst = reinterpret_cast<float4*>(pre + v * C);
#pragma unroll
      for (int c = 0; c < C; c += 4)
        if (owns(c / 16, half)) dst[c / 4] = make_float4(o[c], o[c + 1], o[c + 2], o[c + 3]);
    }
    wg_row_group_stats<C>(o, w, red[wg], gmean[wg], &wsum[wg], acc, wg, wtid);
  }
  wg_write_partial(partials, acc, xs, wg, wtid);
  wg_finish(cx, tmem_all, 2 * NCOL);
}

// Input gate of one branch: out = x sigmoid(gelu(x G1) G2) [+ zp z]. Weights: [g1 (C x C), g2 (C x C)].
template <int C>
__global__ void __launch_bounds__(CT, 1) k_gate_tc(const float* __restrict__ x, long V, const uint8_t* __restrict__ wpack,
                                                const float* __restrict__ zp, const float* __restrict__ z,
                                                float* __restrict__ out, int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(C, C), RB = tile_bytes(C);
  Split g1 = split_at(smem, C, C), g2 = split_at(smem + B1, C, C);
  TC_PROLOGUE_WG(C)
  Split A = split_at(smem + 2 * B1 + wg * RB, TM, C);
  cx.ok = load_weights(smem, wpack, 2 * B1, wcx, err);
  for (long t = 2L * blockIdx.x + wg; cx.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (wtid == 0) prefetch_rows(x, (t + tstep) * TM, V, C);
    wg_fill_tile<C>(A, v0, V, wtid, [&](long v, int k) { return ld4(x + v * C + k); });
    if (!wg_gemms(cx, err, tmem, op_of(A, C), op_of(g1, C), C, C)) break;
#pragma unroll
    for (int jj = 0; jj < C / 16; ++jj) {
      if (!owns(jj, half)) continue;
      const int c0 = 16 * jj;
      float v[16];
      tc::tmem_ld16(tmem + lb + c0, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = gelu(v[i]);
      put16(A, row, c0, C, v);
    }
    if (!wg_gemms(cx, err, tmem, op_of(A, C), op_of(g2, C), C, C)) break;
    const long v = v0 + row;
    const float zv = (zp && v < V) ? __ldg(z + v) : 0.f;
#pragma unroll
    for (int jj = 0; jj < C / 16; ++jj) {
      if (!owns(jj, half)) continue;
      const int c0 = 16 * jj;
      float g[16];
      tc::tmem_ld16(tmem + lb + c0, g);
      if (v < V) {
#pragma unroll
        for (int i = 0; i < 16; i += 4) {
          const float4 xv = ld4(x + v * C + c0 + i);
          float4 o = make_float4(xv.x * sigmoid(g[i]), xv.y * sigmoid(g[i + 1]), xv.z * sigmoid(g[i + 2]),
                                 xv.w * sigmoid(g[i + 3]));
          if (zp) {
            o.x += __ldg(zp + c0 + i) * zv;
            o.y += __ldg(zp + c0 + i + 1) * zv;
            o.z += __ldg(zp + c0 + i + 2) * zv;
            o.w += __ldg(zp + c0 + i + 3) * zv;
          }
          *reinterpret_cast<float4*>(out + v * C + c0 + i) = o;
        }
      }
    }
  }
  wg_finish(cx, tmem_all, 2 * NCOL);
}

// Branch gates (first half of _fuse_branches): gates = sigmoid(gelu([x, spec, vert] Wg1) Wg2 + b), spec =
// gelu(GN(spec_pre)) etc.; optionally the hidden pre-activation [x, spec, vert] Wg1 to hg. Weights: [wg1 (C x 3C),
// wg2 (2C x C)]. The first GEMM runs over three K-slices of C columns (x, spec, vert) through one tile per warpgroup.
template <int C>
__global__ void __launch_bounds__(CT, 1) k_fuse1_tc(const float* __restrict__ x, const float* __restrict__ sp,
                                                 const float* __restrict__ sc, const float* __restrict__ vp,
                                                 const float* __restrict__ vc, long V,
                                                 const uint8_t* __restrict__ wpack, const float* __restrict__ bias,
                                                 float* __restrict__ gates, float* __restrict__ hg,
                                                 int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(C, 3 * C), B2 = mat_bytes(2 * C, C), RB = tile_bytes(C);
  Split wg1 = split_at(smem, C, 3 * C), wg2 = split_at(smem + B1, 2 * C, C);
  TC_PROLOGUE_WG(2 * C)
  Split A = split_at(smem + B1 + B2 + wg * RB, TM, C);
  cx.ok = load_weights(smem, wpack, B1 + B2, wcx, err);
  for (long t = 2L * blockIdx.x + wg; cx.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (wtid == 0) {
      prefetch_rows(x, (t + tstep) * TM, V, C);
      prefetch_rows(sp, (t + tstep) * TM, V, C);
      prefetch_rows(vp, (t + tstep) * TM, V, C);
    }
    for (int kc = 0; kc < 3; ++kc) {
      wg_fill_tile<C>(A, v0, V, wtid, [&](long v, int k) {
        if (kc == 0) return ld4(x + v * C + k);
        if (kc == 1) return gn4<true>(ld4(sp + v * C + k), sc, C, k);
        return gn4<true>(ld4(vp + v * C + k), vc, C, k);
      });
      if (!wg_gemms(cx, err, tmem, op_of(A, C), op_kslice(wg1, 3 * C, kc * C), C, C, kc > 0)) break;
    }
    if (!cx.ok) break;
    const long v = v0 + row;
#pragma unroll
    for (int jj = 0; jj < C / 16; ++jj) {
      if (!owns(jj, half)) continue;
      const int c0 = 16 * jj;
      float h[16];
      tc::tmem_ld16(tmem + lb + c0, h);
      if (hg && v < V)
#pragma unroll
        for (int i = 0; i < 16; i += 4)
          *reinterpret_cast<float4*>(hg + v * C + c0 + i) = make_float4(h[i], h[i + 1], h[i + 2], h[i + 3]);
#pragma unroll
      for (int i = 0; i < 16; ++i) h[i] = gelu(h[i]);
      put16(A, row, c0, C, h);
    }
    if (!wg_gemms(cx, err, tmem, op_of(A, C), op_of(wg2, C), C, 2 * C)) break;
#pragma unroll
    for (int jj = 0; jj < (2 * C) / 16; ++jj) {
      if (!owns(jj, half)) continue;
      const int c0 = 16 * jj;
      float g[16];
      tc::tmem_ld16(tmem + lb + c0, g);
      if (v < V)
#pragma unroll
        for (int i = 0; i < 16; i += 4)
          *reinterpret_cast<float4*>(gates + v * 2 * C + c0 + i) =
              make_float4(sigmoid(g[i] + __ldg(bias + c0 + i)), sigmoid(g[i + 1] + __ldg(bias + c0 + i + 1)),
                          sigmoid(g[i + 2] + __ldg(bias + c0 + i + 2)), sigmoid(g[i + 3] + __ldg(bias + c0 + i + 3)));
    }
  }
  wg_finish(cx, tmem_all, 2 * NCOL);
}

// Fuse (second half of _fuse_branches): B = [spec gs, vert gv], pre = gelu(B Wf1) Wf2 + (spec gs + vert gv) / 2, with
// the GroupNorm partials of pre. Weights: [wf1 (2C x 2C), wf2 (C x 2C)].
template <int C>
__global__ void __launch_bounds__(CT, 1) k_fuse2_tc(const float* __restrict__ sp, const float* __restrict__ sc,
                                                 const float* __restrict__ vp, const float* __restrict__ vc,
                                                 const float* __restrict__ gates, long V,
                                                 const uint8_t* __restrict__ wpack, const float* __restrict__ dw,
                                                 float* __restrict__ pre, double* __restrict__ partials,
                                                 int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(2 * C, 2 * C), B2 = mat_bytes(C, 2 * C), RB = tile_bytes(2 * C);
  Split wf1 = split_at(smem, 2 * C, 2 * C), wf2 = split_at(smem + B1, C, 2 * C);
  __shared__ float red[2][(WGT / 32) * (GMAX + 1)], gmean[2][GMAX], wsum[2];
  __shared__ double xs[3 * GMAX];
  TC_PROLOGUE_WG(2 * C)
  Split A = split_at(smem + B1 + B2 + wg * RB, TM, 2 * C);
  GroupAcc acc{0.0, 0.0, 0.0};
  cx.ok = load_weights(smem, wpack, B1 + B2, wcx, err);
  auto mixed = [&](long v, int k) {  // columns k..k+3 of B
    const float4 g = ld4(gates + v * 2 * C + k);
    const float4 s = (k < C) ? gn4<true>(ld4(sp + v * C + k), sc, C, k) : gn4<true>(ld4(vp + v * C + k - C), vc, C, k - C);
    return make_float4(s.x * g.x, s.y * g.y, s.z * g.z, s.w * g.w);
  };
  for (long t = 2L * blockIdx.x + wg; cx.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (wtid == 0) {
      prefetch_rows(sp, (t + tstep) * TM, V, C);
      prefetch_rows(vp, (t + tstep) * TM, V, C);
      prefetch_rows(gates, (t + tstep) * TM, V, 2 * C);
    }
    wg_fill_tile<2 * C>(A, v0, V, wtid, mixed);
    if (!wg_gemms(cx, err, tmem, op_of(A, 2 * C), op_of(wf1, 2 * C), 2 * C, 2 * C)) break;
#pragma unroll
    for (int jj = 0; jj < (2 * C) / 16; ++jj) {
      if (!owns(jj, half)) continue;
      const int c0 = 16 * jj;
      float h[16];
      tc::tmem_ld16(tmem + lb + c0, h);
#pragma unroll
      for (int i = 0; i < 16; ++i) h[i] = gelu(h[i]);
      put16(A, row, c0, 2 * C, h);
    }
    if (!wg_gemms(cx, err, tmem, op_of(A, 2 * C), op_of(wf2, 2 * C), 2 * C, C)) break;
    const long v = v0 + row;
    float o[C];
#pragma unroll
    for (int jj = 0; jj < C / 16; ++jj) {
      if (!owns(jj, half)) continue;
      float f[16];
      tc::tmem_ld16(tmem + lb + 16 * jj, f);
#pragma unroll
      for (int i = 0; i < 16; ++i) o[16 * jj + i] = f[i];
    }
    float w = 0.f;
    if (v < V) {
      w = __ldg(dw + v);
#pragma unroll
      for (int c = 0; c < C; c += 4) {
        if (!owns(c / 16, half)) continue;
        const float4 a = mixed(v, c), b = mixed(v, C + c);
        o[c] += 0.5f * (a.x + b.x);
        o[c + 1] += 0.5f * (a.y + b.y);
        o[c + 2] += 0.5f * (a.z + b.z);
        o[c + 3] += 0.5f * (a.w + b.w);
        *reinterpret_cast<float4*>(pre + v * C + c) = make_float4(o[c], o[c + 1], o[c + 2], o[c + 3]);
      }
    }
    wg_row_group_stats<C>(o, w, red[wg], gmean[wg], &wsum[wg], acc, wg, wtid);
  }
  wg_write_partial(partials, acc, xs, wg, wtid);
  wg_finish(cx, tmem_all, 2 * NCOL);
}

// ============================================================================================== backward
// a_bar = base + ((pre_bar W2^T) * gelu'(a W1)) W1^T. Weights: [w1 (2C x C), w2t (2C x C), w1t (C x 2C)].
// Per warpgroup: the tiles of a and pre_bar, then (aliased) the hidden tile.
template <int C>
__global__ void __launch_bounds__(CT, 1) k_mlp2_bwd_tc(const float* __restrict__ a, const float* __restrict__ pb,
                                                    const float* __restrict__ base, long V,
                                                    const uint8_t* __restrict__ wpack, float* __restrict__ abar,
                                                    int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(2 * C, C), RB = tile_bytes(2 * C);
  Split w1 = split_at(smem, 2 * C, C), w2t = split_at(smem + B1, 2 * C, C), w1t = split_at(smem + 2 * B1, C, 2 * C);
  TC_PROLOGUE_WG(4 * C)
  uint8_t* region = smem + 3 * B1 + wg * RB;
  Split A = split_at(region, TM, C), P = split_at(region + tile_bytes(C), TM, C), H = split_at(region, TM, 2 * C);
  cx.ok = load_weights(smem, wpack, 3 * B1, wcx, err);
  for (long t = 2L * blockIdx.x + wg; cx.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (wtid == 0) {
      prefetch_rows(a, (t + tstep) * TM, V, C);
      prefetch_rows(pb, (t + tstep) * TM, V, C);
      prefetch_rows(base, (t + tstep) * TM, V, C);
    }
    wg_fill_tile<C>(A, v0, V, wtid, [&](long v, int k) { return ld4(a + v * C + k); });
    wg_fill_tile<C>(P, v0, V, wtid, [&](long v, int k) { return ld4(pb + v * C + k); });
    if (!wg_gemms(cx, err, tmem, op_of(A, C), op_of(w1, C), C, 2 * C, false, tmem + 2 * C, op_of(P, C), op_of(w2t, C),
                  C, 2 * C))
      break;
#pragma unroll
    for (int jj = 0; jj < (2 * C) / 16; ++jj) {
      if (!owns(jj, half)) continue;
      const int c0 = 16 * jj;
      float hp[16], gb[16];
      tc::tmem_ld16(tmem + lb + c0, hp);
      tc::tmem_ld16(tmem + lb + 2 * C + c0, gb);
#pragma unroll
      for (int i = 0; i < 16; ++i) gb[i] *= gelu_grad(hp[i]);
      put16(H, row, c0, 2 * C, gb);
    }
    if (!wg_gemms(cx, err, tmem, op_of(H, 2 * C), op_of(w1t, 2 * C), 2 * C, C)) break;
    const long v = v0 + row;
#pragma unroll
    for (int jj = 0; jj < C / 16; ++jj) {
      if (!owns(jj, half)) continue;
      const int c0 = 16 * jj;
      float r[16];
      tc::tmem_ld16(tmem + lb + c0, r);
      if (v < V)
#pragma unroll
        for (int i = 0; i < 16; i += 4) {
          float4 o = make_float4(r[i], r[i + 1], r[i + 2], r[i + 3]);
          if (base) {
            const float4 b = ld4(base + v * C + c0 + i);
            o.x += b.x;
            o.y += b.y;
            o.z += b.z;
            o.w += b.w;
          }
          *reinterpret_cast<float4*>(abar + v * C + c0 + i) = o;
        }
    }
  }
  wg_finish(cx, tmem_all, 2 * NCOL);
}

// One input gate's backward: x_bar = base + d/dx [x sigmoid(gelu(x G1) G2)] applied to gbar; with zp, z_bar[v] +=
// sum_c gbar zp. Weights: [g1, g2, g2t, g1t] (each C x C).
template <int C>
__global__ void __launch_bounds__(CT, 1) k_gate_bwd_tc(const float* __restrict__ x, const float* __restrict__ gbar,
                                                    const float* __restrict__ base, long V,
                                                    const uint8_t* __restrict__ wpack, const float* __restrict__ zp,
                                                    float* __restrict__ xbar, float* __restrict__ zbar,
                                                    int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(C, C), RB = 2 * tile_bytes(C);
  Split g1 = split_at(smem, C, C), g2 = split_at(smem + B1, C, C), g2t = split_at(smem + 2 * B1, C, C),
        g1t = split_at(smem + 3 * B1, C, C);
  TC_PROLOGUE_WG(4 * C)
  Split X = split_at(smem + 4 * B1 + wg * RB, TM, C), T = split_at(smem + 4 * B1 + wg * RB + tile_bytes(C), TM, C);
  __shared__ float zsh[2][TM];
  const uint32_t D1 = tmem, D2 = tmem + C, D3 = tmem + 2 * C, D4 = tmem + 3 * C;
  cx.ok = load_weights(smem, wpack, 4 * B1, wcx, err);
  for (long t = 2L * blockIdx.x + wg; cx.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (wtid == 0) {
      prefetch_rows(x, (t + tstep) * TM, V, C);
      prefetch_rows(gbar, (t + tstep) * TM, V, C);
      prefetch_rows(base, (t + tstep) * TM, V, C);
    }
    const long v = v0 + row;
    wg_fill_tile<C>(X, v0, V, wtid, [&](long vv, int k) { return ld4(x + vv * C + k); });
    if (!wg_gemms(cx, err, D1, op_of(X, C), op_of(g1, C), C, C)) break;
#pragma unroll
    for (int jj = 0; jj < C / 16; ++jj) {
      if (!owns(jj, half)) continue;
      const int c0 = 16 * jj;
      float h[16];
      tc::tmem_ld16(D1 + lb + c0, h);
#pragma unroll
      for (int i = 0; i < 16; ++i) h[i] = gelu(h[i]);
      put16(T, row, c0, C, h);
    }
    if (!wg_gemms(cx, err, D2, op_of(T, C), op_of(g2, C), C, C)) break;
    float zs = 0.f;
#pragma unroll
    for (int jj = 0; jj < C / 16; ++jj) {
      if (!owns(jj, half)) continue;
      const int c0 = 16 * jj;
      float g[16], q[16];
      tc::tmem_ld16(D2 + lb + c0, g);
#pragma unroll
      for (int i = 0; i < 16; ++i) q[i] = 0.f;
      if (v < V) {
#pragma unroll
        for (int i = 0; i < 16; i += 4) {
          const float4 b = ld4(gbar + v * C + c0 + i), xv = ld4(x + v * C + c0 + i);
          const float bb[4] = {b.x, b.y, b.z, b.w}, xx[4] = {xv.x, xv.y, xv.z, xv.w};
          float o[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const float s = sigmoid(g[i + j]);
            o[j] = bb[j] * s;
            q[i + j] = bb[j] * xx[j] * s * (1.f - s);
            if (zp) zs += bb[j] * __ldg(zp + c0 + i + j);
          }
          float4 r = make_float4(o[0], o[1], o[2], o[3]);
          if (base) {
            const float4 bs = ld4(base + v * C + c0 + i);
            r.x += bs.x;
            r.y += bs.y;
            r.z += bs.z;
            r.w += bs.w;
          }
          *reinterpret_cast<float4*>(xbar + v * C + c0 + i) = r;
        }
      }
      put16(T, row, c0, C, q);
    }
    if (SPL > 1) {   // the two halves of the row add their parts of z_bar in a fixed order
      if (half == 1) zsh[wg][row] = zs;
      wg_sync(wg);
      if (half == 0) zs += zsh[wg][row];
    }
    if (zp && half == 0 && v < V) zbar[v] += zs;
    if (!wg_gemms(cx, err, D3, op_of(T, C), op_of(g2t, C), C, C)) break;
#pragma unroll
    for (int jj = 0; jj < C / 16; ++jj) {
      if (!owns(jj, half)) continue;
      const int c0 = 16 * jj;
      float hb[16], hp[16];
      tc::tmem_ld16(D3 + lb + c0, hb);
      tc::tmem_ld16(D1 + lb + c0, hp);
#pragma unroll
      for (int i = 0; i < 16; ++i) hb[i] *= gelu_grad(hp[i]);
      put16(T, row, c0, C, hb);
    }
    if (!wg_gemms(cx, err, D4, op_of(T, C), op_of(g1t, C), C, C)) break;
#pragma unroll
    for (int jj = 0; jj < C / 16; ++jj) {
      if (!owns(jj, half)) continue;
      const int c0 = 16 * jj;
      float r[16];
      tc::tmem_ld16(D4 + lb + c0, r);
      if (v < V)
#pragma unroll
        for (int i = 0; i < 16; i += 4) {
          float4* p = reinterpret_cast<float4*>(xbar + v * C + c0 + i);
          float4 o = *p;
          o.x += r[i];
          o.y += r[i + 1];
          o.z += r[i + 2];
          o.w += r[i + 3];
          *p = o;
        }
    }
  }
  wg_finish(cx, tmem_all, 2 * NCOL);
}

// Fuse backward, stage a: hf_bar_pre = (F_bar Wf2^T) * gelu'(B Wf1) with B = [spec gs, vert gv], F_bar =
// fused_pre_bar. Weights: [wf1 (2C x 2C), wf2t (2C x C)]. Per warpgroup one tile: B, then (after its GEMM) F_bar.
template <int C>
__global__ void __launch_bounds__(CT, 1) k_fuse_bwd_a_tc(const float* __restrict__ sp, const float* __restrict__ sc,
                                                      const float* __restrict__ vp, const float* __restrict__ vc,
                                                      const float* __restrict__ gates, const float* __restrict__ fb,
                                                      long V, const uint8_t* __restrict__ wpack,
                                                      float* __restrict__ hfb, int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(2 * C, 2 * C), B2 = mat_bytes(2 * C, C), RB = tile_bytes(2 * C);
  Split wf1 = split_at(smem, 2 * C, 2 * C), wf2t = split_at(smem + B1, 2 * C, C);
  TC_PROLOGUE_WG(4 * C)
  Split Bt = split_at(smem + B1 + B2 + wg * RB, TM, 2 * C), Ft = split_at(smem + B1 + B2 + wg * RB, TM, C);
  cx.ok = load_weights(smem, wpack, B1 + B2, wcx, err);
  for (long t = 2L * blockIdx.x + wg; cx.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (wtid == 0) {
      prefetch_rows(sp, (t + tstep) * TM, V, C);
      prefetch_rows(vp, (t + tstep) * TM, V, C);
      prefetch_rows(gates, (t + tstep) * TM, V, 2 * C);
      prefetch_rows(fb, (t + tstep) * TM, V, C);
    }
    wg_fill_tile<2 * C>(Bt, v0, V, wtid, [&](long v, int k) {
      const float4 g = ld4(gates + v * 2 * C + k);
      const float4 s =
          (k < C) ? gn4<true>(ld4(sp + v * C + k), sc, C, k) : gn4<true>(ld4(vp + v * C + k - C), vc, C, k - C);
      return make_float4(s.x * g.x, s.y * g.y, s.z * g.z, s.w * g.w);
    });
    if (!wg_gemms(cx, err, tmem, op_of(Bt, 2 * C), op_of(wf1, 2 * C), 2 * C, 2 * C)) break;
    wg_fill_tile<C>(Ft, v0, V, wtid, [&](long v, int k) { return ld4(fb + v * C + k); });
    if (!wg_gemms(cx, err, tmem + 2 * C, op_of(Ft, C), op_of(wf2t, C), C, 2 * C)) break;
    const long v = v0 + row;
#pragma unroll
    for (int jj = 0; jj < (2 * C) / 16; ++jj) {
      if (!owns(jj, half)) continue;
      const int c0 = 16 * jj;
      float hp[16], hb[16];
      tc::tmem_ld16(tmem + lb + c0, hp);
      tc::tmem_ld16(tmem + lb + 2 * C + c0, hb);
      if (v < V)
#pragma unroll
        for (int i = 0; i < 16; i += 4)
          *reinterpret_cast<float4*>(hfb + v * 2 * C + c0 + i) =
              make_float4(hb[i] * gelu_grad(hp[i]), hb[i + 1] * gelu_grad(hp[i + 1]), hb[i + 2] * gelu_grad(hp[i + 2]),
                          hb[i + 3] * gelu_grad(hp[i + 3]));
    }
  }
  wg_finish(cx, tmem_all, 2 * NCOL);
}

// Fuse backward, stage b: B_bar = hfb Wf1^T + [F_bar, F_bar] / 2; spec/vert grads B_bar g (+ the gate path);
// gate pre-activation grad q = B_bar [spec, vert] g (1 - g); hg_bar = (q Wg2^T) * gelu'(hg); A_bar = hg_bar Wg1^T:
// x_bar = base + A_bar[:C], spec_bar = B_bar_s g_s + A_bar[C:2C], vert_bar likewise.
// Weights: [wf1t (2C x 2C), wg2t (C x 2C), wg1t (3C x C)].
template <int C>
__global__ void __launch_bounds__(TT) k_fuse_bwd_b_tc(const float* __restrict__ sp, const float* __restrict__ sc,
                                                      const float* __restrict__ vp, const float* __restrict__ vc,
                                                      const float* __restrict__ gates, const float* __restrict__ hg,
                                                      const float* __restrict__ fb, const float* __restrict__ hfb,
                                                      const float* __restrict__ base, long V,
                                                      const uint8_t* __restrict__ wpack, float* __restrict__ xbar,
                                                      float* __restrict__ sbar, float* __restrict__ vbar,
                                                      int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(2 * C, 2 * C), B2 = mat_bytes(C, 2 * C), B3 = mat_bytes(3 * C, C);
  Split wf1t = split_at(smem, 2 * C, 2 * C), wg2t = split_at(smem + B1, C, 2 * C), wg1t = split_at(smem + B1 + B2, 3 * C, C);
  uint8_t* region = smem + B1 + B2 + B3;
  Split A2 = split_at(region, TM, 2 * C), A1 = split_at(region, TM, C);
  TC_PROLOGUE(3 * C)
  cx.ok = load_weights(smem, wpack, B1 + B2 + B3, cx, err);
  for (long t = blockIdx.x; cx.ok && t < nt; t += gridDim.x) {
    const long v0 = t * TM;
    if (tid == 0) {
      prefetch_rows(hfb, (t + gridDim.x) * TM, V, 2 * C);
      prefetch_rows(fb, (t + gridDim.x) * TM, V, C);
      prefetch_rows(gates, (t + gridDim.x) * TM, V, 2 * C);
      prefetch_rows(sp, (t + gridDim.x) * TM, V, C);
      prefetch_rows(vp, (t + gridDim.x) * TM, V, C);
      prefetch_rows(hg, (t + gridDim.x) * TM, V, C);
      prefetch_rows(base, (t + gridDim.x) * TM, V, C);
    }
    const long v = v0 + row;
    fill_tile<2 * C>(A2, v0, V, [&](long vv, int k) { return ld4(hfb + vv * 2 * C + k); });
    if (!gemms(cx, err, tmem, A2, wf1t, 2 * C, 2 * C)) break;
#pragma unroll
    for (int jj = 0; jj < (2 * C) / 16; ++jj) if ((jj & 1) == wg) {
      const int c0 = 16 * jj;
      float bb[16], q[16];
      tc::tmem_ld16(tmem + lb + c0, bb);
#pragma unroll
      for (int i = 0; i < 16; ++i) q[i] = 0.f;
      if (v < V) {
        const bool is_s = c0 < C;
        const int cc = is_s ? c0 : c0 - C;
        const float* pre = is_s ? sp : vp;
        const float* cf = is_s ? sc : vc;
        float* gout = is_s ? sbar : vbar;
#pragma unroll
        for (int i = 0; i < 16; i += 4) {
          const float4 f4 = ld4(fb + v * C + cc + i), g4 = ld4(gates + v * 2 * C + c0 + i);
          const float4 s4 = gn4<true>(ld4(pre + v * C + cc + i), cf, C, cc + i);
          const float ff[4] = {f4.x, f4.y, f4.z, f4.w}, gg[4] = {g4.x, g4.y, g4.z, g4.w}, ss[4] = {s4.x, s4.y, s4.z, s4.w};
          float o[4];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const float b = bb[i + j] + 0.5f * ff[j];
            o[j] = b * gg[j];
            q[i + j] = b * ss[j] * gg[j] * (1.f - gg[j]);
          }
          *reinterpret_cast<float4*>(gout + v * C + cc + i) = make_float4(o[0], o[1], o[2], o[3]);
        }
      }
      put16(A2, row, c0, 2 * C, q);
    }
    if (!gemms(cx, err, tmem + 2 * C, A2, wg2t, 2 * C, C)) break;
#pragma unroll
    for (int jj = 0; jj < (C) / 16; ++jj) if ((jj & 1) == wg) {
      const int c0 = 16 * jj;
      float hb[16];
      tc::tmem_ld16(tmem + lb + 2 * C + c0, hb);
      if (v < V)
#pragma unroll
        for (int i = 0; i < 16; i += 4) {
          const float4 h4 = ld4(hg + v * C + c0 + i);
          hb[i] *= gelu_grad(h4.x);
          hb[i + 1] *= gelu_grad(h4.y);
          hb[i + 2] *= gelu_grad(h4.z);
          hb[i + 3] *= gelu_grad(h4.w);
        }
      put16(A1, row, c0, C, hb);
    }
    if (!gemms(cx, err, tmem, A1, wg1t, C, 3 * C)) break;
#pragma unroll
    for (int jj = 0; jj < (3 * C) / 16; ++jj) if ((jj & 1) == wg) {
      const int c0 = 16 * jj;
      float r[16];
      tc::tmem_ld16(tmem + lb + c0, r);
      if (v < V) {
        if (c0 < C) {
#pragma unroll
          for (int i = 0; i < 16; i += 4) {
            float4 o = make_float4(r[i], r[i + 1], r[i + 2], r[i + 3]);
            if (base) {
              const float4 b4 = ld4(base + v * C + c0 + i);
              o.x += b4.x;
              o.y += b4.y;
              o.z += b4.z;
              o.w += b4.w;
            }
            *reinterpret_cast<float4*>(xbar + v * C + c0 + i) = o;
          }
        } else {
          float* g = c0 < 2 * C ? sbar : vbar;
          const int cc = c0 < 2 * C ? c0 - C : c0 - 2 * C;
#pragma unroll
          for (int i = 0; i < 16; i += 4) {
            float4* p = reinterpret_cast<float4*>(g + v * C + cc + i);
            float4 o = *p;
            o.x += r[i];
            o.y += r[i + 1];
            o.z += r[i + 2];
            o.w += r[i + 3];
            *p = o;
          }
        }
      }
    }
  }
  finish(cx, tmem, NCOL);
}

#undef TC_PROLOGUE
#undef TC_PROLOGUE_WG

int g_sms = 0;
int sms() {
  if (!g_sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_sms <= 0) g_sms = 152;
  }
  return g_sms;
}

int grid_tc(long V) {
  const long t = ((V + TM - 1) / TM + 1) / 2;   // two warpgroup pipelines per CTA
  const long g = (long)sms();
  return (int)(t < g ? (t > 0 ? t : 1) : g);
}

template <typename K>
bool launch_prep(K kernel, size_t bytes) {
  if (bytes > 227 * 1024 - 1024) return false;   // leave room for the kernels' static shared memory
  return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) == cudaSuccess;
}

bool tc_width(int C) { return C == 16 || C == 32 || C == 64; }
bool aligned16(const void* p) { return p && (reinterpret_cast<uintptr_t>(p) % 16) == 0; }

}  // namespace

// ====================================================================================================== C ABI
extern "C" {

int ffno_tc_parts(long V) { return grid_tc(V); }

int ffno_tc_width_supported(int C) { return tc_width(C) ? 1 : 0; }

#define TC_DISPATCH(C, ...)  \
  switch (C) {               \
    case 16: {               \
      constexpr int CC = 16; \
      __VA_ARGS__;           \
      break;                 \
    }                        \
    case 32: {               \
      constexpr int CC = 32; \
      __VA_ARGS__;           \
      break;                 \
    }                        \
    case 64: {               \
      constexpr int CC = 64; \
      __VA_ARGS__;           \
      break;                 \
    }                        \
    default:                 \
      return FFNO_EINVAL;    \
  }

int ffno_mlp2_fwd_tc(int mode, const float* in, const float* prev_pre, const float* prev_coefs, float res, float* xout,
                     long V, int C, const void* wpack, const float* dw, float* pre, double* partials, int nparts,
                     int groups, int* err, ffno_stream_t stream) {
  if (!tc_width(C) || V < 1 || mode < 0 || mode > 2 || groups != GMAX || !err || !aligned16(wpack)) return FFNO_EINVAL;
  if (mode && (!prev_pre || !prev_coefs || !xout)) return FFNO_EINVAL;
  if (nparts != grid_tc(V)) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  const auto* w = static_cast<const uint8_t*>(wpack);
  TC_DISPATCH(C, {
    const size_t smem = mat_bytes(2 * CC, CC) + mat_bytes(CC, 2 * CC) + 2 * tile_bytes(2 * CC);
    if (mode == 0) {
      if (!launch_prep(k_mlp2_tc<CC, 0>, smem)) return FFNO_ELAUNCH;
      k_mlp2_tc<CC, 0><<<nparts, CT, smem, s>>>(in, prev_pre, prev_coefs, res, xout, V, w, dw, pre, partials, err);
    } else if (mode == 1) {
      if (!launch_prep(k_mlp2_tc<CC, 1>, smem)) return FFNO_ELAUNCH;
      k_mlp2_tc<CC, 1><<<nparts, CT, smem, s>>>(in, prev_pre, prev_coefs, res, xout, V, w, dw, pre, partials, err);
    } else {
      if (!launch_prep(k_mlp2_tc<CC, 2>, smem)) return FFNO_ELAUNCH;
      k_mlp2_tc<CC, 2><<<nparts, CT, smem, s>>>(in, prev_pre, prev_coefs, res, xout, V, w, dw, pre, partials, err);
    }
  })
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_gate_fwd_tc(const float* x, long V, int C, const void* wpack, const float* zp, const float* z, float* out,
                     int* err, ffno_stream_t stream) {
  if (!tc_width(C) || V < 1 || !err || !aligned16(wpack) || (zp && !z)) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  TC_DISPATCH(C, {
    const size_t smem = 2 * mat_bytes(CC, CC) + 2 * tile_bytes(CC);
    if (!launch_prep(k_gate_tc<CC>, smem)) return FFNO_ELAUNCH;
    k_gate_tc<CC><<<grid_tc(V), CT, smem, s>>>(x, V, static_cast<const uint8_t*>(wpack), zp, z, out, err);
  })
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_fuse1_tc(const float* x, const float* spec_pre, const float* spec_coefs, const float* vert_pre,
                  const float* vert_coefs, long V, int C, const void* wpack, const float* bias, float* gates,
                  float* hg, int* err, ffno_stream_t stream) {
  if (!tc_width(C) || V < 1 || !err || !aligned16(wpack) || !gates) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  TC_DISPATCH(C, {
    const size_t smem = mat_bytes(CC, 3 * CC) + mat_bytes(2 * CC, CC) + 2 * tile_bytes(CC);
    if (!launch_prep(k_fuse1_tc<CC>, smem)) return FFNO_ELAUNCH;
    k_fuse1_tc<CC><<<grid_tc(V), CT, smem, s>>>(x, spec_pre, spec_coefs, vert_pre, vert_coefs, V,
                                               static_cast<const uint8_t*>(wpack), bias, gates, hg, err);
  })
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_fuse2_tc(const float* spec_pre, const float* spec_coefs, const float* vert_pre, const float* vert_coefs,
                  const float* gates, long V, int C, const void* wpack, const float* dw, float* pre, double* partials,
                  int nparts, int groups, int* err, ffno_stream_t stream) {
  if (!tc_width(C) || V < 1 || !err || !aligned16(wpack) || groups != GMAX || nparts != grid_tc(V)) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  TC_DISPATCH(C, {
    const size_t smem = mat_bytes(2 * CC, 2 * CC) + mat_bytes(CC, 2 * CC) + 2 * tile_bytes(2 * CC);
    if (!launch_prep(k_fuse2_tc<CC>, smem)) return FFNO_ELAUNCH;
    k_fuse2_tc<CC><<<nparts, CT, smem, s>>>(spec_pre, spec_coefs, vert_pre, vert_coefs, gates, V,
                                           static_cast<const uint8_t*>(wpack), dw, pre, partials, err);
  })
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_mlp2_bwd_tc(const float* a, const float* pre_bar, const float* base, long V, int C, const void* wpack,
                     float* a_bar, int* err, ffno_stream_t stream) {
  if (!tc_width(C) || V < 1 || !err || !aligned16(wpack)) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  TC_DISPATCH(C, {
    const size_t smem = 3 * mat_bytes(2 * CC, CC) + 2 * tile_bytes(2 * CC);
    if (!launch_prep(k_mlp2_bwd_tc<CC>, smem)) return FFNO_ELAUNCH;
    k_mlp2_bwd_tc<CC><<<grid_tc(V), CT, smem, s>>>(a, pre_bar, base, V, static_cast<const uint8_t*>(wpack), a_bar,
                                                  err);
  })
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_gate_bwd_tc(const float* x, const float* g_bar, const float* base, long V, int C, const void* wpack,
                     const float* zp, float* x_bar, float* z_bar, int* err, ffno_stream_t stream) {
  if (!tc_width(C) || V < 1 || !err || !aligned16(wpack) || (zp && !z_bar)) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  TC_DISPATCH(C, {
    const size_t smem = 4 * mat_bytes(CC, CC) + 4 * tile_bytes(CC);
    if (!launch_prep(k_gate_bwd_tc<CC>, smem)) return FFNO_ELAUNCH;
    k_gate_bwd_tc<CC><<<grid_tc(V), CT, smem, s>>>(x, g_bar, base, V, static_cast<const uint8_t*>(wpack), zp, x_bar,
                                                  z_bar, err);
  })
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_fuse_bwd_a_tc(const float* spec_pre, const float* spec_coefs, const float* vert_pre, const float* vert_coefs,
                       const float* gates, const float* fused_pre_bar, long V, int C, const void* wpack,
                       float* hf_bar, int* err, ffno_stream_t stream) {
  if (!tc_width(C) || V < 1 || !err || !aligned16(wpack)) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  TC_DISPATCH(C, {
    const size_t smem = mat_bytes(2 * CC, 2 * CC) + mat_bytes(2 * CC, CC) + 2 * tile_bytes(2 * CC);
    if (!launch_prep(k_fuse_bwd_a_tc<CC>, smem)) return FFNO_ELAUNCH;
    k_fuse_bwd_a_tc<CC><<<grid_tc(V), CT, smem, s>>>(spec_pre, spec_coefs, vert_pre, vert_coefs, gates, fused_pre_bar,
                                                    V, static_cast<const uint8_t*>(wpack), hf_bar, err);
  })
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_fuse_bwd_b_tc(const float* spec_pre, const float* spec_coefs, const float* vert_pre, const float* vert_coefs,
                       const float* gates, const float* hg, const float* fused_pre_bar, const float* hf_bar,
                       const float* base, long V, int C, const void* wpack, float* x_bar, float* spec_bar,
                       float* vert_bar, int* err, ffno_stream_t stream) {
  if (!tc_width(C) || V < 1 || !err || !aligned16(wpack)) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  TC_DISPATCH(C, {
    const size_t smem =
        mat_bytes(2 * CC, 2 * CC) + mat_bytes(CC, 2 * CC) + mat_bytes(3 * CC, CC) + tile_bytes(2 * CC);
    if (!launch_prep(k_fuse_bwd_b_tc<CC>, smem)) return FFNO_ELAUNCH;
    k_fuse_bwd_b_tc<CC><<<grid_tc(V), TT, smem, s>>>(spec_pre, spec_coefs, vert_pre, vert_coefs, gates, hg,
                                                    fused_pre_bar, hf_bar, base, V,
                                                    static_cast<const uint8_t*>(wpack), x_bar, spec_bar, vert_bar,
                                                    err);
  })
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

}  // extern "C"
