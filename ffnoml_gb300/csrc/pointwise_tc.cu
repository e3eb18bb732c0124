// Tensor-core (tcgen05) versions of the pointwise channel-MLP chains, in split-BF16: every GEMM operand x is carried as
// hi = bf16(x) and lo = bf16(x - hi), and each product as hi*hi + hi*lo + lo*hi on the BF16 tensor cores with FP32
// accumulation in tensor memory (relative error about 2^-16; a single BF16 product, 2^-8, moves log10 n by 1e-2).
// Activations, residuals and GroupNorm statistics stay FP32 in HBM, so every kernel has the contract of an FP32 entry
// point of pointwise_f32.cu / backward_f32.cu (or of a stage of one).
//
// Orientation: every GEMM is computed transposed, D^T [features][128 voxels] = W X^T, with the split weights
// (packed on the host in the canonical K-major order, [out][in]) as the A operand and the voxel tile as the B operand.
// A tensor-memory lane is then an output feature and a column a voxel, so in every epilogue a warp's loads and stores
// cover 32 consecutive channels of one voxel (128-byte runs), and intermediate activations are written back as
// MN-major B tiles (voxels contiguous) with conflict-free 16-byte stores. Weight matrices with fewer than 128 rows
// are read as 128-row A operands whose extra rows (the bytes that follow in shared memory) land in accumulator lanes
// no epilogue reads. Input tiles arrive as split K-major tiles [128 voxels][K], filled from FP32 HBM.
//
// A CTA holds two pipelines of 256 threads (eight warps each) that take alternate 128-voxel tiles; each has its own
// operand tiles, tensor-memory columns, MMA mbarrier and named barrier, so one pipeline's fills and epilogues overlap
// the other's MMAs. In an epilogue, warp w of a pipeline reads lanes 32 (w % 4) .. + 31 and the voxel columns of its
// half (w / 4). MMAs are issued by one thread of the pipeline and complete on its mbarrier; every wait is bounded: a
// timeout sets *err, the pipeline leaves its tile loop, and the CTA frees its tensor memory after one more bounded
// wait.
#include <math.h>

#include "common.cuh"
#include "tc.cuh"
#include "ws.h"

using namespace ffno;

namespace {

constexpr int TM = 128;  // voxels per tile = accumulator columns
constexpr int PT = 256;  // threads per pipeline
constexpr int CT = 512;  // threads per CTA (two pipelines)
constexpr int FB = 8;    // fill: independent loads in flight per thread

__host__ __device__ constexpr uint32_t tmem_cols(int n) {
  return n <= 32 ? 32 : n <= 64 ? 64 : n <= 128 ? 128 : n <= 256 ? 256 : 512;
}

// bytes of one split matrix (hi + lo) of R x K
__host__ __device__ constexpr uint32_t mat_bytes(int R, int K) { return (uint32_t)R * K * 2 * 2; }
// bytes of one split voxel tile of 128 x K
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

// Tiles of L2 prefetch lookahead per pipeline: at tile t a pipeline prefetches the inputs of its tile t + c_pf steps
// ahead (0: none, the default: with 32-byte row requests the prefetched lines only added DRAM traffic). Set by
// ffno_tc_set_prefetch_tiles.
__constant__ int c_pf = 0;

// L2 prefetch of rows [n0, n0 + 128) of a [V][width] FP32 array, by one thread
__device__ __forceinline__ void prefetch_rows(const float* base, long n0, long V, int width) {
  if (!base || n0 >= V) return;
  const long rows = (V - n0) < TM ? (V - n0) : TM;
  tc::prefetch_l2(base + n0 * width, (uint32_t)(rows * width * 4));
}

__device__ __forceinline__ float4 ld4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

__device__ __forceinline__ void ld8(const float* p, float (&o)[8]) { tc::ld8(p, o); }
__device__ __forceinline__ void st8(float* p, const float* v) { tc::st8(p, v); }

// GroupNorm coefficients (mean, gamma * rstd, beta) of 4 consecutive channels, and their application (+ GELU)
struct Gn4 {
  float4 m, s, b;
};
__device__ __forceinline__ Gn4 gn_coefs(const float* __restrict__ cf, int C, int k) {
  return Gn4{ld4(cf + k), ld4(cf + C + k), ld4(cf + 2 * C + k)};
}
template <bool GELU>
__device__ __forceinline__ float4 gn_apply(float4 p, const Gn4& g) {
  float4 y = make_float4((p.x - g.m.x) * g.s.x + g.b.x, (p.y - g.m.y) * g.s.y + g.b.y, (p.z - g.m.z) * g.s.z + g.b.z,
                         (p.w - g.m.w) * g.s.w + g.b.w);
  if (GELU) y = make_float4(gelu_tc(y.x), gelu_tc(y.y), gelu_tc(y.z), gelu_tc(y.w));
  return y;
}

// ---------------------------------------------------------------------------------------------------- pipelines
struct Pipe {
  uint64_t* bar;   // MMA completion
  uint32_t phase;
  bool ok;
  int id, ptid, lane, q, half;
  uint32_t tmem;   // this pipeline's first tensor-memory column (lane 0)
  uint32_t lq;     // lane-quadrant offset of this warp
  __device__ int feat() const { return 32 * q + lane; }   // accumulator lane = output feature of this thread
};

__device__ __forceinline__ void pipe_sync(int id) {
  asm volatile("bar.sync %0, %1;" ::"r"(1 + id), "n"(PT) : "memory");
}

__device__ __forceinline__ bool pipe_sync_and(int id, bool p) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred pi, po;\n setp.ne.u32 pi, %1, 0;\n bar.red.and.pred po, %2, %3, pi;\n selp.u32 %0, 1, 0, po;\n}"
      : "=r"(r)
      : "r"((uint32_t)p), "r"(1 + id), "n"(PT)
      : "memory");
  return r != 0;
}

// An MMA operand in shared memory: hi / lo shared addresses, descriptor strides, bytes per 16-wide k step.
struct Op {
  uint32_t hi, lo, lbo, sbo, step;
  bool mn;
};
// weight matrix [R][K] (K-major) from row r0 (a multiple of 8) and column k0 (a multiple of 8); read as 128 rows
__device__ __forceinline__ Op wop(const uint8_t* p, int R, int K, int r0 = 0, int k0 = 0) {
  const uint32_t h = tc::smem_u32(p) + (uint32_t)(r0 / 8) * (uint32_t)K * 16u + (uint32_t)(k0 / 8) * 128u;
  return Op{h, h + (uint32_t)R * K * 2, 128u, (uint32_t)K * 16u, 256u, false};
}
// voxel tile [128][K] stored K-major (filled from HBM), optionally the K-slice from column k0
__device__ __forceinline__ Op kop(Split t, int K, int k0 = 0) {
  const uint32_t o = (uint32_t)(k0 / 8) * 128u;
  return Op{tc::smem_u32(t.hi()) + o, tc::smem_u32(t.lo()) + o, 128u, (uint32_t)K * 16u, 256u, false};
}
// voxel tile [128][K] stored MN-major (voxels contiguous; written by epilogues)
__device__ __forceinline__ Op mop(Split t) {
  return Op{tc::smem_u32(t.hi()), tc::smem_u32(t.lo()), 2048u, 128u, 4096u, true};
}

// D [128 x N] (+)= A B^T over K, split-BF16 (Ah Bh + Ah Bl + Al Bh); either operand K- or MN-major
__device__ __forceinline__ void mma3(uint32_t d, const Op& a, const Op& b, int K, int N, bool acc) {
  const uint32_t idesc = tc::idesc_bf16_ab(128, N, a.mn, b.mn);
  const uint32_t as[3] = {a.hi, a.hi, a.lo}, bs[3] = {b.hi, b.lo, b.hi};
#pragma unroll
  for (int s = 0; s < 3; ++s)
    for (int k = 0; k < K; k += 16) {
      const uint64_t ad = tc::kmajor_desc(as[s] + (uint32_t)(k / 16) * a.step, a.lbo, a.sbo);
      const uint64_t bd = tc::kmajor_desc(bs[s] + (uint32_t)(k / 16) * b.step, b.lbo, b.sbo);
      tc::mma_bf16(d, ad, bd, idesc, (acc || s > 0 || k > 0) ? 1u : 0u);
    }
}

struct Gemm {
  uint32_t d;
  Op a, b;
  int K;
  bool acc;
  int N = 128;
};

// Issue up to three split GEMMs (the pipeline's thread 0) behind one commit and wait for them (the pipeline).
__device__ __forceinline__ bool pipe_gemms(Pipe& p, int* err, const Gemm& g0, const Gemm* g1 = nullptr,
                                           const Gemm* g2 = nullptr) {
  tc::fence_async_smem();
  tc::tc_before_sync();
  pipe_sync(p.id);
  tc::tc_after_sync();
  if (p.ptid == 0) {
    mma3(g0.d, g0.a, g0.b, g0.K, g0.N, g0.acc);
    if (g1) mma3(g1->d, g1->a, g1->b, g1->K, g1->N, g1->acc);
    if (g2) mma3(g2->d, g2->a, g2->b, g2->K, g2->N, g2->acc);
    tc::mma_commit(p.bar);
  }
  const bool ok = pipe_sync_and(p.id, tc::mbar_wait(p.bar, p.phase));
  p.phase ^= 1u;
  tc::tc_after_sync();
  if (!ok && p.ptid == 0) atomicExch(err, 2);
  p.ok = ok;
  return ok;
}

// 16 accumulator columns (voxels 64 half + 16 c .. + 15) of this thread's lane, from accumulator base column d
__device__ __forceinline__ void tld(const Pipe& p, uint32_t d, int c, float (&v)[16]) {
  tc::tmem_ld16(p.tmem + p.lq + d + (uint32_t)(64 * p.half + 16 * c), v);
}

// Write 16 values of feature j for voxels vl .. vl + 15 (vl a multiple of 8) into an MN-major split tile [128][K]
__device__ __forceinline__ void put_mn(Split t, int j, int vl, const float (&v)[16]) {
#pragma unroll
  for (int g = 0; g < 2; ++g) {
    uint32_t h[4], l[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) tc::split_pack(v[8 * g + 2 * i], v[8 * g + 2 * i + 1], h[i], l[i]);
    const uint32_t o = tc::mnmajor_offset(vl + 8 * g, j, TM);
    *reinterpret_cast<uint4*>(t.hi() + o) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4*>(t.lo() + o) = make_uint4(l[0], l[1], l[2], l[3]);
  }
}

// Fill a split K-major tile [128][KW] from FP32 sources: f(v, k) returns columns k..k+3 of voxel v (v < V); rows past
// the cube are zero. With 256 threads, thread t always serves columns fill_col<KW>(t) .. + 3.
template <int KW>
__device__ __forceinline__ int fill_col(int ptid) {
  return ((ptid >> 4) % (KW / 8)) * 8 + (ptid & 1) * 4;
}
template <int KW, typename F>
__device__ __forceinline__ void fill_tile(Split t, long v0, long V, int ptid, F f) {
  static_assert(16 % (KW / 8) == 0 || (KW / 8) % 16 == 0, "fill columns must be fixed per thread");
  constexpr int NE = TM * KW / 4;
  for (int e0 = ptid; e0 < NE; e0 += PT * FB) {
    float4 a[FB];
#pragma unroll
    for (int u = 0; u < FB; ++u) {  // issue the loads of FB pieces before converting any of them
      const int e = e0 + u * PT;
      const int h = e & 1, r8 = (e >> 1) & 7, q = e >> 4;
      const int kb = q % (KW / 8), rb = q / (KW / 8);
      const long v = v0 + rb * 8 + r8;
      a[u] = (e < NE && v < V) ? f(v, kb * 8 + h * 4) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < FB; ++u) {
      const int e = e0 + u * PT;
      if (e >= NE) break;
      uint32_t h0, l0, h1, l1;
      tc::split_pack(a[u].x, a[u].y, h0, l0);
      tc::split_pack(a[u].z, a[u].w, h1, l1);
      *reinterpret_cast<uint2*>(t.hi() + (size_t)e * 8) = make_uint2(h0, h1);
      *reinterpret_cast<uint2*>(t.lo() + (size_t)e * 8) = make_uint2(l0, l1);
    }
  }
}

// fill_tile with 8 columns a piece: f(v, k, o) writes columns k..k+7 of voxel v into o (32-byte loads; a warp's
// request covers 8 rows x 128 bytes). The pieces land in the same K-major layout, hi and lo in one 16-byte store each.
// Thread t always serves columns fill_col8<KW>(t) .. + 7; half as many pieces in flight as fill_tile, the same bytes.
template <int KW>
__device__ __forceinline__ int fill_col8(int ptid) {
  return ((ptid >> 3) % (KW / 8)) * 8;
}
template <int KW, typename F>
__device__ __forceinline__ void fill_tile8(Split t, long v0, long V, int ptid, F f) {
  static_assert(32 % (KW / 8) == 0, "fill columns must be fixed per thread");
  constexpr int NE = TM * KW / 8;
  constexpr int FB8 = FB / 2;
  for (int e0 = ptid; e0 < NE; e0 += PT * FB8) {
    float a[FB8][8];
#pragma unroll
    for (int u = 0; u < FB8; ++u) {   // issue the loads of FB8 pieces before converting any of them
      const int e = e0 + u * PT;
      const int r8 = e & 7, q = e >> 3;
      const int kb = q % (KW / 8), rb = q / (KW / 8);
      const long v = v0 + rb * 8 + r8;
      if (e < NE && v < V) {
        f(v, kb * 8, a[u]);
      } else {
#pragma unroll
        for (int i = 0; i < 8; ++i) a[u][i] = 0.f;
      }
    }
#pragma unroll
    for (int u = 0; u < FB8; ++u) {
      const int e = e0 + u * PT;
      if (e >= NE) break;
      uint32_t h[4], l[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) tc::split_pack(a[u][2 * i], a[u][2 * i + 1], h[i], l[i]);
      *reinterpret_cast<uint4*>(t.hi() + (size_t)e * 16) = make_uint4(h[0], h[1], h[2], h[3]);
      *reinterpret_cast<uint4*>(t.lo() + (size_t)e * 16) = make_uint4(l[0], l[1], l[2], l[3]);
    }
  }
}

// The production model's width: rows of 12 octets, weights read as transposes (below and in the width-96 kernels).
constexpr int C96 = 96;

// the transpose of the K-major weight matrix [R][K] at p, as the MN-major operand [N = K][K' = R] from k' = r0 and
// n = n0 (multiples of 8)
__device__ __forceinline__ Op wop_t(const uint8_t* p, int R, int K, int r0 = 0, int n0 = 0) {
  const uint32_t h = tc::smem_u32(p) + (uint32_t)(r0 / 8) * (uint32_t)K * 16u + (uint32_t)(n0 / 8) * 128u;
  return Op{h, h + (uint32_t)R * K * 2, (uint32_t)K * 16u, 128u, (uint32_t)K * 32u, true};
}

// fill_tile8 for KW = 48 or 96 columns (6 or 12 octets a row, so a thread's columns change from piece to piece)
template <int KW, typename F>
__device__ __forceinline__ void fill_oct(Split t, long v0, long V, int ptid, F f) {
  constexpr int KB = KW / 8, NE = TM * KB, FB8 = FB / 2;
  for (int e0 = ptid; e0 < NE; e0 += PT * FB8) {
    float a[FB8][8];
#pragma unroll
    for (int u = 0; u < FB8; ++u) {   // the loads of FB8 pieces issued before any is converted
      const int e = e0 + u * PT;
      const int r8 = e & 7, q = e >> 3;
      const long v = v0 + (q / KB) * 8 + r8;
      if (e < NE && v < V) {
        f(v, (q % KB) * 8, a[u]);
      } else {
#pragma unroll
        for (int i = 0; i < 8; ++i) a[u][i] = 0.f;
      }
    }
#pragma unroll
    for (int u = 0; u < FB8; ++u) {
      const int e = e0 + u * PT;
      if (e >= NE) break;
      uint32_t h[4], l[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) tc::split_pack(a[u][2 * i], a[u][2 * i + 1], h[i], l[i]);
      *reinterpret_cast<uint4*>(t.hi() + (size_t)e * 16) = make_uint4(h[0], h[1], h[2], h[3]);
      *reinterpret_cast<uint4*>(t.lo() + (size_t)e * 16) = make_uint4(l[0], l[1], l[2], l[3]);
    }
  }
}

// Plain FP32 rows [V][C] of src into a split K-major tile [128][C]; every width, 96 included (12 octets a row).
template <typename F>
__device__ __forceinline__ void fill96(Split t, long v0, long V, int ptid, F f) {
  fill_oct<C96>(t, v0, V, ptid, f);
}

template <int C>
__device__ __forceinline__ void fill_rows(Split t, long v0, long V, int ptid, const float* __restrict__ src) {
  if constexpr (C == 96)
    fill96(t, v0, V, ptid, [&](long v, int k, float (&o)[8]) { ld8(src + v * C + k, o); });
  else
    fill_tile<C>(t, v0, V, ptid, [&](long v, int k) { return ld4(src + v * C + k); });
}

// The tile's depth weights into shared memory (wt[128]) and their warp partial sums (wpart[4]); threads ptid < 128.
__device__ __forceinline__ void load_tile_weights(const Pipe& p, const float* __restrict__ dw, long v0, long V,
                                                  float* wt, float* wpart) {
  if (p.ptid < TM) {
    const long v = v0 + p.ptid;
    float w = v < V ? __ldg(dw + v) : 0.f;
    wt[p.ptid] = w;
#pragma unroll
    for (int o = 16; o; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
    if (p.lane == 0) wpart[p.ptid >> 5] = w;
  }
}

// Depth-weighted statistics of the tile's output features (lanes < C of the accumulator at column d; the tile's
// weights wt[128], partial sums wpart[4] written before the last pipeline barrier), merged with Chan's update into
// acc[g] = (w, mean, m2) by the thread holding the group's first lane. Fixed order throughout.
template <int C>
__device__ __forceinline__ void tile_stats(const Pipe& p, uint32_t d, const float* wt, const float* wpart,
                                           float* red /* [2][2][GMAX] */, double* acc /* [GMAX][3] */) {
  constexpr int CPG = C / GMAX;
  const int f = p.feat(), g = f / CPG;
  const bool live = f < C;
  const float wsum = (wpart[0] + wpart[1]) + (wpart[2] + wpart[3]);
  float s = 0.f;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float v[16];
    tld(p, d, c, v);
#pragma unroll
    for (int i = 0; i < 16; ++i) s = fmaf(wt[64 * p.half + 16 * c + i], v[i], s);
  }
#pragma unroll
  for (int o = 1; o < CPG; o <<= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (live && f % CPG == 0) red[p.half * GMAX + g] = s;
  pipe_sync(p.id);
  const float wt_g = wsum * CPG;
  const float mean = live && wt_g > 0.f ? (red[g] + red[GMAX + g]) / wt_g : 0.f;
  float s2 = 0.f;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float v[16];
    tld(p, d, c, v);
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const float e = v[i] - mean;
      s2 = fmaf(wt[64 * p.half + 16 * c + i] * e, e, s2);
    }
  }
#pragma unroll
  for (int o = 1; o < CPG; o <<= 1) s2 += __shfl_xor_sync(0xffffffffu, s2, o);
  if (live && f % CPG == 0) red[2 * GMAX + p.half * GMAX + g] = s2;
  pipe_sync(p.id);
  if (live && f % CPG == 0 && p.half == 0) {
    double* a = acc + 3 * g;
    GroupAcc ga{a[0], a[1], a[2]};
    chan_merge(ga, (double)wt_g, (double)mean, (double)(red[2 * GMAX + g] + red[3 * GMAX + g]));
    a[0] = ga.w;
    a[1] = ga.mean;
    a[2] = ga.m2;
  }
  pipe_sync(p.id);
}

// ---------------------------------------------------------------------------------------------- row orientation
// GEMMs with C outputs run untransposed, D [128 voxels][C] = X W^T (the voxel tile as the A operand, K- or MN-major,
// the weights as the B operand), so that every accumulator lane is live: thread feat() of a pipeline serves voxel
// row feat() and the 16-column chunks j with j % 2 == half.
__device__ __forceinline__ bool owns(int j, int half) { return (j & 1) == half; }

__device__ __forceinline__ void rld(const Pipe& p, uint32_t d, int j, float (&v)[16]) {
  tc::tmem_ld16(p.tmem + p.lq + d + (uint32_t)(16 * j), v);
}

// Write 16 values of row r into a split K-major tile with K columns at columns c0..c0+15.
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

// Depth-weighted statistics of a row-oriented tile: every thread holds, in v[C], the chunks of its row it owns and
// the row's weight w (0 past the cube). Merged with Chan's update into acc[g] by thread g < GMAX; fixed order.
// red: [8][GMAX + 1] of this pipeline.
template <int C>
__device__ __forceinline__ void row_stats(const Pipe& p, const float (&v)[C], float w, float* red, float* gm,
                                          float* wsum, double* acc) {
  constexpr int CPG = C / GMAX, NW = PT / 32;
  const int lane = p.lane, wl = p.ptid >> 5;
  float ws = p.half == 0 ? w : 0.f;
#pragma unroll
  for (int o = 16; o; o >>= 1) ws += __shfl_xor_sync(0xffffffffu, ws, o);
  float s[GMAX];
#pragma unroll
  for (int g = 0; g < GMAX; ++g) s[g] = 0.f;
#pragma unroll
  for (int c = 0; c < C; ++c)
    if (owns(c / 16, p.half)) s[c / CPG] += v[c];
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
  pipe_sync(p.id);
  if (p.ptid == 0) {
    float t = 0.f;
    for (int q = 0; q < NW; ++q) t += red[q * (GMAX + 1) + GMAX];
    *wsum = t;
  }
  if (p.ptid < GMAX) {
    float t = 0.f, wt = 0.f;
    for (int q = 0; q < NW; ++q) {
      t += red[q * (GMAX + 1) + p.ptid];
      wt += red[q * (GMAX + 1) + GMAX];
    }
    wt *= CPG;
    gm[p.ptid] = wt > 0.f ? t / wt : 0.f;
  }
  pipe_sync(p.id);
#pragma unroll
  for (int g = 0; g < GMAX; ++g) s[g] = 0.f;
#pragma unroll
  for (int c = 0; c < C; ++c)
    if (owns(c / 16, p.half)) {
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
  pipe_sync(p.id);
  if (p.ptid < GMAX) {
    float t = 0.f;
    for (int q = 0; q < NW; ++q) t += red[q * (GMAX + 1) + p.ptid];
    double* a = acc + 3 * p.ptid;
    GroupAcc ga{a[0], a[1], a[2]};
    chan_merge(ga, (double)*wsum * CPG, (double)gm[p.ptid], (double)t);
    a[0] = ga.w;
    a[1] = ga.mean;
    a[2] = ga.m2;
  }
  pipe_sync(p.id);
}

// The CTA's GroupNorm partial: pipeline 1's statistics merged into pipeline 0's (fixed order). All threads call it.
__device__ __forceinline__ void write_partial2(double* partials, const double* acc /* [2][GMAX][3] */) {
  __syncthreads();
  const int t = threadIdx.x;
  if (t < GMAX) {
    GroupAcc a{acc[3 * t], acc[3 * t + 1], acc[3 * t + 2]};
    chan_merge(a, acc[3 * GMAX + 3 * t], acc[3 * GMAX + 3 * t + 1], acc[3 * GMAX + 3 * t + 2]);
    double* o = partials + ((long)blockIdx.x * GMAX + t) * 3;
    o[0] = a.w;
    o[1] = a.mean;
    o[2] = a.m2;
  }
}

// After both pipelines left their loops: wait once more (bounded) for an MMA of a failed wait, free tensor memory.
__device__ __forceinline__ void pipe_finish(const Pipe& p, uint32_t tmem_all, uint32_t ncol_all) {
  if (!p.ok) tc::mbar_wait(p.bar, p.phase ^ 1u);
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  if (threadIdx.x < 32) tc::tmem_free(tmem_all, ncol_all);
}

// Prologue: tensor memory (NCOLS columns per pipeline), barriers, the pipeline of this thread; NP pipelines per CTA.
#define PIPE_PROLOGUE(NCOLS, NP)                                                         \
  __shared__ uint64_t bars[3];                                                           \
  __shared__ uint32_t tslot;                                                             \
  constexpr uint32_t NCOL = tmem_cols(NCOLS);                                            \
  static_assert((NP) * NCOL <= 512, "accumulators exceed tensor memory");                \
  const int tid = threadIdx.x;                                                           \
  if (tid < 32) tc::tmem_alloc(&tslot, (NP) * NCOL);                                     \
  if (tid == 0) {                                                                        \
    for (int i = 0; i < 3; ++i) tc::mbar_init(&bars[i], 1);                              \
    tc::mbar_init_fence();                                                               \
  }                                                                                      \
  tc::tc_before_sync();                                                                  \
  __syncthreads();                                                                       \
  tc::tc_after_sync();                                                                   \
  const int pid = tid / PT;                                                              \
  Pipe P{&bars[1 + pid], 0u, true, pid, tid % PT, tid & 31, (tid >> 5) & 3, (tid % PT) / 128, \
         tslot + (uint32_t)pid * NCOL, (uint32_t)(32 * ((tid >> 5) & 3)) << 16};          \
  Ctx wcx{&bars[0], 0u, true};                                                           \
  const long nt = (V + TM - 1) / TM;                                                     \
  const long tstep = (long)(NP) * gridDim.x;                                             \
  const long t0 = (long)(NP) * blockIdx.x + pid;

// ============================================================================================== forward
// 2-layer MLP C -> 2C -> C with the residual prologue of ffno_mlp2_fwd and GroupNorm partials of the output.
// Weights: [w1 (2C x C), w2 (C x 2C)]. Per pipeline: the input tile, then (aliased) the hidden tile.
template <int C, int MODE>
__global__ void __launch_bounds__(CT, 1) k_mlp2_tc(const float* __restrict__ in, const float* __restrict__ prev,
                                                   const float* __restrict__ pc, float res, float* __restrict__ xout,
                                                   long V, const uint8_t* __restrict__ wpack,
                                                   const float* __restrict__ dw, float* __restrict__ pre,
                                                   double* __restrict__ partials, int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(2 * C, C), B2 = mat_bytes(C, 2 * C), RB = tile_bytes(2 * C);
  __shared__ float wt[2][TM], wpart[2][4], red[2][4 * GMAX];
  __shared__ double acc[2 * GMAX * 3];
  PIPE_PROLOGUE(TM, 2)
  uint8_t* region = smem + B1 + B2 + pid * RB;
  const Split X = split_at(region, TM, C), H = split_at(region, TM, 2 * C);
  if (tid < 2 * GMAX * 3) acc[tid] = 0.0;
  P.ok = load_weights(smem, wpack, B1 + B2, wcx, err);
  const Op w1 = wop(smem, 2 * C, C), w2 = wop(smem + B1, C, 2 * C);
  Gn4 gc{};
  if (MODE != 0) gc = gn_coefs(pc, C, fill_col<C>(P.ptid));
  const int f = P.feat();
  const int pf = c_pf;
  for (int k = 1; P.ptid == 0 && k < pf; ++k) {
    const long tp = t0 + k * tstep;
    prefetch_rows(in, tp * TM, V, C);
    if (MODE != 0) prefetch_rows(prev, tp * TM, V, C);
  }
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (P.ptid == 0 && pf > 0) {
      const long tp = t + pf * tstep;
      prefetch_rows(in, tp * TM, V, C);
      if (MODE != 0) prefetch_rows(prev, tp * TM, V, C);
    }
    load_tile_weights(P, dw, v0, V, wt[pid], wpart[pid]);
    fill_tile<C>(X, v0, V, P.ptid, [&](long v, int k) {
      float4 a = ld4(in + v * C + k);
      if (MODE != 0) {
        const float4 y = gn_apply<MODE == 1>(ld4(prev + v * C + k), gc);
        a = make_float4(fmaf(res, y.x, a.x), fmaf(res, y.y, a.y), fmaf(res, y.z, a.z), fmaf(res, y.w, a.w));
        *reinterpret_cast<float4*>(xout + v * C + k) = a;
      }
      return a;
    });
    if (!pipe_gemms(P, err, Gemm{P.tmem, w1, kop(X, C), C, false})) break;
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
      float v[16];
      tld(P, 0, c, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = gelu_tc(v[i]);
      if (f < 2 * C) put_mn(H, f, 64 * P.half + 16 * c, v);
    }
    if (!pipe_gemms(P, err, Gemm{P.tmem, w2, mop(H), 2 * C, false})) break;
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
      float v[16];
      tld(P, 0, c, v);
      const long vb = v0 + 64 * P.half + 16 * c;
      if (f < C)
#pragma unroll
        for (int i = 0; i < 16; ++i)
          if (vb + i < V) pre[(vb + i) * C + f] = v[i];
    }
    tile_stats<C>(P, 0, wt[pid], wpart[pid], red[pid], acc + pid * GMAX * 3);
  }
  write_partial2(partials, acc);
  pipe_finish(P, tslot, 2 * NCOL);
}

// Input gate of one branch: out = x sigmoid(gelu(x G1) G2) [+ zp z]. Weights: [g1 (C x C), g2 (C x C)]. Both GEMMs
// have C outputs and run untransposed (lane = voxel).
template <int C>
__global__ void __launch_bounds__(CT, 1) k_gate_tc(const float* __restrict__ x, long V, const uint8_t* __restrict__ wpack,
                                                   const float* __restrict__ zp, const float* __restrict__ z,
                                                   float* __restrict__ out, int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(C, C), RB = tile_bytes(C);
  PIPE_PROLOGUE(C, 2)
  const Split X = split_at(smem + 2 * B1 + pid * RB, TM, C);
  P.ok = load_weights(smem, wpack, 2 * B1, wcx, err);
  const Op g1 = wop(smem, C, C), g2 = wop(smem + B1, C, C);
  const int row = P.feat();
  const int pf = c_pf;
  for (int k = 1; P.ptid == 0 && k < pf; ++k) {
    const long tp = t0 + k * tstep;
    prefetch_rows(x, tp * TM, V, C);
  }
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (P.ptid == 0 && pf > 0) {
      const long tp = t + pf * tstep;
      prefetch_rows(x, tp * TM, V, C);
    }
    fill_rows<C>(X, v0, V, P.ptid, x);
    if (!pipe_gemms(P, err, Gemm{P.tmem, kop(X, C), g1, C, false, C})) break;
#pragma unroll
    for (int j = 0; j < C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      float v[16];
      rld(P, 0, j, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = gelu_tc(v[i]);
      put16(X, row, 16 * j, C, v);
    }
    if (!pipe_gemms(P, err, Gemm{P.tmem, kop(X, C), g2, C, false, C})) break;
    const long v = v0 + row;
    const float zv = (zp && v < V) ? __ldg(z + v) : 0.f;
#pragma unroll
    for (int j = 0; j < C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      const int c0 = 16 * j;
      float g[16];
      rld(P, 0, j, g);
      if (v < V) {
#pragma unroll
        for (int i = 0; i < 16; i += 4) {
          const float4 xv = ld4(x + v * C + c0 + i);
          float4 o = make_float4(xv.x * sigmoid_tc(g[i]), xv.y * sigmoid_tc(g[i + 1]), xv.z * sigmoid_tc(g[i + 2]),
                                 xv.w * sigmoid_tc(g[i + 3]));
          if (zp) {
            const float4 zz = ld4(zp + c0 + i);
            o = make_float4(fmaf(zz.x, zv, o.x), fmaf(zz.y, zv, o.y), fmaf(zz.z, zv, o.z), fmaf(zz.w, zv, o.w));
          }
          *reinterpret_cast<float4*>(out + v * C + c0 + i) = o;
        }
      }
    }
  }
  pipe_finish(P, tslot, 2 * NCOL);
}

// Branch gates (first half of _fuse_branches): gates = sigmoid(gelu([x, spec, vert] Wg1) Wg2 + b), spec =
// gelu(GN(spec_pre)) etc.; optionally the hidden pre-activation [x, spec, vert] Wg1 to hg. Weights: [wg1 (C x 3C),
// wg2 (2C x C)]. The first GEMM (C outputs, untransposed) runs over three K-slices of C columns (x, spec, vert) through
// one tile per pipeline; the second (2C outputs) is transposed.
template <int C>
__global__ void __launch_bounds__(CT, 1) k_fuse1_tc(const float* __restrict__ x, const float* __restrict__ sp,
                                                    const float* __restrict__ sc, const float* __restrict__ vp,
                                                    const float* __restrict__ vc, long V,
                                                    const uint8_t* __restrict__ wpack, const float* __restrict__ bias,
                                                    float* __restrict__ gates, float* __restrict__ hg,
                                                    int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(C, 3 * C), B2 = mat_bytes(2 * C, C), RB = tile_bytes(C);
  PIPE_PROLOGUE(TM, 2)
  const Split A = split_at(smem + B1 + B2 + pid * RB, TM, C);
  P.ok = load_weights(smem, wpack, B1 + B2, wcx, err);
  const Op wg2 = wop(smem + B1, 2 * C, C);
  const int kf = fill_col<C>(P.ptid);
  const Gn4 gs = gn_coefs(sc, C, kf), gv = gn_coefs(vc, C, kf);
  const int f = P.feat();
  const float bf = f < 2 * C ? __ldg(bias + f) : 0.f;
  const int pf = c_pf;
  for (int k = 1; P.ptid == 0 && k < pf; ++k) {
    const long tp = t0 + k * tstep;
    prefetch_rows(x, tp * TM, V, C);
    prefetch_rows(sp, tp * TM, V, C);
    prefetch_rows(vp, tp * TM, V, C);
  }
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (P.ptid == 0 && pf > 0) {
      const long tp = t + pf * tstep;
      prefetch_rows(x, tp * TM, V, C);
      prefetch_rows(sp, tp * TM, V, C);
      prefetch_rows(vp, tp * TM, V, C);
    }
    for (int kc = 0; kc < 3; ++kc) {
      if (kc == 0)
        fill_tile<C>(A, v0, V, P.ptid, [&](long v, int k) { return ld4(x + v * C + k); });
      else if (kc == 1)
        fill_tile<C>(A, v0, V, P.ptid, [&](long v, int k) { return gn_apply<true>(ld4(sp + v * C + k), gs); });
      else
        fill_tile<C>(A, v0, V, P.ptid, [&](long v, int k) { return gn_apply<true>(ld4(vp + v * C + k), gv); });
      if (!pipe_gemms(P, err, Gemm{P.tmem, kop(A, C), wop(smem, C, 3 * C, 0, kc * C), C, kc > 0, C})) break;
    }
    if (!P.ok) break;
    const long v = v0 + f;
#pragma unroll
    for (int j = 0; j < C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      const int c0 = 16 * j;
      float h[16];
      rld(P, 0, j, h);
      if (hg && v < V)
#pragma unroll
        for (int i = 0; i < 16; i += 4)
          *reinterpret_cast<float4*>(hg + v * C + c0 + i) = make_float4(h[i], h[i + 1], h[i + 2], h[i + 3]);
#pragma unroll
      for (int i = 0; i < 16; ++i) h[i] = gelu_tc(h[i]);
      put16(A, f, c0, C, h);
    }
    if (!pipe_gemms(P, err, Gemm{P.tmem, wg2, kop(A, C), C, false})) break;
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
      float g[16];
      tld(P, 0, c, g);
      const long vb = v0 + 64 * P.half + 16 * c;
      if (f < 2 * C)
#pragma unroll
        for (int i = 0; i < 16; ++i)
          if (vb + i < V) gates[(vb + i) * 2 * C + f] = sigmoid_tc(g[i] + bf);
    }
  }
  pipe_finish(P, tslot, 2 * NCOL);
}

// Fuse (second half of _fuse_branches): B = [spec gs, vert gv], pre = gelu(B Wf1) Wf2 + (spec gs + vert gv) / 2, with
// the GroupNorm partials of pre. Weights: [wf1 (2C x 2C), wf2 (C x 2C)]. The residual (spec gs + vert gv) / 2 is read
// from the split B tile (hi + lo) into the second accumulator before the hidden layer overwrites the tile, and GEMM2
// adds onto it, so pre is never recomputed from HBM.
__device__ __forceinline__ float bf16_at(const uint8_t* p) {
  return __uint_as_float((uint32_t)(*reinterpret_cast<const uint16_t*>(p)) << 16);
}

template <int C>
__global__ void __launch_bounds__(CT, 1) k_fuse2_tc(const float* __restrict__ sp, const float* __restrict__ sc,
                                                    const float* __restrict__ vp, const float* __restrict__ vc,
                                                    const float* __restrict__ gates, long V,
                                                    const uint8_t* __restrict__ wpack, const float* __restrict__ dw,
                                                    float* __restrict__ pre, double* __restrict__ partials,
                                                    int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(2 * C, 2 * C), B2 = mat_bytes(C, 2 * C), RB = tile_bytes(2 * C);
  __shared__ float wt[2][TM], wpart[2][4], red[2][4 * GMAX];
  __shared__ double acc[2 * GMAX * 3];
  PIPE_PROLOGUE(2 * TM, 2)
  const Split A = split_at(smem + B1 + B2 + pid * RB, TM, 2 * C);
  if (tid < 2 * GMAX * 3) acc[tid] = 0.0;
  P.ok = load_weights(smem, wpack, B1 + B2, wcx, err);
  const Op wf1 = wop(smem, 2 * C, 2 * C), wf2 = wop(smem + B1, C, 2 * C);
  const int kf = fill_col8<2 * C>(P.ptid);
  const float* cfk = kf < C ? sc : vc;
  const int ks = kf < C ? kf : kf - C;
  const Gn4 gk0 = gn_coefs(cfk, C, ks), gk1 = gn_coefs(cfk, C, ks + 4);
  const float* src = kf < C ? sp : vp;
  const int f = P.feat();
  const int pf = c_pf;
  for (int k = 1; P.ptid == 0 && k < pf; ++k) {
    const long tp = t0 + k * tstep;
    prefetch_rows(sp, tp * TM, V, C);
    prefetch_rows(vp, tp * TM, V, C);
    prefetch_rows(gates, tp * TM, V, 2 * C);
  }
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (P.ptid == 0 && pf > 0) {
      const long tp = t + pf * tstep;
      prefetch_rows(sp, tp * TM, V, C);
      prefetch_rows(vp, tp * TM, V, C);
      prefetch_rows(gates, tp * TM, V, 2 * C);
    }
    load_tile_weights(P, dw, v0, V, wt[pid], wpart[pid]);
    fill_tile8<2 * C>(A, v0, V, P.ptid, [&](long v, int k, float (&o)[8]) {
      float g[8], p[8];
      ld8(gates + v * 2 * C + k, g);
      ld8(src + v * C + ks, p);
      const float4 s0 = gn_apply<true>(make_float4(p[0], p[1], p[2], p[3]), gk0);
      const float4 s1 = gn_apply<true>(make_float4(p[4], p[5], p[6], p[7]), gk1);
      o[0] = s0.x * g[0], o[1] = s0.y * g[1], o[2] = s0.z * g[2], o[3] = s0.w * g[3];
      o[4] = s1.x * g[4], o[5] = s1.y * g[5], o[6] = s1.z * g[6], o[7] = s1.w * g[7];
    });
    if (!pipe_gemms(P, err, Gemm{P.tmem, wf1, kop(A, 2 * C), 2 * C, false})) break;
    if (32 * P.q < C) {   // warps holding output channels: the residual of their lanes, columns of their half
#pragma unroll 1
      for (int c = 0; c < 4; ++c) {
        const int vl0 = 64 * P.half + 16 * c;
        float r[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          float x = 0.f;
          if (f < C) {
            const uint32_t os = tc::kmajor_offset(vl0 + i, f, 2 * C), ov = tc::kmajor_offset(vl0 + i, C + f, 2 * C);
            x = 0.5f * ((bf16_at(A.hi() + os) + bf16_at(A.lo() + os)) + (bf16_at(A.hi() + ov) + bf16_at(A.lo() + ov)));
          }
          r[i] = x;
        }
        tc::tmem_st16(P.tmem + P.lq + TM + (uint32_t)vl0, r);
      }
    }
    pipe_sync(P.id);   // the tile is read; the hidden layer may overwrite it
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
      float h[16];
      tld(P, 0, c, h);
#pragma unroll
      for (int i = 0; i < 16; ++i) h[i] = gelu_tc(h[i]);
      if (f < 2 * C) put_mn(A, f, 64 * P.half + 16 * c, h);
    }
    if (!pipe_gemms(P, err, Gemm{P.tmem + TM, wf2, mop(A), 2 * C, true})) break;
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
      float o[16];
      tld(P, TM, c, o);
      const long vb = v0 + 64 * P.half + 16 * c;
      if (f < C)
#pragma unroll
        for (int i = 0; i < 16; ++i)
          if (vb + i < V) pre[(vb + i) * C + f] = o[i];
    }
    tile_stats<C>(P, TM, wt[pid], wpart[pid], red[pid], acc + pid * GMAX * 3);
  }
  write_partial2(partials, acc);
  pipe_finish(P, tslot, 2 * NCOL);
}

// ============================================================================================== backward
// a_bar = base + ((pre_bar W2^T) * gelu'(a W1)) W1^T. Weights: [w1 (2C x C), w2t (2C x C), w1t (C x 2C)].
// Per pipeline: the tiles of a and pre_bar, then (aliased) the hidden tile; the last GEMM (C outputs) untransposed.
template <int C>
__global__ void __launch_bounds__(CT, 1) k_mlp2_bwd_tc(const float* __restrict__ a, const float* __restrict__ pb,
                                                       const float* __restrict__ base, long V,
                                                       const uint8_t* __restrict__ wpack, float* __restrict__ abar,
                                                       int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(2 * C, C), RB = tile_bytes(2 * C);
  PIPE_PROLOGUE(2 * TM, 2)
  uint8_t* region = smem + 3 * B1 + pid * RB;
  const Split A = split_at(region, TM, C), Pt = split_at(region + tile_bytes(C), TM, C),
              H = split_at(region, TM, 2 * C);
  P.ok = load_weights(smem, wpack, 3 * B1, wcx, err);
  const Op w1 = wop(smem, 2 * C, C), w2t = wop(smem + B1, 2 * C, C), w1t = wop(smem + 2 * B1, C, 2 * C);
  const int f = P.feat();
  const int pf = c_pf;
  for (int k = 1; P.ptid == 0 && k < pf; ++k) {
    const long tp = t0 + k * tstep;
    prefetch_rows(a, tp * TM, V, C);
    prefetch_rows(pb, tp * TM, V, C);
    prefetch_rows(base, tp * TM, V, C);
  }
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (P.ptid == 0 && pf > 0) {
      const long tp = t + pf * tstep;
      prefetch_rows(a, tp * TM, V, C);
      prefetch_rows(pb, tp * TM, V, C);
      prefetch_rows(base, tp * TM, V, C);
    }
    fill_tile<C>(A, v0, V, P.ptid, [&](long v, int k) { return ld4(a + v * C + k); });
    fill_tile<C>(Pt, v0, V, P.ptid, [&](long v, int k) { return ld4(pb + v * C + k); });
    const Gemm g2{P.tmem + TM, w2t, kop(Pt, C), C, false};
    if (!pipe_gemms(P, err, Gemm{P.tmem, w1, kop(A, C), C, false}, &g2)) break;
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
      float hp[16], gb[16];
      tld(P, 0, c, hp);
      tld(P, TM, c, gb);
#pragma unroll
      for (int i = 0; i < 16; ++i) gb[i] *= gelu_grad_tc(hp[i]);
      if (f < 2 * C) put_mn(H, f, 64 * P.half + 16 * c, gb);
    }
    if (!pipe_gemms(P, err, Gemm{P.tmem, mop(H), w1t, 2 * C, false, C})) break;
    const long v = v0 + f;
#pragma unroll
    for (int j = 0; j < C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      const int c0 = 16 * j;
      float r[16];
      rld(P, 0, j, r);
      if (v < V)
#pragma unroll
        for (int i = 0; i < 16; i += 4) {
          float4 o = make_float4(r[i], r[i + 1], r[i + 2], r[i + 3]);
          if (base) {
            const float4 b = ld4(base + v * C + c0 + i);
            o = make_float4(o.x + b.x, o.y + b.y, o.z + b.z, o.w + b.w);
          }
          *reinterpret_cast<float4*>(abar + v * C + c0 + i) = o;
        }
    }
  }
  pipe_finish(P, tslot, 2 * NCOL);
}

// One input gate's backward: x_bar = base + d/dx [x sigmoid(gelu(x G1) G2)] applied to gbar; with zp, z_bar[v] +=
// sum_c gbar zp. Weights: [g1, g2, g2t, g1t] (each C x C). All four GEMMs have C outputs and run untransposed.
// At C = 96 (one pipeline a CTA: tensor memory holds 4C columns) the pack is [g1, g2] and the transposes are read out
// of it as MN-major operands.
template <int C, int NP = 2>
__global__ void __launch_bounds__(NP * PT, 1) k_gate_bwd_tc(const float* __restrict__ x, const float* __restrict__ gbar,
                                                            const float* __restrict__ base, long V,
                                                            const uint8_t* __restrict__ wpack,
                                                            const float* __restrict__ zp, float* __restrict__ xbar,
                                                            float* __restrict__ zbar, int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr bool TW = C == 96;                   // transposes from the forward's matrices
  constexpr uint32_t B1 = mat_bytes(C, C), RB = 2 * tile_bytes(C), WB = (TW ? 2 : 4) * B1;
  __shared__ float zsh[NP][TM];
  PIPE_PROLOGUE(4 * C, NP)
  const Split X = split_at(smem + WB + pid * RB, TM, C), T = split_at(smem + WB + pid * RB + tile_bytes(C), TM, C);
  P.ok = load_weights(smem, wpack, WB, wcx, err);
  const Op g1 = wop(smem, C, C), g2 = wop(smem + B1, C, C);
  const Op g2t = TW ? wop_t(smem + B1, C, C) : wop(smem + 2 * B1, C, C);
  const Op g1t = TW ? wop_t(smem, C, C) : wop(smem + 3 * B1, C, C);
  const uint32_t D1 = 0, D2 = C, D3 = 2 * C, D4 = 3 * C;
  const int row = P.feat();
  const int pf = c_pf;
  for (int k = 1; P.ptid == 0 && k < pf; ++k) {
    const long tp = t0 + k * tstep;
    prefetch_rows(x, tp * TM, V, C);
    prefetch_rows(gbar, tp * TM, V, C);
    prefetch_rows(base, tp * TM, V, C);
  }
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (P.ptid == 0 && pf > 0) {
      const long tp = t + pf * tstep;
      prefetch_rows(x, tp * TM, V, C);
      prefetch_rows(gbar, tp * TM, V, C);
      prefetch_rows(base, tp * TM, V, C);
    }
    const long v = v0 + row;
    fill_rows<C>(X, v0, V, P.ptid, x);
    if (!pipe_gemms(P, err, Gemm{P.tmem + D1, kop(X, C), g1, C, false, C})) break;
#pragma unroll
    for (int j = 0; j < C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      float h[16];
      rld(P, D1, j, h);
#pragma unroll
      for (int i = 0; i < 16; ++i) h[i] = gelu_tc(h[i]);
      put16(T, row, 16 * j, C, h);
    }
    if (!pipe_gemms(P, err, Gemm{P.tmem + D2, kop(T, C), g2, C, false, C})) break;
    float zs = 0.f;
#pragma unroll
    for (int j = 0; j < C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      const int c0 = 16 * j;
      float g[16], q[16], o[16];
      rld(P, D2, j, g);
#pragma unroll
      for (int i = 0; i < 16; ++i) q[i] = o[i] = 0.f;
      if (v < V) {
#pragma unroll
        for (int i = 0; i < 16; i += 4) {
          const float4 b = ld4(gbar + v * C + c0 + i), xv = ld4(x + v * C + c0 + i);
          const float4 bs = base ? ld4(base + v * C + c0 + i) : make_float4(0.f, 0.f, 0.f, 0.f);
          const float bb[4] = {b.x, b.y, b.z, b.w}, xx[4] = {xv.x, xv.y, xv.z, xv.w}, ba[4] = {bs.x, bs.y, bs.z, bs.w};
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const float s = sigmoid_tc(g[i + u]);
            o[i + u] = fmaf(bb[u], s, ba[u]);
            q[i + u] = bb[u] * xx[u] * s * (1.f - s);
            if (zp) zs = fmaf(bb[u], __ldg(zp + c0 + i + u), zs);
          }
        }
      }
      // base + gbar s into the last GEMM's accumulator, which adds the gate-path gradient onto it
      tc::tmem_st16(P.tmem + P.lq + D4 + (uint32_t)c0, o);
      put16(T, row, c0, C, q);
    }
    if (zp) {   // the two halves of the row add their parts of z_bar in a fixed order
      if (P.half == 1) zsh[pid][row] = zs;
      pipe_sync(P.id);
      if (P.half == 0 && v < V) zbar[v] += zs + zsh[pid][row];
    }
    if (!pipe_gemms(P, err, Gemm{P.tmem + D3, kop(T, C), g2t, C, false, C})) break;
#pragma unroll
    for (int j = 0; j < C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      float hb[16], hp[16];
      rld(P, D3, j, hb);
      rld(P, D1, j, hp);
#pragma unroll
      for (int i = 0; i < 16; ++i) hb[i] *= gelu_grad_tc(hp[i]);
      put16(T, row, 16 * j, C, hb);
    }
    if (!pipe_gemms(P, err, Gemm{P.tmem + D4, kop(T, C), g1t, C, true, C})) break;
#pragma unroll
    for (int j = 0; j < C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      const int c0 = 16 * j;
      float r[16];
      rld(P, D4, j, r);
      if (v < V)
#pragma unroll
        for (int i = 0; i < 16; i += 4)
          *reinterpret_cast<float4*>(xbar + v * C + c0 + i) = make_float4(r[i], r[i + 1], r[i + 2], r[i + 3]);
    }
  }
  pipe_finish(P, tslot, NP * NCOL);
}

// Fuse backward, stage a: hf_bar_pre = (F_bar Wf2^T) * gelu'(B Wf1) with B = [spec gs, vert gv], F_bar =
// fused_pre_bar. Weights: [wf1 (2C x 2C), wf2t (2C x C)]. Per pipeline one tile: B, then (after its GEMM) F_bar.
template <int C>
__global__ void __launch_bounds__(CT, 1) k_fuse_bwd_a_tc(const float* __restrict__ sp, const float* __restrict__ sc,
                                                         const float* __restrict__ vp, const float* __restrict__ vc,
                                                         const float* __restrict__ gates, const float* __restrict__ fb,
                                                         long V, const uint8_t* __restrict__ wpack,
                                                         float* __restrict__ hfb, int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(2 * C, 2 * C), B2 = mat_bytes(2 * C, C), RB = tile_bytes(2 * C);
  PIPE_PROLOGUE(2 * TM, 2)
  const Split Bt = split_at(smem + B1 + B2 + pid * RB, TM, 2 * C), Ft = split_at(smem + B1 + B2 + pid * RB, TM, C);
  P.ok = load_weights(smem, wpack, B1 + B2, wcx, err);
  const Op wf1 = wop(smem, 2 * C, 2 * C), wf2t = wop(smem + B1, 2 * C, C);
  const int kf = fill_col8<2 * C>(P.ptid);
  const float* cfk = kf < C ? sc : vc;
  const int ks = kf < C ? kf : kf - C;
  const Gn4 gk0 = gn_coefs(cfk, C, ks), gk1 = gn_coefs(cfk, C, ks + 4);
  const float* src = kf < C ? sp : vp;
  const int f = P.feat();
  // L2 prefetch: the first phase's rows (spec, vert, gates) one tile ahead, F_bar (read after the first GEMM) at
  // the start of its own tile, so that no prefetched line has to outlive a whole tile step of all pipelines
  const int pf = c_pf;
  if (P.ptid == 0 && pf > 0) {
    prefetch_rows(sp, t0 * TM, V, C);
    prefetch_rows(vp, t0 * TM, V, C);
    prefetch_rows(gates, t0 * TM, V, 2 * C);
  }
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (P.ptid == 0 && pf > 0) {
      prefetch_rows(fb, v0, V, C);
      const long tn = (t + tstep) * TM;
      prefetch_rows(sp, tn, V, C);
      prefetch_rows(vp, tn, V, C);
      prefetch_rows(gates, tn, V, 2 * C);
    }
    fill_tile8<2 * C>(Bt, v0, V, P.ptid, [&](long v, int k, float (&o)[8]) {
      float g[8], p[8];
      ld8(gates + v * 2 * C + k, g);
      ld8(src + v * C + ks, p);
      const float4 s0 = gn_apply<true>(make_float4(p[0], p[1], p[2], p[3]), gk0);
      const float4 s1 = gn_apply<true>(make_float4(p[4], p[5], p[6], p[7]), gk1);
      o[0] = s0.x * g[0], o[1] = s0.y * g[1], o[2] = s0.z * g[2], o[3] = s0.w * g[3];
      o[4] = s1.x * g[4], o[5] = s1.y * g[5], o[6] = s1.z * g[6], o[7] = s1.w * g[7];
    });
    if (!pipe_gemms(P, err, Gemm{P.tmem, wf1, kop(Bt, 2 * C), 2 * C, false})) break;
    fill_tile8<C>(Ft, v0, V, P.ptid, [&](long v, int k, float (&o)[8]) { ld8(fb + v * C + k, o); });
    if (!pipe_gemms(P, err, Gemm{P.tmem + TM, wf2t, kop(Ft, C), C, false})) break;
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
      float hp[16], hb[16];
      tld(P, 0, c, hp);
      tld(P, TM, c, hb);
      const long vb = v0 + 64 * P.half + 16 * c;
      if (f < 2 * C)
#pragma unroll
        for (int i = 0; i < 16; ++i)
          if (vb + i < V) hfb[(vb + i) * 2 * C + f] = hb[i] * gelu_grad_tc(hp[i]);
    }
  }
  pipe_finish(P, tslot, 2 * NCOL);
}

// Fuse backward, stage b: B_bar = hfb Wf1^T + [F_bar, F_bar] / 2; spec/vert grads B_bar g (+ the gate path, added by
// the last GEMM onto the direct gradients kept in tensor memory, so each branch gradient is written once);
// gate pre-activation grad q = B_bar [spec, vert] g (1 - g); hg_bar = (q Wg2^T) * gelu'(hg); A_bar = hg_bar Wg1^T:
// x_bar = base + A_bar[:C], spec_bar = B_bar_s g_s + A_bar[C:2C], vert_bar likewise.
// Weights: [wf1t (2C x 2C), wg2t (C x 2C), wg1t (3C x C)]. All three GEMMs run untransposed (lane = voxel; the
// epilogues read and write several tensors per voxel). Each of the two pipelines has one [128][C] operand tile, so the
// K = 2C products run as two K-slices: hfb's spec and vert halves, then q's spec and vert halves (each slice's
// epilogue fills the tile while the other pipeline's MMAs run).
template <int C>
__global__ void __launch_bounds__(CT, 1) k_fuse_bwd_b_tc(const float* __restrict__ sp, const float* __restrict__ sc,
                                                         const float* __restrict__ vp, const float* __restrict__ vc,
                                                         const float* __restrict__ gates, const float* __restrict__ hg,
                                                         const float* __restrict__ fb, const float* __restrict__ hfb,
                                                         const float* __restrict__ base, long V,
                                                         const uint8_t* __restrict__ wpack, float* __restrict__ xbar,
                                                         float* __restrict__ sbar, float* __restrict__ vbar,
                                                         int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(2 * C, 2 * C), B2 = mat_bytes(C, 2 * C), B3 = mat_bytes(3 * C, C),
                     RB = tile_bytes(C);
  PIPE_PROLOGUE(3 * C, 2)
  const Split T = split_at(smem + B1 + B2 + B3 + pid * RB, TM, C);
  P.ok = load_weights(smem, wpack, B1 + B2 + B3, wcx, err);
  const int row = P.feat();
  // L2 prefetch: hfb (the first phase's operand) one tile ahead; the rows the later phases read (F_bar, gates, both
  // pre-activations, hg, base) at the start of their own tile, while the first GEMMs run, so that no prefetched line
  // has to outlive a whole tile step of all pipelines (one tile step reads 9 C floats a voxel: ~90 MB at C = 64)
  const int pf = c_pf;
  if (P.ptid == 0 && pf > 0) prefetch_rows(hfb, t0 * TM, V, 2 * C);
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (P.ptid == 0 && pf > 0) {
      prefetch_rows(fb, v0, V, C);
      prefetch_rows(gates, v0, V, 2 * C);
      prefetch_rows(sp, v0, V, C);
      prefetch_rows(vp, v0, V, C);
      prefetch_rows(hg, v0, V, C);
      prefetch_rows(base, v0, V, C);
      prefetch_rows(hfb, (t + tstep) * TM, V, 2 * C);
    }
    const long v = v0 + row;
    // B_bar (without the F_bar term) = hfb Wf1^T over the spec and vert halves of hfb
    for (int kh = 0; kh < 2; ++kh) {
      fill_tile8<C>(T, v0, V, P.ptid, [&](long vv, int k, float (&o)[8]) { ld8(hfb + vv * 2 * C + kh * C + k, o); });
      if (!pipe_gemms(P, err, Gemm{P.tmem, kop(T, C), wop(smem, 2 * C, 2 * C, 0, kh * C), C, kh > 0, 2 * C})) break;
    }
    if (!P.ok) break;
    // per branch half: the direct spec/vert gradients, q, and its slice of q Wg2^T
    for (int kh = 0; kh < 2; ++kh) {
      const float* pre = kh == 0 ? sp : vp;
      const float* cf = kh == 0 ? sc : vc;
#pragma unroll 1
      for (int jj = 0; jj < C / 16; ++jj) {
        const int j = kh * (C / 16) + jj;
        if (!owns(j, P.half)) continue;
        const int cc = 16 * jj;
        float bb[16], q[16], od[16];
        rld(P, 0, j, bb);
#pragma unroll
        for (int i = 0; i < 16; ++i) q[i] = od[i] = 0.f;
        if (v < V) {
#pragma unroll
          for (int i = 0; i < 16; i += 8) {
            float ff[8], gg[8], pp[8];
            ld8(fb + v * C + cc + i, ff);
            ld8(gates + v * 2 * C + kh * C + cc + i, gg);
            ld8(pre + v * C + cc + i, pp);
#pragma unroll
            for (int h = 0; h < 8; h += 4) {
              const float4 s4 = gn_apply<true>(make_float4(pp[h], pp[h + 1], pp[h + 2], pp[h + 3]),
                                               gn_coefs(cf, C, cc + i + h));
              const float ss[4] = {s4.x, s4.y, s4.z, s4.w};
#pragma unroll
              for (int u = 0; u < 4; ++u) {
                const float b = bb[i + h + u] + 0.5f * ff[h + u];
                od[i + h + u] = b * gg[h + u];
                q[i + h + u] = b * ss[u] * gg[h + u] * (1.f - gg[h + u]);
              }
            }
          }
        }
        // the direct branch gradient replaces B_bar in its own accumulator columns; GEMM3 adds A_bar onto it
        tc::tmem_st16(P.tmem + P.lq + (uint32_t)(16 * j), od);
        put16(T, row, cc, C, q);
      }
      if (!pipe_gemms(P, err, Gemm{P.tmem + 2 * C, kop(T, C), wop(smem + B1, C, 2 * C, 0, kh * C), C, kh > 0, C}))
        break;
    }
    if (!P.ok) break;
#pragma unroll
    for (int j = 0; j < C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      const int c0 = 16 * j;
      float hb[16], h8[16];
      rld(P, 2 * C, j, hb);
      if (v < V) {
        ld8(hg + v * C + c0, *reinterpret_cast<float(*)[8]>(h8));
        ld8(hg + v * C + c0 + 8, *reinterpret_cast<float(*)[8]>(h8 + 8));
      } else {
#pragma unroll
        for (int i = 0; i < 16; ++i) h8[i] = 0.f;
      }
#pragma unroll
      for (int i = 0; i < 16; ++i) hb[i] *= gelu_grad_tc(h8[i]);
      put16(T, row, c0, C, hb);
    }
    // GEMM3: the branch rows of Wg1 accumulate onto the direct gradients (columns 0 .. 2C), the x rows go to the
    // columns GEMM2 used (2C .. 3C)
    const Gemm g3x{P.tmem + 2 * C, kop(T, C), wop(smem + B1 + B2, 3 * C, C, 0), C, false, C};
    if (!pipe_gemms(P, err, Gemm{P.tmem, kop(T, C), wop(smem + B1 + B2, 3 * C, C, C), C, true, 2 * C}, &g3x)) break;
#pragma unroll
    for (int j = 0; j < (3 * C) / 16; ++j) {
      if (!owns(j, P.half)) continue;
      float r[16];
      if (j < 2 * C / 16) {   // spec_bar / vert_bar, written once
        rld(P, 0, j, r);
        float* g = j < C / 16 ? sbar : vbar;
        const int cc = 16 * (j % (C / 16));
        if (v < V) {
          st8(g + v * C + cc, r);
          st8(g + v * C + cc + 8, r + 8);
        }
      } else {                // x_bar = base + A_bar[:C]
        const int c0 = 16 * (j - 2 * C / 16);
        rld(P, 2 * C, j - 2 * C / 16, r);
        if (v < V) {
          if (base) {
            float b8[16];
            ld8(base + v * C + c0, *reinterpret_cast<float(*)[8]>(b8));
            ld8(base + v * C + c0 + 8, *reinterpret_cast<float(*)[8]>(b8 + 8));
#pragma unroll
            for (int i = 0; i < 16; ++i) r[i] += b8[i];
          }
          st8(xbar + v * C + c0, r);
          st8(xbar + v * C + c0 + 8, r + 8);
        }
      }
    }
  }
  pipe_finish(P, tslot, 2 * NCOL);
}

// ============================================================================================== head
// Level-fraction head (FFNO3D proj1 / proj2 and head_output, models/ffno_model.py:712-713, 729-748): o = gelu(x P1)
// P2 + b2 per voxel (P1: C -> 2C without bias, P2: 2C -> nh padded with zero rows to NHP), then the voxel's LTE
// log-softmax (head_voxel_fwd). The first GEMM runs transposed (2C outputs), the second untransposed (lane = voxel);
// the NHP head channels of a voxel reach the thread that owns it through shared memory, rows [128][NHP + 1] over the
// pipeline's tile region (the hidden tile has been consumed by then).
__host__ __device__ constexpr uint32_t head_rows_bytes(int NHP) { return (uint32_t)TM * (NHP + 1) * 4; }
__host__ __device__ constexpr uint32_t head_obar_at(int NHP) { return (head_rows_bytes(NHP) + 1023u) & ~1023u; }
__host__ __device__ constexpr uint32_t head_region(int C, int NHP, bool bwd) {
  const uint32_t need = bwd ? head_obar_at(NHP) + tile_bytes(NHP) : head_rows_bytes(NHP);
  return tile_bytes(2 * C) > need ? tile_bytes(2 * C) : need;
}

template <int C, int NHP, typename T>
__global__ void __launch_bounds__(CT, 1) k_head_tc(const float* __restrict__ x, const float* __restrict__ xin, long V,
                                                   const uint8_t* __restrict__ wpack, const float* __restrict__ b2,
                                                   int nh, const __grid_constant__ ffno_head_params hp,
                                                   float* __restrict__ out, float* __restrict__ head_out,
                                                   int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(2 * C, C), B2 = mat_bytes(NHP, 2 * C), RB = head_region(C, NHP, false);
  constexpr int LO = NHP + 1;
  PIPE_PROLOGUE(TM, 2)
  uint8_t* region = smem + B1 + B2 + pid * RB;
  const Split X = split_at(region, TM, C), H = split_at(region, TM, 2 * C);
  float* os = reinterpret_cast<float*>(region);
  P.ok = load_weights(smem, wpack, B1 + B2, wcx, err);
  const Op w1 = wop(smem, 2 * C, C), w2 = wop(smem + B1, NHP, 2 * C);
  const int f = P.feat();
  const int pf = c_pf;
  for (int k = 1; P.ptid == 0 && k < pf; ++k) prefetch_rows(x, (t0 + k * tstep) * TM, V, C);
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (P.ptid == 0 && pf > 0) prefetch_rows(x, (t + pf * tstep) * TM, V, C);
    fill_tile8<C>(X, v0, V, P.ptid, [&](long v, int k, float (&o)[8]) { ld8(x + v * C + k, o); });
    if (!pipe_gemms(P, err, Gemm{P.tmem, w1, kop(X, C), C, false})) break;
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
      float v[16];
      tld(P, 0, c, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = gelu_tc(v[i]);
      if (f < 2 * C) put_mn(H, f, 64 * P.half + 16 * c, v);
    }
    if (!pipe_gemms(P, err, Gemm{P.tmem, mop(H), w2, 2 * C, false, NHP})) break;
#pragma unroll
    for (int j = 0; j < NHP / 16; ++j) {
      if (!owns(j, P.half)) continue;
      float r[16];
      rld(P, 0, j, r);
#pragma unroll
      for (int i = 0; i < 16; ++i) os[f * LO + 16 * j + i] = r[i] + __ldg(b2 + 16 * j + i);
    }
    pipe_sync(P.id);
    const long v = v0 + f;
    if (P.half == 0 && v < V) {
      const float* o = os + f * LO;
      if (head_out)
        for (int c = 0; c < nh; ++c) head_out[(long)c * V + v] = o[c];
      head_voxel_fwd<T>(hp, o, head_inputs(hp, xin, V, v), out, V, v);
    }
    pipe_sync(P.id);   // the rows are read before the next tile's fill overwrites them
  }
  pipe_finish(P, tslot, 2 * NCOL);
}

// Head backward: the forward recomputed (pre = x P1 kept in tensor memory columns 0..127, o = gelu(pre) P2 + b2 at
// columns 128.. and then as shared rows), o_bar from head_voxel_bwd (which also writes x_in_bar) as a K-major tile,
// h_bar = (o_bar P2^T) * gelu'(pre) (transposed, columns 128..255), x_bar = h_bar P1^T (untransposed, columns 0..C-1).
// Weights: [w1 (2C x C), w2 (NHP x 2C), w2t (2C x NHP), w1t (C x 2C)]. The tile region holds in turn the input tile,
// the hidden tile, the head rows with the o_bar tile behind them, and the hidden-gradient tile.
template <int C, int NHP, typename T>
__global__ void __launch_bounds__(CT, 1) k_head_bwd_tc(const float* __restrict__ x, const float* __restrict__ xin,
                                                       const float* __restrict__ ybar, long V,
                                                       const uint8_t* __restrict__ wpack, const float* __restrict__ b2,
                                                       const __grid_constant__ ffno_head_params hp,
                                                       float* __restrict__ xbar, float* __restrict__ xinbar,
                                                       int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(2 * C, C), B2 = mat_bytes(NHP, 2 * C), RB = head_region(C, NHP, true);
  constexpr int LO = NHP + 1;
  PIPE_PROLOGUE(2 * TM, 2)
  uint8_t* region = smem + 2 * B1 + 2 * B2 + pid * RB;
  const Split X = split_at(region, TM, C), H = split_at(region, TM, 2 * C),
              Ob = split_at(region + head_obar_at(NHP), TM, NHP);
  float* os = reinterpret_cast<float*>(region);
  P.ok = load_weights(smem, wpack, 2 * B1 + 2 * B2, wcx, err);
  const Op w1 = wop(smem, 2 * C, C), w2 = wop(smem + B1, NHP, 2 * C), w2t = wop(smem + B1 + B2, 2 * C, NHP),
           w1t = wop(smem + B1 + 2 * B2, C, 2 * C);
  const int f = P.feat();
  const int pf = c_pf;
  for (int k = 1; P.ptid == 0 && k < pf; ++k) prefetch_rows(x, (t0 + k * tstep) * TM, V, C);
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (P.ptid == 0 && pf > 0) prefetch_rows(x, (t + pf * tstep) * TM, V, C);
    fill_tile8<C>(X, v0, V, P.ptid, [&](long v, int k, float (&o)[8]) { ld8(x + v * C + k, o); });
    if (!pipe_gemms(P, err, Gemm{P.tmem, w1, kop(X, C), C, false})) break;
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
      float v[16];
      tld(P, 0, c, v);
#pragma unroll
      for (int i = 0; i < 16; ++i) v[i] = gelu_tc(v[i]);
      if (f < 2 * C) put_mn(H, f, 64 * P.half + 16 * c, v);
    }
    if (!pipe_gemms(P, err, Gemm{P.tmem + TM, mop(H), w2, 2 * C, false, NHP})) break;
#pragma unroll
    for (int j = 0; j < NHP / 16; ++j) {
      if (!owns(j, P.half)) continue;
      float r[16];
      rld(P, TM, j, r);
#pragma unroll
      for (int i = 0; i < 16; ++i) os[f * LO + 16 * j + i] = r[i] + __ldg(b2 + 16 * j + i);
    }
    pipe_sync(P.id);
    if (P.half == 0) {
      const long v = v0 + f;
      float* o = os + f * LO;
      if (v < V) {
        head_voxel_bwd<T>(hp, o, NHP, head_inputs(hp, xin, V, v), ybar, V, v, xinbar);
      } else {
        for (int c = 0; c < NHP; ++c) o[c] = 0.f;
      }
#pragma unroll
      for (int j = 0; j < NHP / 16; ++j) {
        float r[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) r[i] = o[16 * j + i];
        put16(Ob, f, 16 * j, NHP, r);
      }
    }
    if (!pipe_gemms(P, err, Gemm{P.tmem + TM, w2t, kop(Ob, NHP), NHP, false})) break;
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
      float hp_[16], gb[16];
      tld(P, 0, c, hp_);
      tld(P, TM, c, gb);
#pragma unroll
      for (int i = 0; i < 16; ++i) gb[i] *= gelu_grad_tc(hp_[i]);
      if (f < 2 * C) put_mn(H, f, 64 * P.half + 16 * c, gb);
    }
    if (!pipe_gemms(P, err, Gemm{P.tmem, mop(H), w1t, 2 * C, false, C})) break;
    const long v = v0 + f;
#pragma unroll
    for (int j = 0; j < C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      float r[16];
      rld(P, 0, j, r);
      if (v < V)
#pragma unroll
        for (int i = 0; i < 16; i += 4)
          *reinterpret_cast<float4*>(xbar + v * C + 16 * j + i) = make_float4(r[i], r[i + 1], r[i + 2], r[i + 3]);
    }
  }
  pipe_finish(P, tslot, 2 * NCOL);
}

// ============================================================================================== width 96
// The production model's width (96): a channel MLP's split weights take 144 KB, so a CTA runs one 256-thread pipeline
// and every GEMM runs untransposed (lane = voxel row; the 16-column chunks of a row alternate between its two threads,
// as in the other row-oriented kernels). The 2C = 192 hidden features pass through one [128][96] operand tile in two
// K-halves. The backward reads its transposed weights out of the forward's matrices: a K-major [R][K] matrix read as
// an MN-major operand is its transpose ([K][R]), so one 144 KB pack serves all three of its GEMMs.
// The ffno_mlp2_fwd_tc contract at C = 96: pre = gelu(X W1^T) W2^T with X = in (+ res GN(prev) [gelu] in modes 1 and
// 2, written to xout), and the GroupNorm partials of pre. Weights [w1 (2C x C), w2 (C x 2C)]. Tensor memory: D1 (2C
// columns) at 0, D2 (C) at 2C.
template <int MODE>
__global__ void __launch_bounds__(PT, 1) k_mlp2_tc96(const float* __restrict__ in, const float* __restrict__ prev,
                                                     const float* __restrict__ pc, float res, float* __restrict__ xout,
                                                     long V, const uint8_t* __restrict__ wpack,
                                                     const float* __restrict__ dw, float* __restrict__ pre,
                                                     double* __restrict__ partials, int* __restrict__ err) {
  constexpr int C = C96;
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(2 * C, C), B2 = mat_bytes(C, 2 * C);
  __shared__ float red[(PT / 32) * (GMAX + 1)], gm[GMAX], wsum;
  __shared__ double acc[GMAX * 3];
  PIPE_PROLOGUE(3 * C, 1)
  const Split T = split_at(smem + B1 + B2, TM, C);   // the input tile, then each K-half of the hidden layer
  if (tid < GMAX * 3) acc[tid] = 0.0;
  P.ok = load_weights(smem, wpack, B1 + B2, wcx, err);
  const Op w1 = wop(smem, 2 * C, C);
  const int row = P.feat();
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (P.ptid == 0) {   // the next tile's rows into L2 while this one runs (one tile step: 152 x 48 KB a tensor)
      const long tn = (t + tstep) * TM;
      prefetch_rows(in, tn, V, C);
      prefetch_rows(MODE != 0 ? prev : nullptr, tn, V, C);
    }
    fill96(T, v0, V, P.ptid, [&](long v, int k, float (&o)[8]) {
      ld8(in + v * C + k, o);
      if (MODE != 0) {
        float p[8];
        ld8(prev + v * C + k, p);
        const float4 y0 = gn_apply<MODE == 1>(make_float4(p[0], p[1], p[2], p[3]), gn_coefs(pc, C, k));
        const float4 y1 = gn_apply<MODE == 1>(make_float4(p[4], p[5], p[6], p[7]), gn_coefs(pc, C, k + 4));
        const float y[8] = {y0.x, y0.y, y0.z, y0.w, y1.x, y1.y, y1.z, y1.w};
#pragma unroll
        for (int i = 0; i < 8; ++i) o[i] = fmaf(res, y[i], o[i]);
        st8(xout + v * C + k, o);
      }
    });
    if (!pipe_gemms(P, err, Gemm{P.tmem, kop(T, C), w1, C, false, 2 * C})) break;
    for (int h = 0; h < 2; ++h) {
#pragma unroll 1
      for (int j = 6 * h; j < 6 * h + 6; ++j) {
        if (!owns(j, P.half)) continue;
        float v[16];
        rld(P, 0, j, v);
#pragma unroll
        for (int i = 0; i < 16; ++i) v[i] = gelu_tc(v[i]);
        put16(T, row, 16 * j - C * h, C, v);
      }
      if (!pipe_gemms(P, err, Gemm{P.tmem + 2 * C, kop(T, C), wop(smem + B1, C, 2 * C, 0, C * h), C, h > 0, C}))
        break;
    }
    if (!P.ok) break;
    const long v = v0 + row;
    const float w = v < V ? __ldg(dw + v) : 0.f;
    float vals[C];
#pragma unroll
    for (int j = 0; j < C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      float r[16];
      rld(P, 2 * C, j, r);
#pragma unroll
      for (int i = 0; i < 16; ++i) vals[16 * j + i] = r[i];
      if (v < V) {
        st8(pre + v * C + 16 * j, r);
        st8(pre + v * C + 16 * j + 8, r + 8);
      }
    }
    row_stats<C>(P, vals, w, red, gm, &wsum, acc);
  }
  __syncthreads();
  if (tid < GMAX) {
    double* o = partials + ((long)blockIdx.x * GMAX + tid) * 3;
    o[0] = acc[3 * tid];
    o[1] = acc[3 * tid + 1];
    o[2] = acc[3 * tid + 2];
  }
  pipe_finish(P, tslot, NCOL);
}

// The ffno_mlp2_bwd_tc contract at C = 96: a_bar = base + ((pre_bar W2) * gelu'(a W1^T)) W1, from the forward's pack
// [w1 (2C x C), w2 (C x 2C)]: W2 and W1 as MN-major operands give the second and third GEMMs' transposes. Tensor
// memory: D1 = a W1^T (2C) at 0, D2 = pre_bar W2 (2C) at 2C, D3 (C) at 4C.
__global__ void __launch_bounds__(PT, 1) k_mlp2_bwd_tc96(const float* __restrict__ a, const float* __restrict__ pb,
                                                         const float* __restrict__ base, long V,
                                                         const uint8_t* __restrict__ wpack, float* __restrict__ abar,
                                                         int* __restrict__ err) {
  constexpr int C = C96;
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(2 * C, C), B2 = mat_bytes(C, 2 * C);
  PIPE_PROLOGUE(5 * C, 1)
  const Split T = split_at(smem + B1 + B2, TM, C);
  P.ok = load_weights(smem, wpack, B1 + B2, wcx, err);
  const Op w1 = wop(smem, 2 * C, C), w2t = wop_t(smem + B1, C, 2 * C);
  const int row = P.feat();
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (P.ptid == 0) {   // the next tile's rows into L2 while this one runs (one tile step: 152 x 48 KB a tensor)
      const long tn = (t + tstep) * TM;
      prefetch_rows(a, tn, V, C);
      prefetch_rows(pb, tn, V, C);
      prefetch_rows(base, tn, V, C);
    }
    fill96(T, v0, V, P.ptid, [&](long v, int k, float (&o)[8]) { ld8(a + v * C + k, o); });
    if (!pipe_gemms(P, err, Gemm{P.tmem, kop(T, C), w1, C, false, 2 * C})) break;
    fill96(T, v0, V, P.ptid, [&](long v, int k, float (&o)[8]) { ld8(pb + v * C + k, o); });
    if (!pipe_gemms(P, err, Gemm{P.tmem + 2 * C, kop(T, C), w2t, C, false, 2 * C})) break;
    for (int h = 0; h < 2; ++h) {
#pragma unroll 1
      for (int j = 6 * h; j < 6 * h + 6; ++j) {
        if (!owns(j, P.half)) continue;
        float hp[16], gb[16];
        rld(P, 0, j, hp);
        rld(P, 2 * C, j, gb);
#pragma unroll
        for (int i = 0; i < 16; ++i) gb[i] *= gelu_grad_tc(hp[i]);
        put16(T, row, 16 * j - C * h, C, gb);
      }
      if (!pipe_gemms(P, err, Gemm{P.tmem + 4 * C, kop(T, C), wop_t(smem, 2 * C, C, C * h), C, h > 0, C})) break;
    }
    if (!P.ok) break;
    const long v = v0 + row;
#pragma unroll
    for (int j = 0; j < C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      float r[16];
      rld(P, 4 * C, j, r);
      if (v < V) {
        if (base) {
          float b[16];
          ld8(base + v * C + 16 * j, *reinterpret_cast<float(*)[8]>(b));
          ld8(base + v * C + 16 * j + 8, *reinterpret_cast<float(*)[8]>(b + 8));
#pragma unroll
          for (int i = 0; i < 16; ++i) r[i] += b[i];
        }
        st8(abar + v * C + 16 * j, r);
        st8(abar + v * C + 16 * j + 8, r + 8);
      }
    }
  }
  pipe_finish(P, tslot, NCOL);
}

// ---------------------------------------------------------------------------------------- width 96: branch fusion
// _fuse_branches at C = 96, where its four weight matrices (332 KB split) exceed shared memory: the forward as three
// kernels (the gates and their hidden pre-activation; the fuse hidden pre-activation hf = B Wf1^T; the output with
// its residual and GroupNorm partials), the backward as three (hf_bar; the branch gradients and the gate
// pre-activation gradient q; the input gradients), each holding at most 184 KB of weights. Every GEMM is K-sliced by
// 48 columns through one [128][48] tile; the backward reads its transposed weights out of the forward's packs.
constexpr int KS = 48;

// gelu(GN(p)) of 8 consecutive channels k..k+7 of one branch (cf: the GroupNorm coefficients)
__device__ __forceinline__ void branch8(const float* __restrict__ cf, int k, const float (&p)[8], float (&o)[8]) {
  const float4 a = gn_apply<true>(make_float4(p[0], p[1], p[2], p[3]), gn_coefs(cf, C96, k));
  const float4 b = gn_apply<true>(make_float4(p[4], p[5], p[6], p[7]), gn_coefs(cf, C96, k + 4));
  o[0] = a.x, o[1] = a.y, o[2] = a.z, o[3] = a.w, o[4] = b.x, o[5] = b.y, o[6] = b.z, o[7] = b.w;
}

// gates [V][2C] = sigmoid(gelu(A Wg1^T) Wg2^T + bias), A = [x, gelu(GN_s(sp)), gelu(GN_v(vp))]; hg = A Wg1^T if not
// NULL. Weights [wg1 (C x 3C), wg2 (2C x C)]. Tensor memory: D1 (C) at 0, D2 (2C) at C.
__global__ void __launch_bounds__(PT, 1) k_fuse1_tc96(const float* __restrict__ x, const float* __restrict__ sp,
                                                      const float* __restrict__ sc, const float* __restrict__ vp,
                                                      const float* __restrict__ vc, long V,
                                                      const uint8_t* __restrict__ wpack,
                                                      const float* __restrict__ bias, float* __restrict__ gates,
                                                      float* __restrict__ hg, int* __restrict__ err) {
  constexpr int C = C96;
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(C, 3 * C), B2 = mat_bytes(2 * C, C);
  PIPE_PROLOGUE(3 * C, 1)
  const Split T = split_at(smem + B1 + B2, TM, KS);
  P.ok = load_weights(smem, wpack, B1 + B2, wcx, err);
  const int row = P.feat();
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (P.ptid == 0) {   // the next tile's rows into L2 while this one runs (one tile step: 152 x 48 KB a tensor)
      const long tn = (t + tstep) * TM;
      prefetch_rows(x, tn, V, C);
      prefetch_rows(sp, tn, V, C);
      prefetch_rows(vp, tn, V, C);
    }
    for (int sl = 0; sl < 6; ++sl) {   // K-slices of A: x, then the spec branch, then the vert branch
      const int part = sl / 2, k0 = (sl % 2) * KS;
      fill_oct<KS>(T, v0, V, P.ptid, [&](long v, int k, float (&o)[8]) {
        if (part == 0) {
          ld8(x + v * C + k0 + k, o);
        } else {
          float p[8];
          ld8((part == 1 ? sp : vp) + v * C + k0 + k, p);
          branch8(part == 1 ? sc : vc, k0 + k, p, o);
        }
      });
      if (!pipe_gemms(P, err, Gemm{P.tmem, kop(T, KS), wop(smem, C, 3 * C, 0, sl * KS), KS, sl > 0, C})) break;
    }
    if (!P.ok) break;
    const long v = v0 + row;
    for (int h = 0; h < 2; ++h) {   // the hidden layer: hg out, gelu(hg) into the tile, K-half h of GEMM2
#pragma unroll 1
      for (int j = 3 * h; j < 3 * h + 3; ++j) {
        if (!owns(j, P.half)) continue;
        float hv[16];
        rld(P, 0, j, hv);
        if (hg && v < V) {
          st8(hg + v * C + 16 * j, hv);
          st8(hg + v * C + 16 * j + 8, hv + 8);
        }
#pragma unroll
        for (int i = 0; i < 16; ++i) hv[i] = gelu_tc(hv[i]);
        put16(T, row, 16 * j - KS * h, KS, hv);
      }
      if (!pipe_gemms(P, err, Gemm{P.tmem + C, kop(T, KS), wop(smem + B1, 2 * C, C, 0, KS * h), KS, h > 0, 2 * C}))
        break;
    }
    if (!P.ok) break;
#pragma unroll 1
    for (int j = 0; j < 2 * C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      float g[16];
      rld(P, C, j, g);
#pragma unroll
      for (int i = 0; i < 16; ++i) g[i] = sigmoid_tc(g[i] + __ldg(bias + 16 * j + i));
      if (v < V) {
        st8(gates + v * 2 * C + 16 * j, g);
        st8(gates + v * 2 * C + 16 * j + 8, g + 8);
      }
    }
  }
  pipe_finish(P, tslot, NCOL);
}

// hf [V][2C] = B Wf1^T, B = [gelu(GN_s(sp)) g_s, gelu(GN_v(vp)) g_v]. Weights [wf1 (2C x 2C)].
__global__ void __launch_bounds__(PT, 1) k_fuse_hidden_tc96(const float* __restrict__ sp, const float* __restrict__ sc,
                                                            const float* __restrict__ vp, const float* __restrict__ vc,
                                                            const float* __restrict__ gates, long V,
                                                            const uint8_t* __restrict__ wpack,
                                                            float* __restrict__ hf, int* __restrict__ err) {
  constexpr int C = C96;
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(2 * C, 2 * C);
  PIPE_PROLOGUE(2 * C, 1)
  const Split T = split_at(smem + B1, TM, KS);
  P.ok = load_weights(smem, wpack, B1, wcx, err);
  const int row = P.feat();
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (P.ptid == 0) {   // the next tile's rows into L2 while this one runs (one tile step: 152 x 48 KB a tensor)
      const long tn = (t + tstep) * TM;
      prefetch_rows(sp, tn, V, C);
      prefetch_rows(vp, tn, V, C);
      prefetch_rows(gates, tn, V, 2 * C);
    }
    for (int sl = 0; sl < 4; ++sl) {
      const int part = sl / 2, k0 = (sl % 2) * KS;
      fill_oct<KS>(T, v0, V, P.ptid, [&](long v, int k, float (&o)[8]) {
        float p[8], g[8];
        ld8((part == 0 ? sp : vp) + v * C + k0 + k, p);
        ld8(gates + v * 2 * C + part * C + k0 + k, g);
        branch8(part == 0 ? sc : vc, k0 + k, p, o);
#pragma unroll
        for (int i = 0; i < 8; ++i) o[i] *= g[i];
      });
      if (!pipe_gemms(P, err, Gemm{P.tmem, kop(T, KS), wop(smem, 2 * C, 2 * C, 0, sl * KS), KS, sl > 0, 2 * C}))
        break;
    }
    if (!P.ok) break;
    const long v = v0 + row;
#pragma unroll 1
    for (int j = 0; j < 2 * C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      float r[16];
      rld(P, 0, j, r);
      if (v < V) {
        st8(hf + v * 2 * C + 16 * j, r);
        st8(hf + v * 2 * C + 16 * j + 8, r + 8);
      }
    }
  }
  pipe_finish(P, tslot, NCOL);
}

// pre [V][C] = gelu(hf) Wf2^T + (B_s + B_v) / 2 with the GroupNorm partials of pre. Weights [wf2 (C x 2C)].
__global__ void __launch_bounds__(PT, 1) k_fuse_out_tc96(const float* __restrict__ sp, const float* __restrict__ sc,
                                                         const float* __restrict__ vp, const float* __restrict__ vc,
                                                         const float* __restrict__ gates, const float* __restrict__ hf,
                                                         long V, const uint8_t* __restrict__ wpack,
                                                         const float* __restrict__ dw, float* __restrict__ pre,
                                                         double* __restrict__ partials, int* __restrict__ err) {
  constexpr int C = C96;
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(C, 2 * C);
  __shared__ float red[(PT / 32) * (GMAX + 1)], gm[GMAX], wsum;
  __shared__ double acc[GMAX * 3];
  PIPE_PROLOGUE(C, 1)
  const Split T = split_at(smem + B1, TM, KS);
  if (tid < GMAX * 3) acc[tid] = 0.0;
  P.ok = load_weights(smem, wpack, B1, wcx, err);
  const int row = P.feat();
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (P.ptid == 0) {   // the next tile's rows into L2 while this one runs (one tile step: 152 x 48 KB a tensor)
      const long tn = (t + tstep) * TM;
      prefetch_rows(hf, tn, V, 2 * C);
      prefetch_rows(sp, tn, V, C);
      prefetch_rows(vp, tn, V, C);
      prefetch_rows(gates, tn, V, 2 * C);
    }
    for (int sl = 0; sl < 4; ++sl) {
      fill_oct<KS>(T, v0, V, P.ptid, [&](long v, int k, float (&o)[8]) {
        ld8(hf + v * 2 * C + sl * KS + k, o);
#pragma unroll
        for (int i = 0; i < 8; ++i) o[i] = gelu_tc(o[i]);
      });
      if (!pipe_gemms(P, err, Gemm{P.tmem, kop(T, KS), wop(smem, C, 2 * C, 0, sl * KS), KS, sl > 0, C})) break;
    }
    if (!P.ok) break;
    const long v = v0 + row;
    const float w = v < V ? __ldg(dw + v) : 0.f;
    float vals[C];
#pragma unroll
    for (int j = 0; j < C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      float r[16];
      rld(P, 0, j, r);
      if (v < V) {
#pragma unroll
        for (int e = 0; e < 16; e += 8) {
          float ps[8], pv[8], gs[8], gv[8], bs[8], bv[8];
          ld8(sp + v * C + 16 * j + e, ps);
          ld8(vp + v * C + 16 * j + e, pv);
          ld8(gates + v * 2 * C + 16 * j + e, gs);
          ld8(gates + v * 2 * C + C + 16 * j + e, gv);
          branch8(sc, 16 * j + e, ps, bs);
          branch8(vc, 16 * j + e, pv, bv);
#pragma unroll
          for (int i = 0; i < 8; ++i) r[e + i] += 0.5f * (bs[i] * gs[i] + bv[i] * gv[i]);
        }
        st8(pre + v * C + 16 * j, r);
        st8(pre + v * C + 16 * j + 8, r + 8);
      }
#pragma unroll
      for (int i = 0; i < 16; ++i) vals[16 * j + i] = r[i];
    }
    row_stats<C>(P, vals, w, red, gm, &wsum, acc);
  }
  __syncthreads();
  if (tid < GMAX) {
    double* o = partials + ((long)blockIdx.x * GMAX + tid) * 3;
    o[0] = acc[3 * tid];
    o[1] = acc[3 * tid + 1];
    o[2] = acc[3 * tid + 2];
  }
  pipe_finish(P, tslot, NCOL);
}

// hfb [V][2C] = (fb Wf2) * gelu'(hf), fb = fused_pre_bar. Weights [wf2 (C x 2C)], read as its transpose.
__global__ void __launch_bounds__(PT, 1) k_fuse_bwd_h_tc96(const float* __restrict__ fb, const float* __restrict__ hf,
                                                           long V, const uint8_t* __restrict__ wpack,
                                                           float* __restrict__ hfb, int* __restrict__ err) {
  constexpr int C = C96;
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(C, 2 * C);
  PIPE_PROLOGUE(2 * C, 1)
  const Split T = split_at(smem + B1, TM, KS);
  P.ok = load_weights(smem, wpack, B1, wcx, err);
  const int row = P.feat();
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (P.ptid == 0) {   // the next tile's rows into L2 while this one runs (one tile step: 152 x 48 KB a tensor)
      const long tn = (t + tstep) * TM;
      prefetch_rows(fb, tn, V, C);
      prefetch_rows(hf, tn, V, 2 * C);
    }
    for (int sl = 0; sl < 2; ++sl) {
      fill_oct<KS>(T, v0, V, P.ptid, [&](long v, int k, float (&o)[8]) { ld8(fb + v * C + sl * KS + k, o); });
      if (!pipe_gemms(P, err, Gemm{P.tmem, kop(T, KS), wop_t(smem, C, 2 * C, sl * KS), KS, sl > 0, 2 * C})) break;
    }
    if (!P.ok) break;
    const long v = v0 + row;
#pragma unroll 1
    for (int j = 0; j < 2 * C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      float r[16], h[16];
      rld(P, 0, j, r);
      if (v < V) {
        ld8(hf + v * 2 * C + 16 * j, *reinterpret_cast<float(*)[8]>(h));
        ld8(hf + v * 2 * C + 16 * j + 8, *reinterpret_cast<float(*)[8]>(h + 8));
#pragma unroll
        for (int i = 0; i < 16; ++i) r[i] *= gelu_grad_tc(h[i]);
        st8(hfb + v * 2 * C + 16 * j, r);
        st8(hfb + v * 2 * C + 16 * j + 8, r + 8);
      }
    }
  }
  pipe_finish(P, tslot, NCOL);
}

// B_bar = hfb Wf1 + [fb, fb] / 2; sbar = B_bar_s g_s, vbar = B_bar_v g_v; q [V][2C] = B_bar [s, v] g (1 - g), with
// s = gelu(GN_s(sp)), v = gelu(GN_v(vp)). q may be hfb itself. Weights [wf1 (2C x 2C)], read as its transpose.
__global__ void __launch_bounds__(PT, 1) k_fuse_bwd_q_tc96(const float* __restrict__ sp, const float* __restrict__ sc,
                                                           const float* __restrict__ vp, const float* __restrict__ vc,
                                                           const float* __restrict__ gates,
                                                           const float* __restrict__ fb, const float* hfb, long V,
                                                           const uint8_t* __restrict__ wpack,
                                                           float* __restrict__ sbar, float* __restrict__ vbar,
                                                           float* q, int* __restrict__ err) {
  constexpr int C = C96;
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(2 * C, 2 * C);
  PIPE_PROLOGUE(2 * C, 1)
  const Split T = split_at(smem + B1, TM, KS);
  P.ok = load_weights(smem, wpack, B1, wcx, err);
  const int row = P.feat();
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    for (int sl = 0; sl < 4; ++sl) {
      fill_oct<KS>(T, v0, V, P.ptid, [&](long v, int k, float (&o)[8]) { ld8(hfb + v * 2 * C + sl * KS + k, o); });
      if (!pipe_gemms(P, err, Gemm{P.tmem, kop(T, KS), wop_t(smem, 2 * C, 2 * C, sl * KS), KS, sl > 0, 2 * C}))
        break;
    }
    if (!P.ok) break;
    const long v = v0 + row;
#pragma unroll 1
    for (int j = 0; j < 2 * C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      const int part = j / (C / 16), c0 = 16 * (j % (C / 16));
      float r[16];
      rld(P, 0, j, r);
      if (v < V) {
        float dr[16], qq[16];
#pragma unroll
        for (int e = 0; e < 16; e += 8) {
          float f[8], g[8], p[8], b[8];
          ld8(fb + v * C + c0 + e, f);
          ld8(gates + v * 2 * C + part * C + c0 + e, g);
          ld8((part == 0 ? sp : vp) + v * C + c0 + e, p);
          branch8(part == 0 ? sc : vc, c0 + e, p, b);
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            const float bb = r[e + i] + 0.5f * f[i];
            dr[e + i] = bb * g[i];
            qq[e + i] = bb * b[i] * g[i] * (1.f - g[i]);
          }
        }
        float* dst = part == 0 ? sbar : vbar;
        st8(dst + v * C + c0, dr);
        st8(dst + v * C + c0 + 8, dr + 8);
        st8(q + v * 2 * C + 16 * j, qq);
        st8(q + v * 2 * C + 16 * j + 8, qq + 8);
      }
    }
  }
  pipe_finish(P, tslot, NCOL);
}

// hg_bar = (q Wg2) * gelu'(hg); A_bar = hg_bar Wg1: x_bar = base + A_bar[:C], sbar += A_bar[C:2C], vbar +=
// A_bar[2C:]. Weights [wg1 (C x 3C), wg2 (2C x C)] (the gates' pack), read as their transposes. Tensor memory: D3
// (C) at 0, D4 (3C, two accumulators of 144) at C.
__global__ void __launch_bounds__(PT, 1) k_fuse_bwd_x_tc96(const float* __restrict__ q, const float* __restrict__ hg,
                                                           const float* __restrict__ base, long V,
                                                           const uint8_t* __restrict__ wpack,
                                                           float* __restrict__ xbar, float* __restrict__ sbar,
                                                           float* __restrict__ vbar, int* __restrict__ err) {
  constexpr int C = C96;
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(C, 3 * C), B2 = mat_bytes(2 * C, C);
  PIPE_PROLOGUE(4 * C, 1)
  const Split T = split_at(smem + B1 + B2, TM, KS);
  P.ok = load_weights(smem, wpack, B1 + B2, wcx, err);
  const int row = P.feat();
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (P.ptid == 0) {   // the next tile's rows into L2 while this one runs (one tile step: 152 x 48 KB a tensor)
      const long tn = (t + tstep) * TM;
      prefetch_rows(q, tn, V, 2 * C);
      prefetch_rows(hg, tn, V, C);
      prefetch_rows(base, tn, V, C);
    }
    for (int sl = 0; sl < 4; ++sl) {
      fill_oct<KS>(T, v0, V, P.ptid, [&](long v, int k, float (&o)[8]) { ld8(q + v * 2 * C + sl * KS + k, o); });
      if (!pipe_gemms(P, err, Gemm{P.tmem, kop(T, KS), wop_t(smem + B1, 2 * C, C, sl * KS), KS, sl > 0, C})) break;
    }
    if (!P.ok) break;
    const long v = v0 + row;
    for (int h = 0; h < 2; ++h) {
#pragma unroll 1
      for (int j = 3 * h; j < 3 * h + 3; ++j) {
        if (!owns(j, P.half)) continue;
        float d[16], hv[16];
        rld(P, 0, j, d);
        if (v < V) {
          ld8(hg + v * C + 16 * j, *reinterpret_cast<float(*)[8]>(hv));
          ld8(hg + v * C + 16 * j + 8, *reinterpret_cast<float(*)[8]>(hv + 8));
#pragma unroll
          for (int i = 0; i < 16; ++i) d[i] *= gelu_grad_tc(hv[i]);
        } else {
#pragma unroll
          for (int i = 0; i < 16; ++i) d[i] = 0.f;
        }
        put16(T, row, 16 * j - KS * h, KS, d);
      }
      const Gemm g4b{P.tmem + C + 144, kop(T, KS), wop_t(smem, C, 3 * C, KS * h, 144), KS, h > 0, 144};
      if (!pipe_gemms(P, err, Gemm{P.tmem + C, kop(T, KS), wop_t(smem, C, 3 * C, KS * h, 0), KS, h > 0, 144}, &g4b))
        break;
    }
    if (!P.ok) break;
#pragma unroll 1
    for (int j = 0; j < 3 * C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      const int part = j / (C / 16), c0 = 16 * (j % (C / 16));
      float r[16];
      rld(P, C, j, r);
      if (v < V) {
        const float* add = part == 0 ? base : (part == 1 ? sbar : vbar);
        float* dst = part == 0 ? xbar : (part == 1 ? sbar : vbar);
        if (add) {
          float b[16];
          ld8(add + v * C + c0, *reinterpret_cast<float(*)[8]>(b));
          ld8(add + v * C + c0 + 8, *reinterpret_cast<float(*)[8]>(b + 8));
#pragma unroll
          for (int i = 0; i < 16; ++i) r[i] += b[i];
        }
        st8(dst + v * C + c0, r);
        st8(dst + v * C + c0 + 8, r + 8);
      }
    }
  }
  pipe_finish(P, tslot, NCOL);
}

// ---------------------------------------------------------------------------------------- width 96: mixing
// ffno_spectral_mix at C = 96 (SpectralConv2dFull.mix_spectrum, HeightSpectralConv's mode mixing): for frequency f and
// row b, x = [re | im] (2C), out = g_f (x M) + [U_f t_re, U_f t_im], t = [V_f x_re, V_f x_im], with M the pack (wbig
// for the mixing, wbig^T for its adjoint) read through its transpose view. An item is 128 rows b of one frequency; two
// pipelines a CTA take alternate items and share M. x arrives in four K-slices of 48 through the pipeline's tile, and
// each slice feeds x M (N = 2C) and the projections t (N = 16: a block-diagonal [16][2C] operand whose rows 0..7 hold
// V_f on the re half and rows 8..15 on the im half; its zero blocks and the rows beyond the rank are written once, the
// rest per item); the epilogue applies g_f and U_f (FP32, U_f in shared memory). Tensor memory per pipeline: x M at 0
// (2C columns), t at 2C (16).
constexpr int MIXR = 8;   // the low-rank terms this kernel carries (the model's freq_mix_rank)

__global__ void __launch_bounds__(CT, 1) k_mix_tc96(const float* __restrict__ in, float* __restrict__ out, long F,
                                                    long nb, long sf, long sb, long s_im,
                                                    const uint8_t* __restrict__ wpack, const float* __restrict__ g,
                                                    const float* __restrict__ U, const float* __restrict__ Vm,
                                                    int rank, int* __restrict__ err) {
  constexpr int C = C96, K2 = 2 * C;
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(K2, K2), VB = mat_bytes(16, K2), RB = tile_bytes(KS) + VB;
  __shared__ float us_all[2][C * MIXR];
  const long nbt = (nb + TM - 1) / TM;
  const long V = F * nbt * TM;   // the prologue's tiles are the items: (frequency, block of 128 rows) pairs
  PIPE_PROLOGUE(K2 + 16, 2)
  const Split T = split_at(smem + B1 + pid * RB, TM, KS);
  uint8_t* vblk = smem + B1 + pid * RB + tile_bytes(KS);   // [16][2C] split, K-major
  float* us = us_all[pid];
  for (int e = P.ptid; e < (int)(VB / 16); e += PT) reinterpret_cast<uint4*>(vblk)[e] = make_uint4(0u, 0u, 0u, 0u);
  for (int e = P.ptid; e < C * MIXR; e += PT) us[e] = 0.f;
  P.ok = load_weights(smem, wpack, B1, wcx, err);
  const int row = P.feat();
  // the per-frequency values of the pipeline's next item (g_f; this thread's U_f and V_f elements e = ptid + u PT,
  // e < C rank <= 3 PT), loaded one item ahead so that their latency stays off the item's path
  static_assert(C * MIXR <= 3 * PT, "three U_f and V_f elements a thread");
  float un[3], vn[3], grn = 0.f, gin = 0.f;
  auto load_freq = [&](long it2) {
    const long f2 = it2 / nbt;
    grn = __ldg(g + 2 * f2);
    gin = __ldg(g + 2 * f2 + 1);
#pragma unroll
    for (int u = 0; u < 3; ++u) {
      const int e = P.ptid + u * PT;
      const bool in = rank && e < C * rank;
      un[u] = in ? __ldg(U + f2 * C * rank + e) : 0.f;
      vn[u] = in ? __ldg(Vm + f2 * rank * C + e) : 0.f;
    }
  };
  if (t0 < nt) load_freq(t0);
  for (long it = t0; P.ok && it < nt; it += tstep) {
    const long f = it / nbt, b0 = (it % nbt) * TM;
    const float gr = grn, gi = gin;
    if (rank) {   // this frequency's U_f and V_f into shared memory
      pipe_sync(P.id);   // the previous item's epilogue has read U_f (its MMAs, which read V_f, have completed)
#pragma unroll
      for (int u = 0; u < 3; ++u) {
        const int e = P.ptid + u * PT;
        if (e >= C * rank) break;
        us[(e / rank) * MIXR + e % rank] = un[u];
        const int r = e / C, k = e % C;   // V_f element (r, k)
        uint32_t h, l;
        tc::split_pack(vn[u], 0.f, h, l);
        const uint32_t o0 = tc::kmajor_offset(r, k, K2), o1 = tc::kmajor_offset(8 + r, C + k, K2);
        *reinterpret_cast<uint16_t*>(vblk + o0) = (uint16_t)(h & 0xffffu);
        *reinterpret_cast<uint16_t*>(vblk + VB / 2 + o0) = (uint16_t)(l & 0xffffu);
        *reinterpret_cast<uint16_t*>(vblk + o1) = (uint16_t)(h & 0xffffu);
        *reinterpret_cast<uint16_t*>(vblk + VB / 2 + o1) = (uint16_t)(l & 0xffffu);
      }
    }
    if (it + tstep < nt) load_freq(it + tstep);
    const float* fin = in + f * sf;
    for (int sl = 0; sl < 4; ++sl) {
      const int part = sl / 2, k0 = (sl % 2) * KS;
      fill_oct<KS>(T, b0, nb, P.ptid, [&](long b, int k, float (&o)[8]) { ld8(fin + b * sb + part * s_im + k0 + k, o); });
      const Op vo = wop(vblk, 16, K2, 0, sl * KS);
      const Gemm gt{P.tmem + K2, kop(T, KS), vo, KS, sl > 0, 16};
      if (!pipe_gemms(P, err, Gemm{P.tmem, kop(T, KS), wop_t(smem, K2, K2, sl * KS), KS, sl > 0, K2},
                      rank ? &gt : nullptr))
        break;
    }
    if (!P.ok) break;
    const long b = b0 + row;
    float t[16];
    if (rank) rld(P, K2, 0, t);
#pragma unroll 1
    for (int j = 0; j < C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      float yr[16], yi[16];
      rld(P, 0, j, yr);
      rld(P, 0, j + C / 16, yi);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const float ar = yr[i], ai = yi[i];
        yr[i] = ar * gr - ai * gi;
        yi[i] = ar * gi + ai * gr;
      }
      if (rank) {
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const float* u = us + (16 * j + i) * MIXR;
          float lr = 0.f, li = 0.f;
#pragma unroll
          for (int r = 0; r < MIXR; ++r) {
            lr = fmaf(u[r], t[r], lr);
            li = fmaf(u[r], t[8 + r], li);
          }
          yr[i] += lr;
          yi[i] += li;
        }
      }
      if (b < nb) {
        float* fo = out + f * sf + b * sb + 16 * j;
        st8(fo, yr);
        st8(fo + 8, yr + 8);
        st8(fo + s_im, yi);
        st8(fo + s_im + 8, yi + 8);
      }
    }
  }
  pipe_finish(P, tslot, 2 * NCOL);
}

// ---------------------------------------------------------------------------------------- width 96: head
// The level-fraction head at C = 96 (proj1 -> GELU -> proj2, head_output): o = gelu(x P1^T) P2^T + b2 (row-oriented,
// the hidden layer in four K-slices of 48 through the tile), then the voxel's LTE log-softmax (head_voxel_fwd) by
// the row's first thread. Weights [P1 (2C x C), P2 (NHP x 2C)]. Tensor memory: the hidden layer (2C) at 0, o at 2C.
template <int NHP, typename T>
__global__ void __launch_bounds__(PT, 1) k_head_tc96(const float* __restrict__ x, const float* __restrict__ xin, long V,
                                                     const uint8_t* __restrict__ wpack, const float* __restrict__ b2,
                                                     int nh, const __grid_constant__ ffno_head_params hp,
                                                     float* __restrict__ out, float* __restrict__ head_out,
                                                     int* __restrict__ err) {
  constexpr int C = C96;
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(2 * C, C), B2 = mat_bytes(NHP, 2 * C);
  PIPE_PROLOGUE(2 * C + NHP, 1)
  const Split T_ = split_at(smem + B1 + B2, TM, KS);
  P.ok = load_weights(smem, wpack, B1 + B2, wcx, err);
  const int row = P.feat();
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (P.ptid == 0) {   // the next tile's rows into L2 while this one runs (one tile step: 152 x 48 KB a tensor)
      const long tn = (t + tstep) * TM;
      prefetch_rows(x, tn, V, C);
    }
    for (int sl = 0; sl < 2; ++sl) {
      fill_oct<KS>(T_, v0, V, P.ptid, [&](long v, int k, float (&o)[8]) { ld8(x + v * C + sl * KS + k, o); });
      if (!pipe_gemms(P, err, Gemm{P.tmem, kop(T_, KS), wop(smem, 2 * C, C, 0, sl * KS), KS, sl > 0, 2 * C})) break;
    }
    if (!P.ok) break;
    for (int sl = 0; sl < 4; ++sl) {
#pragma unroll 1
      for (int j = 3 * sl; j < 3 * sl + 3; ++j) {
        if (!owns(j, P.half)) continue;
        float h[16];
        rld(P, 0, j, h);
#pragma unroll
        for (int i = 0; i < 16; ++i) h[i] = gelu_tc(h[i]);
        put16(T_, row, 16 * j - KS * sl, KS, h);
      }
      if (!pipe_gemms(P, err, Gemm{P.tmem + 2 * C, kop(T_, KS), wop(smem + B1, NHP, 2 * C, 0, sl * KS), KS, sl > 0,
                                   NHP}))
        break;
    }
    if (!P.ok) break;
    const long v = v0 + row;
    if (P.half == 0) {   // whole warps (tensor-memory loads are warp-collective); rows past the cube skip the head
      float o[NHP];
#pragma unroll
      for (int j = 0; j < NHP / 16; ++j) {
        float r[16];
        rld(P, 2 * C, j, r);
#pragma unroll
        for (int i = 0; i < 16; ++i) o[16 * j + i] = r[i] + __ldg(b2 + 16 * j + i);
      }
      if (v < V) {
        if (head_out)
          for (int c = 0; c < nh; ++c) head_out[(long)c * V + v] = o[c];
        head_voxel_fwd<T>(hp, o, head_inputs(hp, xin, V, v), out, V, v);
      }
    }
  }
  pipe_finish(P, tslot, NCOL);
}

// Its backward: the forward recomputed (the hidden pre-activation kept in tensor memory), o_bar from head_voxel_bwd
// (which writes x_in_bar), h_bar = (o_bar P2) * gelu'(pre), x_bar = h_bar P1, both products reading the transposes
// out of the forward's pack [P1, P2]. Tensor memory: pre (2C) at 0, o (NHP) at 2C, o_bar P2 (2C) at 2C + NHP, x_bar
// (C) at 4C + NHP.
template <int NHP, typename T>
__global__ void __launch_bounds__(PT, 1) k_head_bwd_tc96(const float* __restrict__ x, const float* __restrict__ xin,
                                                         const float* __restrict__ ybar, long V,
                                                         const uint8_t* __restrict__ wpack,
                                                         const float* __restrict__ b2,
                                                         const __grid_constant__ ffno_head_params hp,
                                                         float* __restrict__ xbar, float* __restrict__ xinbar,
                                                         int* __restrict__ err) {
  constexpr int C = C96;
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr uint32_t B1 = mat_bytes(2 * C, C), B2 = mat_bytes(NHP, 2 * C);
  constexpr uint32_t DO = 2 * C, D3 = 2 * C + NHP, D4 = 4 * C + NHP;
  static_assert(D4 + C <= 512, "tensor memory");
  PIPE_PROLOGUE(D4 + C, 1)
  const Split T_ = split_at(smem + B1 + B2, TM, KS), Ob = split_at(smem + B1 + B2, TM, NHP);
  P.ok = load_weights(smem, wpack, B1 + B2, wcx, err);
  const int row = P.feat();
  for (long t = t0; P.ok && t < nt; t += tstep) {
    const long v0 = t * TM;
    if (P.ptid == 0) {   // the next tile's rows into L2 while this one runs (one tile step: 152 x 48 KB a tensor)
      const long tn = (t + tstep) * TM;
      prefetch_rows(x, tn, V, C);
    }
    for (int sl = 0; sl < 2; ++sl) {
      fill_oct<KS>(T_, v0, V, P.ptid, [&](long v, int k, float (&o)[8]) { ld8(x + v * C + sl * KS + k, o); });
      if (!pipe_gemms(P, err, Gemm{P.tmem, kop(T_, KS), wop(smem, 2 * C, C, 0, sl * KS), KS, sl > 0, 2 * C})) break;
    }
    if (!P.ok) break;
    for (int sl = 0; sl < 4; ++sl) {
#pragma unroll 1
      for (int j = 3 * sl; j < 3 * sl + 3; ++j) {
        if (!owns(j, P.half)) continue;
        float h[16];
        rld(P, 0, j, h);
#pragma unroll
        for (int i = 0; i < 16; ++i) h[i] = gelu_tc(h[i]);
        put16(T_, row, 16 * j - KS * sl, KS, h);
      }
      if (!pipe_gemms(P, err, Gemm{P.tmem + DO, kop(T_, KS), wop(smem + B1, NHP, 2 * C, 0, sl * KS), KS, sl > 0,
                                   NHP}))
        break;
    }
    if (!P.ok) break;
    const long v = v0 + row;
    if (P.half == 0) {
      float o[NHP];
#pragma unroll
      for (int j = 0; j < NHP / 16; ++j) {
        float r[16];
        rld(P, DO, j, r);
#pragma unroll
        for (int i = 0; i < 16; ++i) o[16 * j + i] = r[i] + __ldg(b2 + 16 * j + i);
      }
      if (v < V) {
        head_voxel_bwd<T>(hp, o, NHP, head_inputs(hp, xin, V, v), ybar, V, v, xinbar);
      } else {
#pragma unroll
        for (int c = 0; c < NHP; ++c) o[c] = 0.f;
      }
#pragma unroll
      for (int j = 0; j < NHP / 16; ++j) {
        float r[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) r[i] = o[16 * j + i];
        put16(Ob, row, 16 * j, NHP, r);
      }
    }
    if (!pipe_gemms(P, err, Gemm{P.tmem + D3, kop(Ob, NHP), wop_t(smem + B1, NHP, 2 * C), NHP, false, 2 * C})) break;
    for (int sl = 0; sl < 4; ++sl) {
#pragma unroll 1
      for (int j = 3 * sl; j < 3 * sl + 3; ++j) {
        if (!owns(j, P.half)) continue;
        float hp_[16], gb[16];
        rld(P, 0, j, hp_);
        rld(P, D3, j, gb);
#pragma unroll
        for (int i = 0; i < 16; ++i) gb[i] *= gelu_grad_tc(hp_[i]);
        put16(T_, row, 16 * j - KS * sl, KS, gb);
      }
      if (!pipe_gemms(P, err, Gemm{P.tmem + D4, kop(T_, KS), wop_t(smem, 2 * C, C, sl * KS), KS, sl > 0, C})) break;
    }
    if (!P.ok) break;
#pragma unroll
    for (int j = 0; j < C / 16; ++j) {
      if (!owns(j, P.half)) continue;
      float r[16];
      rld(P, D4, j, r);
      if (v < V) {
        st8(xbar + v * C + 16 * j, r);
        st8(xbar + v * C + 16 * j + 8, r + 8);
      }
    }
  }
  pipe_finish(P, tslot, NCOL);
}

#undef PIPE_PROLOGUE

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
  return ffno::smem_cap_ok(kernel, bytes);
}

bool tc_width(int C) { return C == 16 || C == 32 || C == 64; }
bool chan_width(int C) { return tc_width(C) || C == C96; }   // channel MLPs and input gates: also width 96
bool aligned16(const void* p) { return p && (reinterpret_cast<uintptr_t>(p) % 16) == 0; }
bool aligned32(const void* p) { return p && (reinterpret_cast<uintptr_t>(p) % 32) == 0; }

}  // namespace

// The width-96 mixing, launched by ffno_spectral_mix_tc (spectral_tc.cu) after its argument checks.
namespace ffno {
int launch_mix_tc96(const float* in, float* out, long F, long nb, long sf, long sb, long s_im, const void* wpack,
                    const float* g, const float* U, const float* Vm, int rank, int* err, cudaStream_t s) {
  if (rank > MIXR) return FFNO_EINVAL;
  if (sf % 8 || sb % 8 || s_im % 8 || !aligned32(in) || !aligned32(out)) return FFNO_EINVAL;   // 32-byte rows
  const size_t smem = mat_bytes(2 * C96, 2 * C96) + 2 * (tile_bytes(KS) + mat_bytes(16, 2 * C96));
  if (!launch_prep(k_mix_tc96, smem)) return FFNO_ELAUNCH;
  const long items = F * ((nb + TM - 1) / TM);
  const long pairs = (items + 1) / 2;   // two pipelines a CTA
  const long grid = pairs < sms() ? pairs : sms();
  k_mix_tc96<<<(unsigned)grid, CT, smem, s>>>(in, out, F, nb, sf, sb, s_im, static_cast<const uint8_t*>(wpack), g, U,
                                              Vm, rank, err);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}
}  // namespace ffno

// ====================================================================================================== C ABI
extern "C" {

int ffno_tc_parts(long V) { return grid_tc(V); }

int ffno_tc_width_supported(int C) { return tc_width(C) ? 1 : 0; }

int ffno_tc_channel_width_supported(int C) { return chan_width(C) ? 1 : 0; }

int ffno_tc_set_prefetch_tiles(int tiles) {
  if (tiles < 0 || tiles > 4) return FFNO_EINVAL;
  return cudaMemcpyToSymbol(c_pf, &tiles, sizeof(int)) == cudaSuccess ? FFNO_OK : FFNO_ELAUNCH;
}

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
  if (!in || !wpack || !dw || !pre || !partials) return FFNO_EINVAL;
  if (!chan_width(C) || V < 1 || mode < 0 || mode > 2 || groups != GMAX || !err || !aligned16(wpack)) return FFNO_EINVAL;
  if (mode && (!prev_pre || !prev_coefs || !xout)) return FFNO_EINVAL;
  if (nparts != grid_tc(V)) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  if (C == C96) {   // rows are moved 32 bytes a request
    if (!aligned32(in) || !aligned32(pre) || (mode && (!aligned32(prev_pre) || !aligned32(xout)))) return FFNO_EINVAL;
    const auto* w = static_cast<const uint8_t*>(wpack);
    const size_t smem = mat_bytes(2 * C96, C96) + mat_bytes(C96, 2 * C96) + tile_bytes(C96);
#define L96(M)                                                                                                    \
  if (mode == M) {                                                                                              \
    if (!launch_prep(k_mlp2_tc96<M>, smem)) return FFNO_ELAUNCH;                                                \
    k_mlp2_tc96<M><<<nparts, PT, smem, s>>>(in, prev_pre, prev_coefs, res, xout, V, w, dw, pre, partials, err); \
  }
    L96(0) L96(1) L96(2)
#undef L96
    FFNO_CHECK_LAUNCH();
    return FFNO_OK;
  }
  if (ws::mlp2_fwd_supported(C))
    return ws::mlp2_fwd(mode, in, prev_pre, prev_coefs, res, xout, V, C, wpack, dw, pre, partials, nparts, err, s);
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
  if (!x || !wpack || !out || !chan_width(C) || V < 1 || !err || !aligned16(wpack) || (zp && !z)) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  if (ws::gate_fwd_supported(C)) return ws::gate_fwd(x, V, C, wpack, zp, z, out, err, s);
  if (C == C96) {
    if (!aligned32(x)) return FFNO_EINVAL;   // rows are read 32 bytes a request
    const size_t smem = 2 * mat_bytes(C96, C96) + 2 * tile_bytes(C96);
    if (!launch_prep(k_gate_tc<C96>, smem)) return FFNO_ELAUNCH;
    k_gate_tc<C96><<<grid_tc(V), CT, smem, s>>>(x, V, static_cast<const uint8_t*>(wpack), zp, z, out, err);
    FFNO_CHECK_LAUNCH();
    return FFNO_OK;
  }
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
  if (!x || !spec_pre || !spec_coefs || !vert_pre || !vert_coefs || !wpack || !bias) return FFNO_EINVAL;
  if (!chan_width(C) || V < 1 || !err || !aligned16(wpack) || !gates) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  if (C == C96) {
    if (!aligned32(x) || !aligned32(spec_pre) || !aligned32(vert_pre) || !aligned32(gates) || (hg && !aligned32(hg)))
      return FFNO_EINVAL;
    const size_t smem = mat_bytes(C96, 3 * C96) + mat_bytes(2 * C96, C96) + tile_bytes(KS);
    if (!launch_prep(k_fuse1_tc96, smem)) return FFNO_ELAUNCH;
    k_fuse1_tc96<<<grid_tc(V), PT, smem, s>>>(x, spec_pre, spec_coefs, vert_pre, vert_coefs, V,
                                             static_cast<const uint8_t*>(wpack), bias, gates, hg, err);
    FFNO_CHECK_LAUNCH();
    return FFNO_OK;
  }
  if (ws::fuse1_supported(C))
    return ws::fuse1(x, spec_pre, spec_coefs, vert_pre, vert_coefs, V, C, wpack, bias, gates, hg, err, s);
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
  if (!spec_pre || !spec_coefs || !vert_pre || !vert_coefs || !gates || !wpack || !dw || !pre || !partials)
    return FFNO_EINVAL;
  if (!tc_width(C) || V < 1 || !err || !aligned16(wpack) || groups != GMAX || nparts != grid_tc(V)) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  if (ws::fuse2_supported(C))
    return ws::fuse2(spec_pre, spec_coefs, vert_pre, vert_coefs, gates, V, C, wpack, dw, pre, partials, nparts, err,
                     s);
  if (!aligned32(spec_pre) || !aligned32(vert_pre) || !aligned32(gates)) return FFNO_EINVAL;   // 32-byte fills
  TC_DISPATCH(C, {
    const size_t smem = mat_bytes(2 * CC, 2 * CC) + mat_bytes(CC, 2 * CC) + 2 * tile_bytes(2 * CC);
    if (!launch_prep(k_fuse2_tc<CC>, smem)) return FFNO_ELAUNCH;
    k_fuse2_tc<CC><<<nparts, CT, smem, s>>>(spec_pre, spec_coefs, vert_pre, vert_coefs, gates, V,
                                           static_cast<const uint8_t*>(wpack), dw, pre, partials, err);
  })
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_fuse_hidden_tc(const float* spec_pre, const float* spec_coefs, const float* vert_pre, const float* vert_coefs,
                        const float* gates, long V, int C, const void* wpack, float* hf, int* err,
                        ffno_stream_t stream) {
  if (!spec_pre || !spec_coefs || !vert_pre || !vert_coefs || !gates || !wpack || !hf || !err) return FFNO_EINVAL;
  if (C != C96 || V < 1 || !aligned16(wpack)) return FFNO_EINVAL;
  if (!aligned32(spec_pre) || !aligned32(vert_pre) || !aligned32(gates) || !aligned32(hf)) return FFNO_EINVAL;
  const size_t smem = mat_bytes(2 * C96, 2 * C96) + tile_bytes(KS);
  if (!launch_prep(k_fuse_hidden_tc96, smem)) return FFNO_ELAUNCH;
  k_fuse_hidden_tc96<<<grid_tc(V), PT, smem, (cudaStream_t)stream>>>(spec_pre, spec_coefs, vert_pre, vert_coefs,
                                                                     gates, V, static_cast<const uint8_t*>(wpack), hf,
                                                                     err);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_fuse_out_tc(const float* spec_pre, const float* spec_coefs, const float* vert_pre, const float* vert_coefs,
                     const float* gates, const float* hf, long V, int C, const void* wpack, const float* dw,
                     float* pre, double* partials, int nparts, int groups, int* err, ffno_stream_t stream) {
  if (!spec_pre || !spec_coefs || !vert_pre || !vert_coefs || !gates || !hf || !wpack || !dw || !pre || !partials ||
      !err)
    return FFNO_EINVAL;
  if (C != C96 || V < 1 || !aligned16(wpack) || groups != GMAX || nparts != grid_tc(V)) return FFNO_EINVAL;
  if (!aligned32(spec_pre) || !aligned32(vert_pre) || !aligned32(gates) || !aligned32(hf) || !aligned32(pre))
    return FFNO_EINVAL;
  const size_t smem = mat_bytes(C96, 2 * C96) + tile_bytes(KS);
  if (!launch_prep(k_fuse_out_tc96, smem)) return FFNO_ELAUNCH;
  k_fuse_out_tc96<<<nparts, PT, smem, (cudaStream_t)stream>>>(spec_pre, spec_coefs, vert_pre, vert_coefs, gates, hf, V,
                                                              static_cast<const uint8_t*>(wpack), dw, pre, partials,
                                                              err);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_fuse_bwd_h_tc(const float* fused_pre_bar, const float* hf, long V, int C, const void* wpack, float* hf_bar,
                       int* err, ffno_stream_t stream) {
  if (!fused_pre_bar || !hf || !wpack || !hf_bar || !err) return FFNO_EINVAL;
  if (C != C96 || V < 1 || !aligned16(wpack)) return FFNO_EINVAL;
  if (!aligned32(fused_pre_bar) || !aligned32(hf) || !aligned32(hf_bar)) return FFNO_EINVAL;
  const size_t smem = mat_bytes(C96, 2 * C96) + tile_bytes(KS);
  if (!launch_prep(k_fuse_bwd_h_tc96, smem)) return FFNO_ELAUNCH;
  k_fuse_bwd_h_tc96<<<grid_tc(V), PT, smem, (cudaStream_t)stream>>>(fused_pre_bar, hf, V,
                                                                    static_cast<const uint8_t*>(wpack), hf_bar, err);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_fuse_bwd_q_tc(const float* spec_pre, const float* spec_coefs, const float* vert_pre, const float* vert_coefs,
                       const float* gates, const float* fused_pre_bar, const float* hf_bar, long V, int C,
                       const void* wpack, float* spec_bar, float* vert_bar, float* q, int* err, ffno_stream_t stream) {
  if (!spec_pre || !spec_coefs || !vert_pre || !vert_coefs || !gates || !fused_pre_bar || !hf_bar || !wpack ||
      !spec_bar || !vert_bar || !q || !err)
    return FFNO_EINVAL;
  if (C != C96 || V < 1 || !aligned16(wpack)) return FFNO_EINVAL;
  if (!aligned32(spec_pre) || !aligned32(vert_pre) || !aligned32(gates) || !aligned32(fused_pre_bar) ||
      !aligned32(hf_bar) || !aligned32(spec_bar) || !aligned32(vert_bar) || !aligned32(q))
    return FFNO_EINVAL;
  const size_t smem = mat_bytes(2 * C96, 2 * C96) + tile_bytes(KS);
  if (!launch_prep(k_fuse_bwd_q_tc96, smem)) return FFNO_ELAUNCH;
  k_fuse_bwd_q_tc96<<<grid_tc(V), PT, smem, (cudaStream_t)stream>>>(spec_pre, spec_coefs, vert_pre, vert_coefs, gates,
                                                                    fused_pre_bar, hf_bar, V,
                                                                    static_cast<const uint8_t*>(wpack), spec_bar,
                                                                    vert_bar, q, err);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_fuse_bwd_x_tc(const float* q, const float* hg, const float* base, long V, int C, const void* wpack,
                       float* x_bar, float* spec_bar, float* vert_bar, int* err, ffno_stream_t stream) {
  if (!q || !hg || !wpack || !x_bar || !spec_bar || !vert_bar || !err) return FFNO_EINVAL;
  if (C != C96 || V < 1 || !aligned16(wpack)) return FFNO_EINVAL;
  if (!aligned32(q) || !aligned32(hg) || (base && !aligned32(base)) || !aligned32(x_bar) || !aligned32(spec_bar) ||
      !aligned32(vert_bar))
    return FFNO_EINVAL;
  const size_t smem = mat_bytes(C96, 3 * C96) + mat_bytes(2 * C96, C96) + tile_bytes(KS);
  if (!launch_prep(k_fuse_bwd_x_tc96, smem)) return FFNO_ELAUNCH;
  k_fuse_bwd_x_tc96<<<grid_tc(V), PT, smem, (cudaStream_t)stream>>>(q, hg, base, V, static_cast<const uint8_t*>(wpack),
                                                                    x_bar, spec_bar, vert_bar, err);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_mlp2_bwd_tc(const float* a, const float* pre_bar, const float* base, long V, int C, const void* wpack,
                     float* a_bar, int* err, ffno_stream_t stream) {
  if (!a || !pre_bar || !wpack || !a_bar || !chan_width(C) || V < 1 || !err || !aligned16(wpack)) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  if (C == C96) {
    if (!aligned32(a) || !aligned32(pre_bar) || !aligned32(a_bar) || (base && !aligned32(base))) return FFNO_EINVAL;
    const size_t smem = mat_bytes(2 * C96, C96) + mat_bytes(C96, 2 * C96) + tile_bytes(C96);
    if (!launch_prep(k_mlp2_bwd_tc96, smem)) return FFNO_ELAUNCH;
    k_mlp2_bwd_tc96<<<grid_tc(V), PT, smem, s>>>(a, pre_bar, base, V, static_cast<const uint8_t*>(wpack), a_bar, err);
    FFNO_CHECK_LAUNCH();
    return FFNO_OK;
  }
  if (ws::mlp2_bwd_supported(C)) return ws::mlp2_bwd(a, pre_bar, base, V, C, wpack, a_bar, err, s);
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
  if (!x || !g_bar || !wpack || !x_bar) return FFNO_EINVAL;
  if (!chan_width(C) || V < 1 || !err || !aligned16(wpack) || (zp && !z_bar)) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  if (ws::gate_bwd_supported(C)) return ws::gate_bwd(x, g_bar, base, V, C, wpack, zp, x_bar, z_bar, err, s);
  if (C == C96) {
    if (!aligned32(x)) return FFNO_EINVAL;
    const size_t smem = 2 * mat_bytes(C96, C96) + 2 * tile_bytes(C96);   // one pipeline; pack [g1, g2]
    if (!launch_prep(k_gate_bwd_tc<C96, 1>, smem)) return FFNO_ELAUNCH;
    k_gate_bwd_tc<C96, 1><<<grid_tc(V), PT, smem, s>>>(x, g_bar, base, V, static_cast<const uint8_t*>(wpack), zp,
                                                       x_bar, z_bar, err);
    FFNO_CHECK_LAUNCH();
    return FFNO_OK;
  }
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
  if (!spec_pre || !spec_coefs || !vert_pre || !vert_coefs || !gates || !fused_pre_bar || !wpack || !hf_bar)
    return FFNO_EINVAL;
  if (!tc_width(C) || V < 1 || !err || !aligned16(wpack)) return FFNO_EINVAL;
  // the operand fills read 32 bytes of a row per request
  if (!aligned32(spec_pre) || !aligned32(vert_pre) || !aligned32(gates) || !aligned32(fused_pre_bar))
    return FFNO_EINVAL;
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
  if (!spec_pre || !spec_coefs || !vert_pre || !vert_coefs || !gates || !hg || !fused_pre_bar || !hf_bar || !wpack ||
      !x_bar || !spec_bar || !vert_bar)
    return FFNO_EINVAL;
  if (!tc_width(C) || V < 1 || !err || !aligned16(wpack)) return FFNO_EINVAL;
  // the epilogues move 32 bytes of a row per request
  if (!aligned32(spec_pre) || !aligned32(vert_pre) || !aligned32(gates) || !aligned32(hg) ||
      !aligned32(fused_pre_bar) || !aligned32(hf_bar) || (base && !aligned32(base)) || !aligned32(x_bar) ||
      !aligned32(spec_bar) || !aligned32(vert_bar))
    return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  TC_DISPATCH(C, {
    const size_t smem =
        mat_bytes(2 * CC, 2 * CC) + mat_bytes(CC, 2 * CC) + mat_bytes(3 * CC, CC) + 2 * tile_bytes(CC);
    if (!launch_prep(k_fuse_bwd_b_tc<CC>, smem)) return FFNO_ELAUNCH;
    k_fuse_bwd_b_tc<CC><<<grid_tc(V), CT, smem, s>>>(spec_pre, spec_coefs, vert_pre, vert_coefs, gates, hg,
                                                    fused_pre_bar, hf_bar, base, V,
                                                    static_cast<const uint8_t*>(wpack), x_bar, spec_bar, vert_bar,
                                                    err);
  })
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

// head parameters the tensor-core head kernels accept: species and levels within the kernels' fixed arrays, and
// nh = sum (levels + 1) head channels within nhp
static bool head_ok(const ffno_head_params* hp, int nh, int nhp) {
  if (!hp || (nhp != 16 && nhp != 32) || hp->nspecies < 1 || hp->nspecies > FFNO_MAX_SPECIES) return false;
  if (hp->in_channels < 1 || hp->in_channels > 8) return false;
  int tot = 0, lv = 0;
  for (int s = 0; s < hp->nspecies; ++s) {
    if (hp->levels[s] < 1) return false;
    tot += hp->levels[s] + 1;
    lv += hp->levels[s];
  }
  const int ch[3] = {hp->temperature_channel, hp->ne_channel, hp->rho_channel};
  for (int c : ch)
    if (c < 0 || c >= hp->in_channels) return false;
  return lv <= FFNO_MAX_LEVELS && tot <= nhp && (nh < 0 || tot == nh);
}

#define HEAD_DISPATCH(KERNEL, SMEM, ...)                                                     \
  TC_DISPATCH(C, {                                                                           \
    if (nhp == 16) {                                                                         \
      constexpr int NN = 16;                                                                 \
      if (params->math32) {                                                                  \
        if (!launch_prep(KERNEL<CC, NN, float>, SMEM)) return FFNO_ELAUNCH;                  \
        KERNEL<CC, NN, float><<<grid_tc(V), CT, SMEM, s>>>(__VA_ARGS__);                     \
      } else {                                                                               \
        if (!launch_prep(KERNEL<CC, NN, double>, SMEM)) return FFNO_ELAUNCH;                 \
        KERNEL<CC, NN, double><<<grid_tc(V), CT, SMEM, s>>>(__VA_ARGS__);                    \
      }                                                                                      \
    } else {                                                                                 \
      constexpr int NN = 32;                                                                 \
      if (params->math32) {                                                                  \
        if (!launch_prep(KERNEL<CC, NN, float>, SMEM)) return FFNO_ELAUNCH;                  \
        KERNEL<CC, NN, float><<<grid_tc(V), CT, SMEM, s>>>(__VA_ARGS__);                     \
      } else {                                                                               \
        if (!launch_prep(KERNEL<CC, NN, double>, SMEM)) return FFNO_ELAUNCH;                 \
        KERNEL<CC, NN, double><<<grid_tc(V), CT, SMEM, s>>>(__VA_ARGS__);                    \
      }                                                                                      \
    }                                                                                        \
  })

#define HEAD96(KERNEL, SMEM, ...)                                                                    \
  if (nhp == 16) {                                                                                  \
    if (params->math32) {                                                                           \
      if (!launch_prep(KERNEL<16, float>, SMEM)) return FFNO_ELAUNCH;                               \
      KERNEL<16, float><<<grid_tc(V), PT, SMEM, s>>>(__VA_ARGS__);                                  \
    } else {                                                                                        \
      if (!launch_prep(KERNEL<16, double>, SMEM)) return FFNO_ELAUNCH;                              \
      KERNEL<16, double><<<grid_tc(V), PT, SMEM, s>>>(__VA_ARGS__);                                 \
    }                                                                                               \
  } else {                                                                                          \
    if (params->math32) {                                                                           \
      if (!launch_prep(KERNEL<32, float>, SMEM)) return FFNO_ELAUNCH;                               \
      KERNEL<32, float><<<grid_tc(V), PT, SMEM, s>>>(__VA_ARGS__);                                  \
    } else {                                                                                        \
      if (!launch_prep(KERNEL<32, double>, SMEM)) return FFNO_ELAUNCH;                              \
      KERNEL<32, double><<<grid_tc(V), PT, SMEM, s>>>(__VA_ARGS__);                                 \
    }                                                                                               \
  }

int ffno_head_fwd_tc(const float* x, const float* x_in, long V, int C, const void* wpack, const float* b2, int nh,
                     int nhp, const ffno_head_params* params, float* out, float* head_out, int* err,
                     ffno_stream_t stream) {
  if (!chan_width(C) || V < 1 || !x || !x_in || !wpack || !b2 || !out || !err || !aligned16(wpack)) return FFNO_EINVAL;
  if (!aligned32(x)) return FFNO_EINVAL;   // the hidden rows are read 32 bytes a request
  if (!head_ok(params, nh, nhp)) return FFNO_EINVAL;
  const uint8_t* w = static_cast<const uint8_t*>(wpack);
  cudaStream_t s = (cudaStream_t)stream;
  if (C == C96) {
    HEAD96(k_head_tc96, mat_bytes(2 * C96, C96) + mat_bytes(nhp, 2 * C96) + tile_bytes(KS),
           x, x_in, V, w, b2, nh, *params, out, head_out, err)
    FFNO_CHECK_LAUNCH();
    return FFNO_OK;
  }
  HEAD_DISPATCH(k_head_tc,
                mat_bytes(2 * CC, CC) + mat_bytes(NN, 2 * CC) + 2 * (size_t)head_region(CC, NN, false),
                x, x_in, V, w, b2, nh, *params, out, head_out, err)
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_head_bwd_tc(const float* x, const float* x_in, const float* y_bar, long V, int C, const void* wpack,
                     const float* b2, int nhp, const ffno_head_params* params, float* x_bar, float* x_in_bar,
                     int* err, ffno_stream_t stream) {
  if (!chan_width(C) || V < 1 || !x || !x_in || !y_bar || !wpack || !b2 || !x_bar || !x_in_bar || !err ||
      !aligned16(wpack) || !aligned32(x))
    return FFNO_EINVAL;
  if (!head_ok(params, -1, nhp)) return FFNO_EINVAL;
  const uint8_t* w = static_cast<const uint8_t*>(wpack);
  cudaStream_t s = (cudaStream_t)stream;
  if (C == C96) {   // the pack is the forward's [P1, P2]
    if (!aligned32(x_bar)) return FFNO_EINVAL;
    HEAD96(k_head_bwd_tc96, mat_bytes(2 * C96, C96) + mat_bytes(nhp, 2 * C96) + tile_bytes(KS),
           x, x_in, y_bar, V, w, b2, *params, x_bar, x_in_bar, err)
    FFNO_CHECK_LAUNCH();
    return FFNO_OK;
  }
  HEAD_DISPATCH(k_head_bwd_tc,
                2 * mat_bytes(2 * CC, CC) + 2 * mat_bytes(NN, 2 * CC) + 2 * (size_t)head_region(CC, NN, true),
                x, x_in, y_bar, V, w, b2, *params, x_bar, x_in_bar, err)
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

}  // extern "C"
