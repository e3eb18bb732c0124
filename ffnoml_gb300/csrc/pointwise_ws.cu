// Warp-specialised tensor-core form of the channel-MLP backward (the ffno_mlp2_bwd contract):
//   a_bar = base + ((pre_bar W2^T) * gelu'(a W1)) W1^T,   W1: [2C][C], W2: [C][2C], split-BF16 products.
//
// One persistent CTA per SM walks 128-voxel tiles with five roles that hand work to each other through mbarriers, so
// HBM reads, format conversion, tensor-core MMAs and the two epilogues of different tiles overlap:
//   warp 0       TMA: FP32 tiles of a and pre_bar ([128 voxels][32 channels] boxes, 128-byte swizzle) into a
//                two-stage shared-memory ring;
//   warp 1       MMA issue (one thread): GEMM1 D1 = a W1^T and GEMM2 D2 = pre_bar W2, then GEMM3 D3 = G W1;
//   warps 2-5    conversion: FP32 rows from the ring -> split BF16 (hi = bf16(x), lo = bf16(x - hi)) written straight
//                into tensor memory, where they are the A operands of GEMM1/2 (lane = voxel);
//   warps 6-13   epilogue 1: G = D2 * gelu'(D1), split and written back over D1 (per 16-feature chunk: 8 columns hi,
//                8 columns lo), the A operand of GEMM3;
//   warps 14-17  epilogue 2: a_bar = base + D3 to HBM.
// Tensor memory (512 columns): two A stages of 128 columns [a hi | a lo | pre_bar hi | pre_bar lo] (D3 of the stage's
// tile lands over its a half), D1 at 256, D2 at 384. Every wait is bounded; a time-out records a code in *err, the
// role stops, the others run into their own bounded waits, and the CTA frees tensor memory only after the last MMA
// commit and every issued TMA copy have been waited for.
#include "common.cuh"
#include "tc.cuh"
#include "ws.h"

using namespace ffno;

namespace {

constexpr int TM = 128;
constexpr int NWARPS = 18;
constexpr int NTHREADS = NWARPS * 32;
constexpr int W_TMA = 0, W_MMA = 1, W_CVT = 2, W_E1 = 6, W_E2 = 14;
constexpr uint32_t BOX_BYTES = TM * 32 * 4;   // one [128][32] FP32 box
constexpr uint32_t D1 = 256, D2 = 384;        // accumulator columns

__host__ __device__ constexpr uint32_t mat_bytes(int R, int K) { return (uint32_t)R * K * 2 * 2; }

struct Bars {
  uint64_t stg_full[2], stg_empty[2], a_full[2], a_empty[2], d3_full[2], d_full, g_full, w;
};

constexpr uint64_t WAIT_NS = 1000000000ull;   // one second: every legitimate wait here lasts microseconds

__device__ __forceinline__ bool wait_or_flag(uint64_t* bar, uint32_t parity, int* err, int code) {
  if (tc::mbar_wait_for(bar, parity, WAIT_NS)) return true;
  atomicExch(err, code);
  return false;
}

// The same for a whole warp (tcgen05.ld / st are warp-collective): the warp goes on only if every lane saw the phase.
__device__ __forceinline__ bool warp_wait(uint64_t* bar, uint32_t parity, int* err, int code) {
  const bool ok = __all_sync(0xffffffffu, tc::mbar_wait_for(bar, parity, WAIT_NS)) != 0;
  if (!ok && (threadIdx.x & 31) == 0) atomicExch(err, code);
  return ok;
}

// three split products into d: (A hi, B hi), (A hi, B lo), (A lo, B hi) for one 16-wide k step
__device__ __forceinline__ void mma3_ta(uint32_t d, uint32_t a_hi, uint32_t a_lo, uint64_t b_hi, uint64_t b_lo,
                                        uint32_t idesc, bool acc) {
  tc::mma_bf16_ta(d, a_hi, b_hi, idesc, acc ? 1u : 0u);
  tc::mma_bf16_ta(d, a_hi, b_lo, idesc, 1u);
  tc::mma_bf16_ta(d, a_lo, b_hi, idesc, 1u);
}

__device__ __forceinline__ uint8_t* align1024(uint8_t* p) {
  return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
}

// barrier of the four epilogue-2 warps (named barrier 1)
__device__ __forceinline__ void e2_sync() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

// The same barrier returning whether p holds in all four warps, so that they leave their tile loop together.
__device__ __forceinline__ bool e2_sync_and(bool p) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred pi, po;\n setp.ne.u32 pi, %1, 0;\n bar.red.and.pred po, 1, 128, pi;\n selp.u32 %0, 1, 0, po;\n}"
      : "=r"(r)
      : "r"((uint32_t)p)
      : "memory");
  return r != 0;
}

template <int C>
__global__ void __launch_bounds__(NTHREADS, 1)
    k_mlp2_bwd_ws(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_pb,
                  const float* __restrict__ base, long V, const uint8_t* __restrict__ wpack, float* __restrict__ abar,
                  int* __restrict__ err) {
  static_assert(C == 32 || C == 64, "widths 32 and 64");
  constexpr uint32_t B1 = mat_bytes(2 * C, C);   // each of w1 (2C x C), w2t (2C x C), w1t (C x 2C)
  constexpr uint32_t WB = 3 * B1;
  constexpr int NB = C / 32;                     // TMA boxes per tensor tile
  constexpr uint32_t XB = NB * BOX_BYTES;        // one tensor's FP32 tile
  constexpr uint32_t SB = 2 * XB;                // one ring stage: a, pre_bar
  static_assert(WB % 1024 == 0, "the ring must stay 1024-byte aligned (128-byte swizzle)");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* ring = smem + WB;
  __shared__ Bars bars;
  __shared__ uint32_t tslot;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) tc::tmem_alloc(&tslot, 512);
  if (threadIdx.x == 0) {
    for (int s = 0; s < 2; ++s) {
      tc::mbar_init(&bars.stg_full[s], 1);
      tc::mbar_init(&bars.stg_empty[s], 128);
      tc::mbar_init(&bars.a_full[s], 128);
      tc::mbar_init(&bars.a_empty[s], 128);
      tc::mbar_init(&bars.d3_full[s], 1);
    }
    tc::mbar_init(&bars.d_full, 1);
    tc::mbar_init(&bars.g_full, 256);
    tc::mbar_init(&bars.w, 1);
    tc::mbar_init_fence();
  }
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  const uint32_t tmem = tslot;
  if (threadIdx.x == 0) {
    tc::mbar_arrive_expect_tx(&bars.w, WB);
    for (uint32_t off = 0; off < WB; off += 32768u)
      tc::bulk_g2s(smem + off, wpack + off, WB - off < 32768u ? WB - off : 32768u, &bars.w);
  }
  const bool ok = __syncthreads_and(tc::mbar_wait_for(&bars.w, 0, WAIT_NS)) != 0;
  if (!ok && threadIdx.x == 0) atomicExch(err, 1);

  const long nt = (V + TM - 1) / TM;
  const int niter = (long)blockIdx.x < nt ? (int)((nt - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  auto tile_of = [&](int i) { return (long)blockIdx.x + (long)i * gridDim.x; };

  if (ok && warp == W_TMA && lane == 0) {
    int issued[2] = {0, 0};
    for (int i = 0; i < niter; ++i) {
      const int s = i & 1;
      const uint32_t n = (uint32_t)i >> 1;
      if (!wait_or_flag(&bars.stg_empty[s], (n & 1u) ^ 1u, err, 3)) break;
      const int row = (int)(tile_of(i) * TM);
      tc::mbar_arrive_expect_tx(&bars.stg_full[s], SB);
      uint8_t* st = ring + s * SB;
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        tc::tma_load_2d(st + b * BOX_BYTES, &map_a, 32 * b, row, &bars.stg_full[s]);
        tc::tma_load_2d(st + XB + b * BOX_BYTES, &map_pb, 32 * b, row, &bars.stg_full[s]);
      }
      ++issued[s];
    }
    for (int s = 0; s < 2; ++s)   // every copy has landed before the CTA may exit
      if (issued[s]) tc::mbar_wait_for(&bars.stg_full[s], (uint32_t)(issued[s] - 1) & 1u, WAIT_NS);
  } else if (ok && warp == W_MMA && lane == 0) {
    const uint32_t i12 = tc::idesc_bf16(128, 2 * C), i3 = tc::idesc_bf16(128, C);
    const uint32_t w1 = tc::smem_u32(smem), w2t = w1 + B1, w1t = w1 + 2 * B1, LO = B1 / 2;
    uint64_t* last = nullptr;   // the last commit's barrier and phase parity, waited for before exit
    uint32_t last_par = 0;
    bool last_seen = true;
    for (int i = 0; i < niter; ++i) {
      const int s = i & 1;
      const uint32_t n = (uint32_t)i >> 1;
      if (!wait_or_flag(&bars.a_full[s], n & 1u, err, 4)) break;
      if (i > 0) {   // GEMM3 of the previous tile has read G out of D1
        if (!wait_or_flag(&bars.d3_full[(i - 1) & 1], ((uint32_t)(i - 1) >> 1) & 1u, err, 5)) break;
        last_seen = true;
      }
      tc::tc_after_sync();
      const uint32_t A = tmem + (uint32_t)(128 * s);
#pragma unroll 1
      for (int k = 0; k < C / 16; ++k) {
        const uint32_t ah = A + 8u * k, al = A + C / 2 + 8u * k;
        const uint32_t ph = A + C + 8u * k, pl = A + C + C / 2 + 8u * k;
        const uint32_t bo = 256u * k;
        mma3_ta(tmem + D1, ah, al, tc::kmajor_desc(w1 + bo, 128u, C * 16u), tc::kmajor_desc(w1 + LO + bo, 128u, C * 16u),
                i12, k > 0);
        mma3_ta(tmem + D2, ph, pl, tc::kmajor_desc(w2t + bo, 128u, C * 16u),
                tc::kmajor_desc(w2t + LO + bo, 128u, C * 16u), i12, k > 0);
      }
      tc::mma_commit(&bars.d_full);
      last = &bars.d_full;
      last_par = (uint32_t)i & 1u;
      last_seen = false;
      if (!wait_or_flag(&bars.g_full, (uint32_t)i & 1u, err, 6)) break;
      tc::tc_after_sync();
#pragma unroll 1
      for (int j = 0; j < 2 * C / 16; ++j) {
        const uint32_t bo = 256u * j;
        mma3_ta(tmem + (uint32_t)(128 * s), tmem + D1 + 16u * j, tmem + D1 + 16u * j + 8u,
                tc::kmajor_desc(w1t + bo, 128u, 2 * C * 16u), tc::kmajor_desc(w1t + LO + bo, 128u, 2 * C * 16u), i3,
                j > 0);
      }
      tc::mma_commit(&bars.d3_full[s]);
      last = &bars.d3_full[s];
      last_par = n & 1u;
      last_seen = false;
    }
    if (last && !last_seen) tc::mbar_wait_for(last, last_par, WAIT_NS);   // no MMA in flight when tensor memory is freed
  } else if (ok && warp >= W_CVT && warp < W_E1) {
    const int q = warp & 3, r = 32 * q + lane;
    const uint32_t lq = (uint32_t)(32 * q) << 16;
    for (int i = 0; i < niter; ++i) {
      const int s = i & 1;
      const uint32_t n = (uint32_t)i >> 1;
      if (!warp_wait(&bars.stg_full[s], n & 1u, err, 7)) break;
      if (!warp_wait(&bars.a_empty[s], (n & 1u) ^ 1u, err, 8)) break;
      tc::tc_after_sync();
      const uint8_t* st = ring + s * SB;
      const uint32_t A = tmem + lq + (uint32_t)(128 * s);
#pragma unroll
      for (int x = 0; x < 2; ++x)
#pragma unroll
        for (int b = 0; b < NB; ++b) {
          const uint8_t* rowp = st + x * XB + b * BOX_BYTES + r * 128;
          uint32_t hi[16], lo[16];
#pragma unroll
          for (int c = 0; c < 8; ++c) {
            const float4 v = *reinterpret_cast<const float4*>(rowp + ((c ^ (r & 7)) << 4));
            tc::split_pack(v.x, v.y, hi[2 * c], lo[2 * c]);
            tc::split_pack(v.z, v.w, hi[2 * c + 1], lo[2 * c + 1]);
          }
          tc::tmem_st16u(A + (uint32_t)(x * C + 16 * b), hi);
          tc::tmem_st16u(A + (uint32_t)(x * C + C / 2 + 16 * b), lo);
        }
      tc::mbar_arrive(&bars.stg_empty[s]);
      tc::tmem_wait_st();
      tc::tc_before_sync();
      tc::mbar_arrive(&bars.a_full[s]);
    }
  } else if (ok && warp >= W_E1 && warp < W_E2) {
    const int q = warp & 3, hf = (warp - W_E1) >> 2;
    const uint32_t lq = (uint32_t)(32 * q) << 16;
    for (int i = 0; i < niter; ++i) {
      if (!warp_wait(&bars.d_full, (uint32_t)i & 1u, err, 9)) break;
      tc::tc_after_sync();
#pragma unroll 1
      for (int j = hf; j < 2 * C / 16; j += 2) {
        uint32_t h[16], gb[16];
        tc::tmem_ld16u(tmem + lq + D1 + 16u * j, h);
        tc::tmem_ld16u(tmem + lq + D2 + 16u * j, gb);
        tc::tmem_wait_ld();
        uint32_t hi[8], lo[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
          const float g0 = __uint_as_float(gb[2 * e]) * gelu_grad_tc(__uint_as_float(h[2 * e]));
          const float g1 = __uint_as_float(gb[2 * e + 1]) * gelu_grad_tc(__uint_as_float(h[2 * e + 1]));
          tc::split_pack(g0, g1, hi[e], lo[e]);
        }
        tc::tmem_st8u(tmem + lq + D1 + 16u * j, hi);
        tc::tmem_st8u(tmem + lq + D1 + 16u * j + 8u, lo);
      }
      tc::tmem_wait_st();
      tc::tc_before_sync();
      tc::mbar_arrive(&bars.g_full);
    }
  } else if (ok && warp >= W_E2) {
    const int q = warp & 3, r = 32 * q + lane;
    const uint32_t lq = (uint32_t)(32 * q) << 16;
    for (int i = 0; i < niter; ++i) {
      const int s = i & 1;
      const uint32_t n = (uint32_t)i >> 1;
      const long v = tile_of(i) * TM + r;
      const bool live = v < V;
      float bv[C];
#pragma unroll
      for (int c = 0; c < C; c += 8) {
        if (base && live) {
          tc::ld8(base + v * C + c, bv + c);
        } else {
#pragma unroll
          for (int e = 0; e < 8; ++e) bv[c + e] = 0.f;
        }
      }
      if (!warp_wait(&bars.d3_full[s], n & 1u, err, 10)) break;
      tc::tc_after_sync();
#pragma unroll
      for (int k = 0; k < C / 16; ++k) {
        uint32_t d[16];
        tc::tmem_ld16u(tmem + lq + (uint32_t)(128 * s + 16 * k), d);
        tc::tmem_wait_ld();
        if (k == C / 16 - 1) {   // the stage's tensor memory is free once D3 is in registers
          tc::tc_before_sync();
          tc::mbar_arrive(&bars.a_empty[s]);
        }
        if (live) {
          float o[16];
#pragma unroll
          for (int e = 0; e < 16; ++e) o[e] = bv[16 * k + e] + __uint_as_float(d[e]);
          tc::st8(abar + v * C + 16 * k, o);
          tc::st8(abar + v * C + 16 * k + 8, o + 8);
        }
      }
    }
  }
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  if (warp == 0) tc::tmem_free(tmem, 512);
}

// ================================================================================================ forward
// The ffno_mlp2_fwd contract: pre = W2 gelu(W1 x) with x = in (MODE 0) or x = in + res act(GN(prev)) written to xout
// (MODE 1: act = GELU, MODE 2: identity), and the depth-weighted GroupNorm partials of pre (one per CTA, its tiles
// merged in order with Chan's update, so the statistics do not depend on timing). Roles as in the backward:
//   warp 0 TMA ring of in [and prev]; warp 1 MMA: GEMM1 D1[t % 2] = x W1^T (N = 2C), and GEMM2 D2 = H W2^T (N = C)
//   one tile behind, so that epilogue 1 of a tile overlaps GEMM1 of the next; warps 2-5 conversion with the residual
//   prologue (xout); warps 6-13 epilogue 1: H = gelu(D1), split over D1; warps 14-17 epilogue 2: pre and statistics.
// Tensor memory: four A stages of C columns from column 0 ([x hi | x lo], D2 of the stage's tile over them: a stage is
// held from conversion to epilogue 2), D1 buffers at 256 and 384.
template <int C, int MODE>
__global__ void __launch_bounds__(NTHREADS, 1)
    k_mlp2_fwd_ws(const __grid_constant__ CUtensorMap map_in, const __grid_constant__ CUtensorMap map_prev,
                  const float* __restrict__ pc, float res, float* __restrict__ xout, long V,
                  const uint8_t* __restrict__ wpack, const float* __restrict__ dw, float* __restrict__ pre,
                  double* __restrict__ partials, int* __restrict__ err) {
  static_assert(C == 32 || C == 64, "widths 32 and 64");
  constexpr uint32_t B1 = mat_bytes(2 * C, C);   // w1 (2C x C); w2 (C x 2C) has the same size
  constexpr uint32_t WB = 2 * B1;
  constexpr int NB = C / 32, NX = MODE == 0 ? 1 : 2, CPG = C / GMAX;
  constexpr uint32_t XB = NB * BOX_BYTES, SB = NX * XB;
  static_assert(WB % 1024 == 0, "the ring must stay 1024-byte aligned (128-byte swizzle)");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint8_t* ring = smem + WB;
  constexpr int NA = 4;   // A stages
  __shared__ uint64_t stg_full[2], stg_empty[2], a_full[NA], a_empty[NA], d2_full[NA], d1_full[2], h_full[2], wbar;
  __shared__ uint32_t tslot;
  __shared__ float cf[3 * C];                 // GroupNorm coefficients of prev: mean, gamma rstd, beta
  __shared__ float red[4][GMAX + 1], gmean[GMAX], wsum;
  __shared__ double acc[GMAX * 3];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) tc::tmem_alloc(&tslot, 512);
  if (threadIdx.x == 0) {
    for (int s = 0; s < 2; ++s) {
      tc::mbar_init(&stg_full[s], 1);
      tc::mbar_init(&stg_empty[s], 128);
      tc::mbar_init(&d1_full[s], 1);
      tc::mbar_init(&h_full[s], 256);
    }
    for (int s = 0; s < NA; ++s) {
      tc::mbar_init(&a_full[s], 128);
      tc::mbar_init(&a_empty[s], 128);
      tc::mbar_init(&d2_full[s], 1);
    }
    tc::mbar_init(&wbar, 1);
    tc::mbar_init_fence();
  }
  if (MODE != 0)
    for (int e = threadIdx.x; e < 3 * C; e += NTHREADS) cf[e] = pc[e];
  if (threadIdx.x < GMAX * 3) acc[threadIdx.x] = 0.0;
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  const uint32_t tmem = tslot;
  if (threadIdx.x == 0) {
    tc::mbar_arrive_expect_tx(&wbar, WB);
    for (uint32_t off = 0; off < WB; off += 32768u)
      tc::bulk_g2s(smem + off, wpack + off, WB - off < 32768u ? WB - off : 32768u, &wbar);
  }
  const bool ok = __syncthreads_and(tc::mbar_wait_for(&wbar, 0, WAIT_NS)) != 0;
  if (!ok && threadIdx.x == 0) atomicExch(err, 1);

  const long nt = (V + TM - 1) / TM;
  const int niter = (long)blockIdx.x < nt ? (int)((nt - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  auto tile_of = [&](int i) { return (long)blockIdx.x + (long)i * gridDim.x; };

  if (ok && warp == W_TMA && lane == 0) {
    int issued[2] = {0, 0};
    for (int i = 0; i < niter; ++i) {
      const int s = i & 1;
      const uint32_t n = (uint32_t)i >> 1;
      if (!wait_or_flag(&stg_empty[s], (n & 1u) ^ 1u, err, 3)) break;
      const int row = (int)(tile_of(i) * TM);
      tc::mbar_arrive_expect_tx(&stg_full[s], SB);
      uint8_t* st = ring + s * SB;
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        tc::tma_load_2d(st + b * BOX_BYTES, &map_in, 32 * b, row, &stg_full[s]);
        if (MODE != 0) tc::tma_load_2d(st + XB + b * BOX_BYTES, &map_prev, 32 * b, row, &stg_full[s]);
      }
      ++issued[s];
    }
    for (int s = 0; s < 2; ++s)
      if (issued[s]) tc::mbar_wait_for(&stg_full[s], (uint32_t)(issued[s] - 1) & 1u, WAIT_NS);
  } else if (ok && warp == W_MMA && lane == 0) {
    const uint32_t i1 = tc::idesc_bf16(128, 2 * C), i2 = tc::idesc_bf16(128, C);
    const uint32_t w1 = tc::smem_u32(smem), w2 = w1 + B1, LO = B1 / 2;
    uint64_t* last = nullptr;
    uint32_t last_par = 0;
    bool alive = true;
    auto gemm2 = [&](int j) {   // D2 (A stage j % NA) = H(j) (in D1[j % 2]) W2^T, K = 2C
      const uint32_t h = tmem + 256u + 128u * (j & 1);
#pragma unroll 1
      for (int k = 0; k < 2 * C / 16; ++k)
        mma3_ta(tmem + (uint32_t)(C * (j % NA)), h + 16u * k, h + 16u * k + 8u,
                tc::kmajor_desc(w2 + 256u * k, 128u, 2 * C * 16u), tc::kmajor_desc(w2 + LO + 256u * k, 128u, 2 * C * 16u),
                i2, k > 0);
      tc::mma_commit(&d2_full[j % NA]);
      last = &d2_full[j % NA];
      last_par = (uint32_t)(j / NA) & 1u;
    };
    for (int i = 0; i < niter && alive; ++i) {
      const int s = i & 1, sa = i % NA;
      const uint32_t n = (uint32_t)i >> 1;
      if (!wait_or_flag(&a_full[sa], (uint32_t)(i / NA) & 1u, err, 4)) {
        alive = false;
        break;
      }
      if (i >= 2 && !wait_or_flag(&d2_full[(i - 2) % NA], (uint32_t)((i - 2) / NA) & 1u, err, 11)) {
        alive = false;   // GEMM2 of tile i-2, the last reader of D1[s], has completed
        break;
      }
      tc::tc_after_sync();
      const uint32_t A = tmem + (uint32_t)(C * sa), D = tmem + 256u + 128u * s;
#pragma unroll 1
      for (int k = 0; k < C / 16; ++k)
        mma3_ta(D, A + 8u * k, A + C / 2 + 8u * k, tc::kmajor_desc(w1 + 256u * k, 128u, C * 16u),
                tc::kmajor_desc(w1 + LO + 256u * k, 128u, C * 16u), i1, k > 0);
      tc::mma_commit(&d1_full[s]);
      last = &d1_full[s];
      last_par = n & 1u;
      if (i >= 1) {
        if (!wait_or_flag(&h_full[(i - 1) & 1], ((uint32_t)(i - 1) >> 1) & 1u, err, 5)) { alive = false; break; }
        tc::tc_after_sync();
        gemm2(i - 1);
      }
    }
    if (alive && niter >= 1) {
      const int j = niter - 1;
      if (wait_or_flag(&h_full[j & 1], ((uint32_t)j >> 1) & 1u, err, 6)) {
        tc::tc_after_sync();
        gemm2(j);
      }
    }
    if (last) tc::mbar_wait_for(last, last_par, WAIT_NS);   // no MMA in flight when tensor memory is freed
  } else if (ok && warp >= W_CVT && warp < W_E1) {
    const int q = warp & 3, r = 32 * q + lane;
    const uint32_t lq = (uint32_t)(32 * q) << 16;
    for (int i = 0; i < niter; ++i) {
      const int s = i & 1;
      const uint32_t n = (uint32_t)i >> 1;
      const int sa = i % NA;
      if (!warp_wait(&stg_full[s], n & 1u, err, 7)) break;
      if (!warp_wait(&a_empty[sa], ((uint32_t)(i / NA) & 1u) ^ 1u, err, 8)) break;
      tc::tc_after_sync();
      const uint8_t* st = ring + s * SB;
      const uint32_t A = tmem + lq + (uint32_t)(C * sa);
      const long v = tile_of(i) * TM + r;
#pragma unroll 1
      for (int bh = 0; bh < 2 * NB; ++bh) {   // half boxes: 16 channels, 8 hi and 8 lo columns
        const int b = bh >> 1;
        const uint8_t* rin = st + b * BOX_BYTES + r * 128;
        uint32_t hi[8], lo[8];
        float xs[16];   // the half box's 16 channels of x, stored to xout in two 32-byte requests
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) {
          const int c = 4 * (bh & 1) + cc;
          const uint32_t o = (uint32_t)((c ^ (r & 7)) << 4);
          float4 x = *reinterpret_cast<const float4*>(rin + o);
          if (MODE != 0) {
            const float4 p = *reinterpret_cast<const float4*>(rin + XB + o);
            const int k = 32 * b + 4 * c;
            float y[4] = {p.x, p.y, p.z, p.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              y[e] = (y[e] - cf[k + e]) * cf[C + k + e] + cf[2 * C + k + e];
              if (MODE == 1) y[e] = gelu_tc(y[e]);
            }
            x = make_float4(fmaf(res, y[0], x.x), fmaf(res, y[1], x.y), fmaf(res, y[2], x.z), fmaf(res, y[3], x.w));
            xs[4 * cc] = x.x;
            xs[4 * cc + 1] = x.y;
            xs[4 * cc + 2] = x.z;
            xs[4 * cc + 3] = x.w;
          }
          tc::split_pack(x.x, x.y, hi[2 * cc], lo[2 * cc]);
          tc::split_pack(x.z, x.w, hi[2 * cc + 1], lo[2 * cc + 1]);
        }
        if (MODE != 0 && v < V) {
          float* xo = xout + v * C + 32 * b + 16 * (bh & 1);
          tc::st8(xo, xs);
          tc::st8(xo + 8, xs + 8);
        }
        tc::tmem_st8u(A + (uint32_t)(8 * bh), hi);
        tc::tmem_st8u(A + (uint32_t)(C / 2 + 8 * bh), lo);
      }
      tc::mbar_arrive(&stg_empty[s]);
      tc::tmem_wait_st();
      tc::tc_before_sync();
      tc::mbar_arrive(&a_full[sa]);
    }
  } else if (ok && warp >= W_E1 && warp < W_E2) {
    const int q = warp & 3, hf = (warp - W_E1) >> 2;
    const uint32_t lq = (uint32_t)(32 * q) << 16;
    for (int i = 0; i < niter; ++i) {
      const int s = i & 1;
      const uint32_t n = (uint32_t)i >> 1;
      if (!warp_wait(&d1_full[s], n & 1u, err, 9)) break;
      tc::tc_after_sync();
      const uint32_t D = tmem + lq + 256u + 128u * s;
#pragma unroll 1
      for (int j = hf; j < 2 * C / 16; j += 2) {
        uint32_t h[16];
        tc::tmem_ld16u(D + 16u * j, h);
        tc::tmem_wait_ld();
        uint32_t hi[8], lo[8];
#pragma unroll
        for (int e = 0; e < 8; ++e)
          tc::split_pack(gelu_tc(__uint_as_float(h[2 * e])), gelu_tc(__uint_as_float(h[2 * e + 1])), hi[e], lo[e]);
        tc::tmem_st8u(D + 16u * j, hi);
        tc::tmem_st8u(D + 16u * j + 8u, lo);
      }
      tc::tmem_wait_st();
      tc::tc_before_sync();
      tc::mbar_arrive(&h_full[s]);
    }
  } else if (ok && warp >= W_E2) {
    const int q = warp & 3, r = 32 * q + lane, wl = warp - W_E2;
    const uint32_t lq = (uint32_t)(32 * q) << 16;
    for (int i = 0; i < niter; ++i) {
      const int sa = i % NA;
      const long v = tile_of(i) * TM + r;
      const bool live = v < V;
      const float w = live ? __ldg(dw + v) : 0.f;
      if (!e2_sync_and(tc::mbar_wait_for(&d2_full[sa], (uint32_t)(i / NA) & 1u, WAIT_NS))) {
        if (lane == 0) atomicExch(err, 10);
        break;
      }
      tc::tc_after_sync();
      // pass 1: pre to HBM and the weighted group sums (CPG = C / 8 channels per group; a 16-column chunk holds
      // 16 / CPG groups)
      const uint32_t D = tmem + lq + (uint32_t)(C * sa);
      float gs[GMAX];
#pragma unroll
      for (int k = 0; k < C / 16; ++k) {
        uint32_t d[16];
        tc::tmem_ld16u(D + 16u * k, d);
        tc::tmem_wait_ld();
        if (live) {
          float o[16];
#pragma unroll
          for (int e = 0; e < 16; ++e) o[e] = __uint_as_float(d[e]);
          tc::st8(pre + v * C + 16 * k, o);
          tc::st8(pre + v * C + 16 * k + 8, o + 8);
        }
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          const int g = (16 * k + e) / CPG;
          if (e % CPG == 0) gs[g] = 0.f;
          gs[g] += __uint_as_float(d[e]);
        }
      }
      float ws = w;
#pragma unroll
      for (int m = 16; m; m >>= 1) ws += __shfl_xor_sync(0xffffffffu, ws, m);
#pragma unroll
      for (int g = 0; g < GMAX; ++g) {
        float t = w * gs[g];
#pragma unroll
        for (int m = 16; m; m >>= 1) t += __shfl_xor_sync(0xffffffffu, t, m);
        if (lane == 0) red[wl][g] = t;
      }
      if (lane == 0) red[wl][GMAX] = ws;
      e2_sync();
      if (threadIdx.x - 32 * W_E2 < GMAX) {
        const int g = threadIdx.x - 32 * W_E2;
        const float wt = ((red[0][GMAX] + red[1][GMAX]) + (red[2][GMAX] + red[3][GMAX])) * CPG;
        gmean[g] = wt > 0.f ? ((red[0][g] + red[1][g]) + (red[2][g] + red[3][g])) / wt : 0.f;
        if (g == 0) wsum = wt;
      }
      e2_sync();
      // pass 2 (D2 read again from tensor memory): centred sums of squares
#pragma unroll
      for (int k = 0; k < C / 16; ++k) {
        uint32_t d[16];
        tc::tmem_ld16u(D + 16u * k, d);
        tc::tmem_wait_ld();
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          const int g = (16 * k + e) / CPG;
          if (e % CPG == 0) gs[g] = 0.f;
          const float x = __uint_as_float(d[e]) - gmean[g];
          gs[g] = fmaf(x, x, gs[g]);
        }
      }
      tc::tc_before_sync();
      tc::mbar_arrive(&a_empty[sa]);   // D2 has been read: the stage may take a new tile
#pragma unroll
      for (int g = 0; g < GMAX; ++g) {
        float t = w * gs[g];
#pragma unroll
        for (int m = 16; m; m >>= 1) t += __shfl_xor_sync(0xffffffffu, t, m);
        if (lane == 0) red[wl][g] = t;
      }
      e2_sync();
      if (threadIdx.x - 32 * W_E2 < GMAX) {
        const int g = threadIdx.x - 32 * W_E2;
        GroupAcc a{acc[3 * g], acc[3 * g + 1], acc[3 * g + 2]};
        chan_merge(a, (double)wsum, (double)gmean[g], (double)((red[0][g] + red[1][g]) + (red[2][g] + red[3][g])));
        acc[3 * g] = a.w;
        acc[3 * g + 1] = a.mean;
        acc[3 * g + 2] = a.m2;
      }
      e2_sync();
    }
  }
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  if (threadIdx.x < GMAX) {
    double* o = partials + ((long)blockIdx.x * GMAX + threadIdx.x) * 3;
    o[0] = acc[3 * threadIdx.x];
    o[1] = acc[3 * threadIdx.x + 1];
    o[2] = acc[3 * threadIdx.x + 2];
  }
  if (warp == 0) tc::tmem_free(tmem, 512);
}

// ================================================================================================ input gate
// The ffno_gate_fwd_tc contract: out = x sigmoid(gelu(x G1^T) G2^T) [+ zp z], G1, G2: [C][C]. Roles as in the forward
// MLP: warp 0 TMA ring of x; warp 1 MMA: GEMM1 D1[t % 2] = x G1^T, and GEMM2 D2 = H G2^T one tile behind; warps 2-5
// conversion into the A stages; warps 6-13 epilogue 1: H = gelu(D1), split over D1; warps 14-17 epilogue 2: the gate
// applied to the tile's x rows (loaded from HBM before D2 is waited for) and the z_proj term. Tensor memory: four A
// stages of C columns from column 0 (D2 of a stage's tile over them), D1 buffers at 256 and 256 + C.
template <int C>
__global__ void __launch_bounds__(NTHREADS, 1)
    k_gate_fwd_ws(const __grid_constant__ CUtensorMap map_x, const float* __restrict__ x, long V,
                  const uint8_t* __restrict__ wpack, const float* __restrict__ zp, const float* __restrict__ z,
                  float* __restrict__ out, int* __restrict__ err) {
  static_assert(C == 32 || C == 64, "widths 32 and 64");
  constexpr uint32_t B1 = mat_bytes(C, C);       // each of g1, g2
  constexpr uint32_t WB = 2 * B1;
  constexpr int NB = C / 32;
  constexpr uint32_t SB = NB * BOX_BYTES;        // one ring stage: x
  constexpr int NA = 4;                          // A stages
  static_assert(WB % 1024 == 0, "the ring must stay 1024-byte aligned (128-byte swizzle)");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint8_t* ring = smem + WB;
  __shared__ uint64_t stg_full[2], stg_empty[2], a_full[NA], a_empty[NA], d2_full[NA], d1_full[2], h_full[2], wbar;
  __shared__ uint32_t tslot;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) tc::tmem_alloc(&tslot, 512);
  if (threadIdx.x == 0) {
    for (int s = 0; s < 2; ++s) {
      tc::mbar_init(&stg_full[s], 1);
      tc::mbar_init(&stg_empty[s], 128);
      tc::mbar_init(&d1_full[s], 1);
      tc::mbar_init(&h_full[s], 256);
    }
    for (int s = 0; s < NA; ++s) {
      tc::mbar_init(&a_full[s], 128);
      tc::mbar_init(&a_empty[s], 128);
      tc::mbar_init(&d2_full[s], 1);
    }
    tc::mbar_init(&wbar, 1);
    tc::mbar_init_fence();
  }
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  const uint32_t tmem = tslot;
  if (threadIdx.x == 0) {
    tc::mbar_arrive_expect_tx(&wbar, WB);
    tc::bulk_g2s(smem, wpack, WB, &wbar);
  }
  const bool ok = __syncthreads_and(tc::mbar_wait_for(&wbar, 0, WAIT_NS)) != 0;
  if (!ok && threadIdx.x == 0) atomicExch(err, 1);

  const long nt = (V + TM - 1) / TM;
  const int niter = (long)blockIdx.x < nt ? (int)((nt - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  auto tile_of = [&](int i) { return (long)blockIdx.x + (long)i * gridDim.x; };
  constexpr uint32_t D1C = 256;

  if (ok && warp == W_TMA && lane == 0) {
    int issued[2] = {0, 0};
    for (int i = 0; i < niter; ++i) {
      const int s = i & 1;
      const uint32_t n = (uint32_t)i >> 1;
      if (!wait_or_flag(&stg_empty[s], (n & 1u) ^ 1u, err, 3)) break;
      const int row = (int)(tile_of(i) * TM);
      tc::mbar_arrive_expect_tx(&stg_full[s], SB);
      uint8_t* st = ring + s * SB;
#pragma unroll
      for (int b = 0; b < NB; ++b) tc::tma_load_2d(st + b * BOX_BYTES, &map_x, 32 * b, row, &stg_full[s]);
      ++issued[s];
    }
    for (int s = 0; s < 2; ++s)
      if (issued[s]) tc::mbar_wait_for(&stg_full[s], (uint32_t)(issued[s] - 1) & 1u, WAIT_NS);
  } else if (ok && warp == W_MMA && lane == 0) {
    const uint32_t id = tc::idesc_bf16(128, C);
    const uint32_t g1 = tc::smem_u32(smem), g2 = g1 + B1, LO = B1 / 2;
    uint64_t* last = nullptr;
    uint32_t last_par = 0;
    bool alive = true;
    auto gemm2 = [&](int j) {   // D2 (A stage j % NA) = H(j) (in D1[j % 2]) G2^T, K = C
      const uint32_t h = tmem + D1C + (uint32_t)(C * (j & 1));
#pragma unroll 1
      for (int k = 0; k < C / 16; ++k)
        mma3_ta(tmem + (uint32_t)(C * (j % NA)), h + 16u * k, h + 16u * k + 8u,
                tc::kmajor_desc(g2 + 256u * k, 128u, C * 16u), tc::kmajor_desc(g2 + LO + 256u * k, 128u, C * 16u),
                id, k > 0);
      tc::mma_commit(&d2_full[j % NA]);
      last = &d2_full[j % NA];
      last_par = (uint32_t)(j / NA) & 1u;
    };
    for (int i = 0; i < niter && alive; ++i) {
      const int s = i & 1, sa = i % NA;
      const uint32_t n = (uint32_t)i >> 1;
      if (!wait_or_flag(&a_full[sa], (uint32_t)(i / NA) & 1u, err, 4)) {
        alive = false;
        break;
      }
      if (i >= 2 && !wait_or_flag(&d2_full[(i - 2) % NA], (uint32_t)((i - 2) / NA) & 1u, err, 11)) {
        alive = false;   // GEMM2 of tile i-2, the last reader of D1[s], has completed
        break;
      }
      tc::tc_after_sync();
      const uint32_t A = tmem + (uint32_t)(C * sa), D = tmem + D1C + (uint32_t)(C * s);
#pragma unroll 1
      for (int k = 0; k < C / 16; ++k)
        mma3_ta(D, A + 8u * k, A + C / 2 + 8u * k, tc::kmajor_desc(g1 + 256u * k, 128u, C * 16u),
                tc::kmajor_desc(g1 + LO + 256u * k, 128u, C * 16u), id, k > 0);
      tc::mma_commit(&d1_full[s]);
      last = &d1_full[s];
      last_par = n & 1u;
      if (i >= 1) {
        if (!wait_or_flag(&h_full[(i - 1) & 1], ((uint32_t)(i - 1) >> 1) & 1u, err, 5)) { alive = false; break; }
        tc::tc_after_sync();
        gemm2(i - 1);
      }
    }
    if (alive && niter >= 1) {
      const int j = niter - 1;
      if (wait_or_flag(&h_full[j & 1], ((uint32_t)j >> 1) & 1u, err, 6)) {
        tc::tc_after_sync();
        gemm2(j);
      }
    }
    if (last) tc::mbar_wait_for(last, last_par, WAIT_NS);   // no MMA in flight when tensor memory is freed
  } else if (ok && warp >= W_CVT && warp < W_E1) {
    const int q = warp & 3, r = 32 * q + lane;
    const uint32_t lq = (uint32_t)(32 * q) << 16;
    for (int i = 0; i < niter; ++i) {
      const int s = i & 1;
      const uint32_t n = (uint32_t)i >> 1;
      const int sa = i % NA;
      if (!warp_wait(&stg_full[s], n & 1u, err, 7)) break;
      if (!warp_wait(&a_empty[sa], ((uint32_t)(i / NA) & 1u) ^ 1u, err, 8)) break;
      tc::tc_after_sync();
      const uint8_t* st = ring + s * SB;
      const uint32_t A = tmem + lq + (uint32_t)(C * sa);
#pragma unroll 1
      for (int bh = 0; bh < 2 * NB; ++bh) {   // half boxes: 16 channels, 8 hi and 8 lo columns
        const uint8_t* rin = st + (bh >> 1) * BOX_BYTES + r * 128;
        uint32_t hi[8], lo[8];
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) {
          const int c = 4 * (bh & 1) + cc;
          const float4 v = *reinterpret_cast<const float4*>(rin + ((c ^ (r & 7)) << 4));
          tc::split_pack(v.x, v.y, hi[2 * cc], lo[2 * cc]);
          tc::split_pack(v.z, v.w, hi[2 * cc + 1], lo[2 * cc + 1]);
        }
        tc::tmem_st8u(A + (uint32_t)(8 * bh), hi);
        tc::tmem_st8u(A + (uint32_t)(C / 2 + 8 * bh), lo);
      }
      tc::mbar_arrive(&stg_empty[s]);
      tc::tmem_wait_st();
      tc::tc_before_sync();
      tc::mbar_arrive(&a_full[sa]);
    }
  } else if (ok && warp >= W_E1 && warp < W_E2) {
    const int q = warp & 3, hf = (warp - W_E1) >> 2;
    const uint32_t lq = (uint32_t)(32 * q) << 16;
    for (int i = 0; i < niter; ++i) {
      const int s = i & 1;
      const uint32_t n = (uint32_t)i >> 1;
      if (!warp_wait(&d1_full[s], n & 1u, err, 9)) break;
      tc::tc_after_sync();
      const uint32_t D = tmem + lq + D1C + (uint32_t)(C * s);
#pragma unroll 1
      for (int j = hf; j < C / 16; j += 2) {
        uint32_t h[16];
        tc::tmem_ld16u(D + 16u * j, h);
        tc::tmem_wait_ld();
        uint32_t hi[8], lo[8];
#pragma unroll
        for (int e = 0; e < 8; ++e)
          tc::split_pack(gelu_tc(__uint_as_float(h[2 * e])), gelu_tc(__uint_as_float(h[2 * e + 1])), hi[e], lo[e]);
        tc::tmem_st8u(D + 16u * j, hi);
        tc::tmem_st8u(D + 16u * j + 8u, lo);
      }
      tc::tmem_wait_st();
      tc::tc_before_sync();
      tc::mbar_arrive(&h_full[s]);
    }
  } else if (ok && warp >= W_E2) {
    const int q = warp & 3, r = 32 * q + lane;
    const uint32_t lq = (uint32_t)(32 * q) << 16;
    for (int i = 0; i < niter; ++i) {
      const int sa = i % NA;
      const long v = tile_of(i) * TM + r;
      const bool live = v < V;
      float xv[C];
#pragma unroll
      for (int c = 0; c < C; c += 8) {
        if (live) {
          tc::ld8(x + v * C + c, xv + c);
        } else {
#pragma unroll
          for (int e = 0; e < 8; ++e) xv[c + e] = 0.f;
        }
      }
      const float zv = (zp && live) ? __ldg(z + v) : 0.f;
      if (!warp_wait(&d2_full[sa], (uint32_t)(i / NA) & 1u, err, 10)) break;
      tc::tc_after_sync();
#pragma unroll
      for (int k = 0; k < C / 16; ++k) {
        uint32_t d[16];
        tc::tmem_ld16u(tmem + lq + (uint32_t)(C * sa + 16 * k), d);
        tc::tmem_wait_ld();
        if (k == C / 16 - 1) {   // the stage's tensor memory is free once D2 is in registers
          tc::tc_before_sync();
          tc::mbar_arrive(&a_empty[sa]);
        }
        if (live) {
          float y[16];
#pragma unroll
          for (int e = 0; e < 16; ++e) y[e] = xv[16 * k + e] * sigmoid_tc(__uint_as_float(d[e]));
          if (zp)
#pragma unroll
            for (int e = 0; e < 16; ++e) y[e] = fmaf(__ldg(zp + 16 * k + e), zv, y[e]);
          tc::st8(out + v * C + 16 * k, y);
          tc::st8(out + v * C + 16 * k + 8, y + 8);
        }
      }
    }
  }
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  if (warp == 0) tc::tmem_free(tmem, 512);
}

// ================================================================================================ fuse, first half
// The ffno_fuse1_tc contract: gates [V][2C] = sigmoid(gelu(A Wg1^T) Wg2^T + bias), A = [x, gelu(GN_s(spec_pre)),
// gelu(GN_v(vert_pre))] (K = 3C), and hg [V][C] = A Wg1^T when hg is not NULL. Roles as in the forward MLP: warp 0 TMA,
// 3 NB phases of 32 channels per tile (x, spec_pre, vert_pre boxes) through a four-stage ring; warp 1 MMA: GEMM1
// D1[t % 2] = A Wg1^T (N = C), and GEMM2 D2 = H Wg2^T (N = 2C) one tile behind, over the tile's A stage; warps 2-5
// conversion; warps 6-13 epilogue 1: hg to HBM, H = gelu(D1) split over D1; warps 14-17 epilogue 2: the gates.
// Tensor memory: A stages of 3C columns at 0 and 3C, D1 buffers at 6C and 7C.
template <int C>
__global__ void __launch_bounds__(NTHREADS, 1)
    k_fuse1_ws(const __grid_constant__ CUtensorMap map_x, const __grid_constant__ CUtensorMap map_sp,
               const __grid_constant__ CUtensorMap map_vp, const float* __restrict__ sc, const float* __restrict__ vc,
               long V, const uint8_t* __restrict__ wpack, const float* __restrict__ bias, float* __restrict__ gates,
               float* __restrict__ hg, int* __restrict__ err) {
  static_assert(C == 32 || C == 64, "widths 32 and 64");
  constexpr uint32_t B1 = mat_bytes(C, 3 * C), B2 = mat_bytes(2 * C, C);
  constexpr uint32_t WB = B1 + B2;
  constexpr int NB = C / 32, NPH = 3 * NB, NS = 4;
  constexpr uint32_t SB = BOX_BYTES;             // one ring stage: one box
  constexpr uint32_t TD1 = 6 * C;
  static_assert(WB % 1024 == 0, "the ring must stay 1024-byte aligned (128-byte swizzle)");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint8_t* ring = smem + WB;
  __shared__ uint64_t stg_full[NS], stg_empty[NS], a_full[2], a_empty[2], d1_full[2], h_full[2], d2_full[2], wbar;
  __shared__ uint32_t tslot;
  __shared__ float cf[2][3 * C], bs[2 * C];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) tc::tmem_alloc(&tslot, 512);
  if (threadIdx.x == 0) {
    for (int s = 0; s < NS; ++s) {
      tc::mbar_init(&stg_full[s], 1);
      tc::mbar_init(&stg_empty[s], 128);
    }
    for (int s = 0; s < 2; ++s) {
      tc::mbar_init(&a_full[s], 128);
      tc::mbar_init(&a_empty[s], 128);
      tc::mbar_init(&d1_full[s], 1);
      tc::mbar_init(&h_full[s], 256);
      tc::mbar_init(&d2_full[s], 1);
    }
    tc::mbar_init(&wbar, 1);
    tc::mbar_init_fence();
  }
  for (int e = threadIdx.x; e < 3 * C; e += NTHREADS) {
    cf[0][e] = sc[e];
    cf[1][e] = vc[e];
  }
  for (int e = threadIdx.x; e < 2 * C; e += NTHREADS) bs[e] = bias[e];
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  const uint32_t tmem = tslot;
  if (threadIdx.x == 0) {
    tc::mbar_arrive_expect_tx(&wbar, WB);
    for (uint32_t off = 0; off < WB; off += 32768u)
      tc::bulk_g2s(smem + off, wpack + off, WB - off < 32768u ? WB - off : 32768u, &wbar);
  }
  const bool ok = __syncthreads_and(tc::mbar_wait_for(&wbar, 0, WAIT_NS)) != 0;
  if (!ok && threadIdx.x == 0) atomicExch(err, 1);

  const long nt = (V + TM - 1) / TM;
  const int niter = (long)blockIdx.x < nt ? (int)((nt - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  auto tile_of = [&](int i) { return (long)blockIdx.x + (long)i * gridDim.x; };

  if (ok && warp == W_TMA && lane == 0) {
    int issued[NS] = {0, 0, 0, 0};
    bool alive = true;
    for (int i = 0; i < niter && alive; ++i) {
      const int row = (int)(tile_of(i) * TM);
      for (int ph = 0; ph < NPH; ++ph) {
        const int u = i * NPH + ph, st = u % NS;
        const uint32_t n = (uint32_t)(u / NS);
        if (!wait_or_flag(&stg_empty[st], (n & 1u) ^ 1u, err, 3)) {
          alive = false;
          break;
        }
        tc::mbar_arrive_expect_tx(&stg_full[st], SB);
        const int t = ph / NB;
        tc::tma_load_2d(ring + st * SB, t == 0 ? &map_x : (t == 1 ? &map_sp : &map_vp), 32 * (ph % NB), row,
                        &stg_full[st]);
        ++issued[st];
      }
    }
    for (int s = 0; s < NS; ++s)
      if (issued[s]) tc::mbar_wait_for(&stg_full[s], (uint32_t)(issued[s] - 1) & 1u, WAIT_NS);
  } else if (ok && warp == W_MMA && lane == 0) {
    const uint32_t i1 = tc::idesc_bf16(128, C), i2 = tc::idesc_bf16(128, 2 * C);
    const uint32_t w1 = tc::smem_u32(smem), w2 = w1 + B1;
    uint64_t* last = nullptr;
    uint32_t last_par = 0;
    bool alive = true;
    auto gemm2 = [&](int j) {   // D2 (over A stage j % 2) = H(j) Wg2^T, H in D1[j % 2] as [hi 8 | lo 8], K = C
      const uint32_t h = tmem + TD1 + (uint32_t)(C * (j & 1));
#pragma unroll 1
      for (int k = 0; k < C / 16; ++k)
        mma3_ta(tmem + (uint32_t)(3 * C * (j & 1)), h + 16u * k, h + 16u * k + 8u,
                tc::kmajor_desc(w2 + 256u * k, 128u, C * 16u), tc::kmajor_desc(w2 + B2 / 2 + 256u * k, 128u, C * 16u),
                i2, k > 0);
      tc::mma_commit(&d2_full[j & 1]);
      last = &d2_full[j & 1];
      last_par = ((uint32_t)j >> 1) & 1u;
    };
    for (int i = 0; i < niter && alive; ++i) {
      const int s = i & 1;
      const uint32_t n = (uint32_t)i >> 1;
      if (!wait_or_flag(&a_full[s], n & 1u, err, 4)) {
        alive = false;
        break;
      }
      if (i >= 2 && !wait_or_flag(&d2_full[s], ((uint32_t)(i - 2) >> 1) & 1u, err, 11)) {
        alive = false;   // GEMM2 of tile i-2, the last reader of D1[s], has completed
        break;
      }
      tc::tc_after_sync();
      const uint32_t A = tmem + (uint32_t)(3 * C * s), D = tmem + TD1 + (uint32_t)(C * s);
#pragma unroll 1
      for (int k = 0; k < 3 * C / 16; ++k)
        mma3_ta(D, A + 8u * k, A + 3 * C / 2 + 8u * k, tc::kmajor_desc(w1 + 256u * k, 128u, 3 * C * 16u),
                tc::kmajor_desc(w1 + B1 / 2 + 256u * k, 128u, 3 * C * 16u), i1, k > 0);
      tc::mma_commit(&d1_full[s]);
      last = &d1_full[s];
      last_par = n & 1u;
      if (i >= 1) {
        if (!wait_or_flag(&h_full[(i - 1) & 1], ((uint32_t)(i - 1) >> 1) & 1u, err, 5)) { alive = false; break; }
        tc::tc_after_sync();
        gemm2(i - 1);
      }
    }
    if (alive && niter >= 1) {
      const int j = niter - 1;
      if (wait_or_flag(&h_full[j & 1], ((uint32_t)j >> 1) & 1u, err, 6)) {
        tc::tc_after_sync();
        gemm2(j);
      }
    }
    if (last) tc::mbar_wait_for(last, last_par, WAIT_NS);   // no MMA in flight when tensor memory is freed
  } else if (ok && warp >= W_CVT && warp < W_E1) {
    const int q = warp & 3, r = 32 * q + lane;
    const uint32_t lq = (uint32_t)(32 * q) << 16;
    bool alive = true;
    for (int i = 0; i < niter && alive; ++i) {
      const int s = i & 1;
      if (!warp_wait(&a_empty[s], (((uint32_t)i >> 1) & 1u) ^ 1u, err, 7)) break;   // D2 of tile i-2 read
      tc::tc_after_sync();
      const uint32_t A = tmem + lq + (uint32_t)(3 * C * s);
      for (int ph = 0; ph < NPH; ++ph) {
        const int u = i * NPH + ph, st = u % NS;
        if (!warp_wait(&stg_full[st], (uint32_t)(u / NS) & 1u, err, 8)) {
          alive = false;
          break;
        }
        const int t = ph / NB, c0 = 32 * (ph % NB);
        const uint8_t* rp = ring + st * SB + r * 128;
        uint32_t hi[16], lo[16];
#pragma unroll
        for (int cc = 0; cc < 8; ++cc) {
          const float4 p = *reinterpret_cast<const float4*>(rp + ((cc ^ (r & 7)) << 4));
          float y[4] = {p.x, p.y, p.z, p.w};
          if (t > 0) {
            const float* k = cf[t - 1];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
              const int c = c0 + 4 * cc + e;
              y[e] = gelu_tc((y[e] - k[c]) * k[C + c] + k[2 * C + c]);
            }
          }
          tc::split_pack(y[0], y[1], hi[2 * cc], lo[2 * cc]);
          tc::split_pack(y[2], y[3], hi[2 * cc + 1], lo[2 * cc + 1]);
        }
        tc::mbar_arrive(&stg_empty[st]);
        const uint32_t kc = (uint32_t)((t * C + c0) / 2);
        tc::tmem_st16u(A + kc, hi);
        tc::tmem_st16u(A + (uint32_t)(3 * C / 2) + kc, lo);
      }
      if (!alive) break;
      tc::tmem_wait_st();
      tc::tc_before_sync();
      tc::mbar_arrive(&a_full[s]);
    }
  } else if (ok && warp >= W_E1 && warp < W_E2) {
    const int q = warp & 3, hf = (warp - W_E1) >> 2, r = 32 * q + lane;
    const uint32_t lq = (uint32_t)(32 * q) << 16;
    for (int i = 0; i < niter; ++i) {
      const int s = i & 1;
      const long v = tile_of(i) * TM + r;
      if (!warp_wait(&d1_full[s], ((uint32_t)i >> 1) & 1u, err, 9)) break;
      tc::tc_after_sync();
      const uint32_t D = tmem + lq + TD1 + (uint32_t)(C * s);
#pragma unroll 1
      for (int j = hf; j < C / 16; j += 2) {
        uint32_t h[16];
        tc::tmem_ld16u(D + 16u * j, h);
        tc::tmem_wait_ld();
        if (hg && v < V) {
          float o[16];
#pragma unroll
          for (int e = 0; e < 16; ++e) o[e] = __uint_as_float(h[e]);
          tc::st8(hg + v * C + 16 * j, o);
          tc::st8(hg + v * C + 16 * j + 8, o + 8);
        }
        uint32_t hi[8], lo[8];
#pragma unroll
        for (int e = 0; e < 8; ++e)
          tc::split_pack(gelu_tc(__uint_as_float(h[2 * e])), gelu_tc(__uint_as_float(h[2 * e + 1])), hi[e], lo[e]);
        tc::tmem_st8u(D + 16u * j, hi);
        tc::tmem_st8u(D + 16u * j + 8u, lo);
      }
      tc::tmem_wait_st();
      tc::tc_before_sync();
      tc::mbar_arrive(&h_full[s]);
    }
  } else if (ok && warp >= W_E2) {
    const int q = warp & 3, r = 32 * q + lane;
    const uint32_t lq = (uint32_t)(32 * q) << 16;
    for (int i = 0; i < niter; ++i) {
      const int s = i & 1;
      const long v = tile_of(i) * TM + r;
      if (!warp_wait(&d2_full[s], ((uint32_t)i >> 1) & 1u, err, 10)) break;
      tc::tc_after_sync();
      const uint32_t D = tmem + lq + (uint32_t)(3 * C * s);
#pragma unroll
      for (int k = 0; k < 2 * C / 16; ++k) {
        uint32_t d[16];
        tc::tmem_ld16u(D + 16u * k, d);
        tc::tmem_wait_ld();
        if (k == 2 * C / 16 - 1) {   // the A stage is free once D2 is in registers
          tc::tc_before_sync();
          tc::mbar_arrive(&a_empty[s]);
        }
        if (v < V) {
          float o[16];
#pragma unroll
          for (int e = 0; e < 16; ++e) o[e] = sigmoid_tc(__uint_as_float(d[e]) + bs[16 * k + e]);
          tc::st8(gates + v * 2 * C + 16 * k, o);
          tc::st8(gates + v * 2 * C + 16 * k + 8, o + 8);
        }
      }
    }
  }
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  if (warp == 0) tc::tmem_free(tmem, 512);
}

// ================================================================================================ fuse, second half
// The ffno_fuse2_tc contract: B = [gelu(GN_s(spec_pre)) g_s, gelu(GN_v(vert_pre)) g_v] (g = the branch gates [V][2C]),
// pre = gelu(B Wf1^T) Wf2^T + (B[:, :C] + B[:, C:]) / 2, with the depth-weighted GroupNorm partials of pre.
// Roles: warp 0 TMA: per tile 2 NB phases of 32 channels (spec_pre boxes, then vert_pre boxes), each a pre box and the
// matching gates box, through a three-stage ring; warp 1 MMA: GEMM1 D1 = B Wf1^T (N = K = 2C) and, one tile behind,
// GEMM2 D2 += H Wf2^T (N = C); warps 2-5 conversion: B split into the tile's A stage and the FP32 residual
// (B[:, c] + B[:, C + c]) / 2 into its D2 buffer (GEMM2 accumulates onto it); warps 6-13 epilogue 1: H = gelu(D1),
// split over D1; warps 14-17 epilogue 2: pre and its statistics, as in the forward MLP. Tensor memory (8C columns):
// A stages at 0 and 2C, D1 at 4C, D2 buffers at 6C and 7C.
template <int C>
__global__ void __launch_bounds__(NTHREADS, 1)
    k_fuse2_ws(const __grid_constant__ CUtensorMap map_sp, const __grid_constant__ CUtensorMap map_vp,
               const __grid_constant__ CUtensorMap map_g, const float* __restrict__ sc, const float* __restrict__ vc,
               long V, const uint8_t* __restrict__ wpack, const float* __restrict__ dw, float* __restrict__ pre,
               double* __restrict__ partials, int* __restrict__ err) {
  static_assert(C == 32 || C == 64, "widths 32 and 64");
  constexpr uint32_t B1 = mat_bytes(2 * C, 2 * C), B2 = mat_bytes(C, 2 * C);
  constexpr uint32_t WB = B1 + B2;
  constexpr int NB = C / 32, NPH = 2 * NB, NS = 3, CPG = C / GMAX;
  constexpr uint32_t SB = 2 * BOX_BYTES;         // one ring stage: a pre box and its gates box
  constexpr uint32_t TA = 0, TD1 = 4 * C, TD2 = 6 * C;
  static_assert(WB % 1024 == 0, "the ring must stay 1024-byte aligned (128-byte swizzle)");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint8_t* ring = smem + WB;
  __shared__ uint64_t stg_full[NS], stg_empty[NS], a_full[2], a_empty[2], d2_free[2], d2_full[2], d1_full, h_full,
      wbar;
  __shared__ uint32_t tslot;
  __shared__ float cf[2][3 * C];              // GroupNorm coefficients of spec and vert: mean, gamma rstd, beta
  __shared__ float red[4][GMAX + 1], gmean[GMAX], wsum;
  __shared__ double acc[GMAX * 3];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) tc::tmem_alloc(&tslot, 512);
  if (threadIdx.x == 0) {
    for (int s = 0; s < NS; ++s) {
      tc::mbar_init(&stg_full[s], 1);
      tc::mbar_init(&stg_empty[s], 128);
    }
    for (int s = 0; s < 2; ++s) {
      tc::mbar_init(&a_full[s], 128);
      tc::mbar_init(&a_empty[s], 1);
      tc::mbar_init(&d2_free[s], 128);
      tc::mbar_init(&d2_full[s], 1);
    }
    tc::mbar_init(&d1_full, 1);
    tc::mbar_init(&h_full, 256);
    tc::mbar_init(&wbar, 1);
    tc::mbar_init_fence();
  }
  for (int e = threadIdx.x; e < 3 * C; e += NTHREADS) {
    cf[0][e] = sc[e];
    cf[1][e] = vc[e];
  }
  if (threadIdx.x < GMAX * 3) acc[threadIdx.x] = 0.0;
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  const uint32_t tmem = tslot;
  if (threadIdx.x == 0) {
    tc::mbar_arrive_expect_tx(&wbar, WB);
    for (uint32_t off = 0; off < WB; off += 32768u)
      tc::bulk_g2s(smem + off, wpack + off, WB - off < 32768u ? WB - off : 32768u, &wbar);
  }
  const bool ok = __syncthreads_and(tc::mbar_wait_for(&wbar, 0, WAIT_NS)) != 0;
  if (!ok && threadIdx.x == 0) atomicExch(err, 1);

  const long nt = (V + TM - 1) / TM;
  const int niter = (long)blockIdx.x < nt ? (int)((nt - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  auto tile_of = [&](int i) { return (long)blockIdx.x + (long)i * gridDim.x; };

  if (ok && warp == W_TMA && lane == 0) {
    int issued[NS] = {0, 0, 0};
    bool alive = true;
    for (int i = 0; i < niter && alive; ++i) {
      const int row = (int)(tile_of(i) * TM);
      for (int ph = 0; ph < NPH; ++ph) {
        const int u = i * NPH + ph, st = u % NS;
        const uint32_t n = (uint32_t)(u / NS);
        if (!wait_or_flag(&stg_empty[st], (n & 1u) ^ 1u, err, 3)) {
          alive = false;
          break;
        }
        tc::mbar_arrive_expect_tx(&stg_full[st], SB);
        uint8_t* sp = ring + st * SB;
        tc::tma_load_2d(sp, ph < NB ? &map_sp : &map_vp, 32 * (ph % NB), row, &stg_full[st]);
        tc::tma_load_2d(sp + BOX_BYTES, &map_g, 32 * ph, row, &stg_full[st]);
        ++issued[st];
      }
    }
    for (int s = 0; s < NS; ++s)
      if (issued[s]) tc::mbar_wait_for(&stg_full[s], (uint32_t)(issued[s] - 1) & 1u, WAIT_NS);
  } else if (ok && warp == W_MMA && lane == 0) {
    const uint32_t i1 = tc::idesc_bf16(128, 2 * C), i2 = tc::idesc_bf16(128, C);
    const uint32_t w1 = tc::smem_u32(smem), w2 = w1 + B1;
    uint64_t* last = nullptr;
    uint32_t last_par = 0;
    bool alive = true;
    auto gemm2 = [&](int j) {   // D2[j % 2] += H(j) Wf2^T, H in D1 as [hi 8 | lo 8] per 16-wide k chunk, K = 2C
#pragma unroll 1
      for (int k = 0; k < 2 * C / 16; ++k)
        mma3_ta(tmem + TD2 + (uint32_t)(C * (j & 1)), tmem + TD1 + 16u * k, tmem + TD1 + 16u * k + 8u,
                tc::kmajor_desc(w2 + 256u * k, 128u, 2 * C * 16u),
                tc::kmajor_desc(w2 + B2 / 2 + 256u * k, 128u, 2 * C * 16u), i2, true);
      tc::mma_commit(&d2_full[j & 1]);
      last = &d2_full[j & 1];
      last_par = ((uint32_t)j >> 1) & 1u;
    };
    for (int i = 0; i < niter && alive; ++i) {
      const int s = i & 1;
      if (!wait_or_flag(&a_full[s], ((uint32_t)i >> 1) & 1u, err, 4)) {
        alive = false;
        break;
      }
      if (i >= 1) {   // GEMM2 of the previous tile reads D1 before GEMM1 of this one overwrites it
        if (!wait_or_flag(&h_full, (uint32_t)(i - 1) & 1u, err, 5)) {
          alive = false;
          break;
        }
        tc::tc_after_sync();
        gemm2(i - 1);
      }
      tc::tc_after_sync();
      const uint32_t A = tmem + TA + (uint32_t)(2 * C * s);
#pragma unroll 1
      for (int k = 0; k < 2 * C / 16; ++k)
        mma3_ta(tmem + TD1, A + 8u * k, A + C + 8u * k, tc::kmajor_desc(w1 + 256u * k, 128u, 2 * C * 16u),
                tc::kmajor_desc(w1 + B1 / 2 + 256u * k, 128u, 2 * C * 16u), i1, k > 0);
      tc::mma_commit(&d1_full);
      tc::mma_commit(&a_empty[s]);
      last = &a_empty[s];
      last_par = ((uint32_t)i >> 1) & 1u;
    }
    if (alive && niter >= 1) {
      const int j = niter - 1;
      if (wait_or_flag(&h_full, (uint32_t)j & 1u, err, 6)) {
        tc::tc_after_sync();
        gemm2(j);
      }
    }
    if (last) tc::mbar_wait_for(last, last_par, WAIT_NS);   // no MMA in flight when tensor memory is freed
  } else if (ok && warp >= W_CVT && warp < W_E1) {
    const int q = warp & 3, r = 32 * q + lane;
    const uint32_t lq = (uint32_t)(32 * q) << 16;
    bool alive = true;
    for (int i = 0; i < niter && alive; ++i) {
      const int s = i & 1;
      const uint32_t n2 = ((uint32_t)i >> 1) & 1u;
      if (!warp_wait(&a_empty[s], n2 ^ 1u, err, 7)) break;    // GEMM1 of tile i-2 has read the A stage
      if (!warp_wait(&d2_free[s], n2 ^ 1u, err, 8)) break;    // epilogue 2 of tile i-2 has read D2[s]
      tc::tc_after_sync();
      const uint32_t A = tmem + lq + TA + (uint32_t)(2 * C * s), D2 = tmem + lq + TD2 + (uint32_t)(C * s);
      for (int ph = 0; ph < NPH; ++ph) {
        const int u = i * NPH + ph, st = u % NS;
        if (!warp_wait(&stg_full[st], (uint32_t)(u / NS) & 1u, err, 12)) {
          alive = false;
          break;
        }
        const int br = ph / NB, c0 = 32 * (ph % NB);   // branch (0 spec, 1 vert) and its first channel
        const float* k = cf[br];
        const uint8_t* rp = ring + st * SB + r * 128;
        float b[32];
#pragma unroll
        for (int cc = 0; cc < 8; ++cc) {
          const uint32_t o = (uint32_t)((cc ^ (r & 7)) << 4);
          const float4 p = *reinterpret_cast<const float4*>(rp + o);
          const float4 g = *reinterpret_cast<const float4*>(rp + BOX_BYTES + o);
          const float pp[4] = {p.x, p.y, p.z, p.w}, gg[4] = {g.x, g.y, g.z, g.w};
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int c = c0 + 4 * cc + e;
            b[4 * cc + e] = gelu_tc((pp[e] - k[c]) * k[C + c] + k[2 * C + c]) * gg[e];
          }
        }
        tc::mbar_arrive(&stg_empty[st]);
        uint32_t hi[16], lo[16];
#pragma unroll
        for (int e = 0; e < 16; ++e) tc::split_pack(b[2 * e], b[2 * e + 1], hi[e], lo[e]);
        const uint32_t kc = (uint32_t)((br * C + c0) / 2);   // first column of this phase's channel pairs
        tc::tmem_st16u(A + kc, hi);
        tc::tmem_st16u(A + (uint32_t)C + kc, lo);
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {   // residual (B[c] + B[C + c]) / 2 in D2
          float rr[16];
          if (br == 0) {
#pragma unroll
            for (int e = 0; e < 16; ++e) rr[e] = 0.5f * b[16 * hh + e];
          } else {
            tc::tmem_ld16(D2 + (uint32_t)(c0 + 16 * hh), rr);
#pragma unroll
            for (int e = 0; e < 16; ++e) rr[e] = fmaf(0.5f, b[16 * hh + e], rr[e]);
          }
          tc::tmem_st16(D2 + (uint32_t)(c0 + 16 * hh), rr);
        }
      }
      if (!alive) break;
      tc::tmem_wait_st();
      tc::tc_before_sync();
      tc::mbar_arrive(&a_full[s]);
    }
  } else if (ok && warp >= W_E1 && warp < W_E2) {
    const int q = warp & 3, hf = (warp - W_E1) >> 2;
    const uint32_t lq = (uint32_t)(32 * q) << 16;
    for (int i = 0; i < niter; ++i) {
      if (!warp_wait(&d1_full, (uint32_t)i & 1u, err, 9)) break;
      tc::tc_after_sync();
      const uint32_t D = tmem + lq + TD1;
#pragma unroll 1
      for (int j = hf; j < 2 * C / 16; j += 2) {
        uint32_t h[16];
        tc::tmem_ld16u(D + 16u * j, h);
        tc::tmem_wait_ld();
        uint32_t hi[8], lo[8];
#pragma unroll
        for (int e = 0; e < 8; ++e)
          tc::split_pack(gelu_tc(__uint_as_float(h[2 * e])), gelu_tc(__uint_as_float(h[2 * e + 1])), hi[e], lo[e]);
        tc::tmem_st8u(D + 16u * j, hi);
        tc::tmem_st8u(D + 16u * j + 8u, lo);
      }
      tc::tmem_wait_st();
      tc::tc_before_sync();
      tc::mbar_arrive(&h_full);
    }
  } else if (ok && warp >= W_E2) {
    const int q = warp & 3, r = 32 * q + lane, wl = warp - W_E2;
    const uint32_t lq = (uint32_t)(32 * q) << 16;
    for (int i = 0; i < niter; ++i) {
      const int s = i & 1;
      const long v = tile_of(i) * TM + r;
      const bool live = v < V;
      const float w = live ? __ldg(dw + v) : 0.f;
      if (!e2_sync_and(tc::mbar_wait_for(&d2_full[s], ((uint32_t)i >> 1) & 1u, WAIT_NS))) {
        if (lane == 0) atomicExch(err, 10);
        break;
      }
      tc::tc_after_sync();
      const uint32_t D = tmem + lq + TD2 + (uint32_t)(C * s);
      float gs[GMAX];
#pragma unroll
      for (int k = 0; k < C / 16; ++k) {
        uint32_t d[16];
        tc::tmem_ld16u(D + 16u * k, d);
        tc::tmem_wait_ld();
        if (live) {
          float o[16];
#pragma unroll
          for (int e = 0; e < 16; ++e) o[e] = __uint_as_float(d[e]);
          tc::st8(pre + v * C + 16 * k, o);
          tc::st8(pre + v * C + 16 * k + 8, o + 8);
        }
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          const int g = (16 * k + e) / CPG;
          if (e % CPG == 0) gs[g] = 0.f;
          gs[g] += __uint_as_float(d[e]);
        }
      }
      float ws = w;
#pragma unroll
      for (int m = 16; m; m >>= 1) ws += __shfl_xor_sync(0xffffffffu, ws, m);
#pragma unroll
      for (int g = 0; g < GMAX; ++g) {
        float t = w * gs[g];
#pragma unroll
        for (int m = 16; m; m >>= 1) t += __shfl_xor_sync(0xffffffffu, t, m);
        if (lane == 0) red[wl][g] = t;
      }
      if (lane == 0) red[wl][GMAX] = ws;
      e2_sync();
      if (threadIdx.x - 32 * W_E2 < GMAX) {
        const int g = threadIdx.x - 32 * W_E2;
        const float wt = ((red[0][GMAX] + red[1][GMAX]) + (red[2][GMAX] + red[3][GMAX])) * CPG;
        gmean[g] = wt > 0.f ? ((red[0][g] + red[1][g]) + (red[2][g] + red[3][g])) / wt : 0.f;
        if (g == 0) wsum = wt;
      }
      e2_sync();
#pragma unroll
      for (int k = 0; k < C / 16; ++k) {
        uint32_t d[16];
        tc::tmem_ld16u(D + 16u * k, d);
        tc::tmem_wait_ld();
#pragma unroll
        for (int e = 0; e < 16; ++e) {
          const int g = (16 * k + e) / CPG;
          if (e % CPG == 0) gs[g] = 0.f;
          const float x = __uint_as_float(d[e]) - gmean[g];
          gs[g] = fmaf(x, x, gs[g]);
        }
      }
      tc::tc_before_sync();
      tc::mbar_arrive(&d2_free[s]);   // D2[s] has been read: conversion may write the residual of tile i + 2
#pragma unroll
      for (int g = 0; g < GMAX; ++g) {
        float t = w * gs[g];
#pragma unroll
        for (int m = 16; m; m >>= 1) t += __shfl_xor_sync(0xffffffffu, t, m);
        if (lane == 0) red[wl][g] = t;
      }
      e2_sync();
      if (threadIdx.x - 32 * W_E2 < GMAX) {
        const int g = threadIdx.x - 32 * W_E2;
        GroupAcc a{acc[3 * g], acc[3 * g + 1], acc[3 * g + 2]};
        chan_merge(a, (double)wsum, (double)gmean[g], (double)((red[0][g] + red[1][g]) + (red[2][g] + red[3][g])));
        acc[3 * g] = a.w;
        acc[3 * g + 1] = a.mean;
        acc[3 * g + 2] = a.m2;
      }
      e2_sync();
    }
  }
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  if (threadIdx.x < GMAX) {
    double* o = partials + ((long)blockIdx.x * GMAX + threadIdx.x) * 3;
    o[0] = acc[3 * threadIdx.x];
    o[1] = acc[3 * threadIdx.x + 1];
    o[2] = acc[3 * threadIdx.x + 2];
  }
  if (warp == 0) tc::tmem_free(tmem, 512);
}

// ============================================================================================ input gate, VJP
// The ffno_gate_bwd_tc contract: x_bar = base + d/dx [x sigmoid(gelu(x G1^T) G2^T)] applied to g_bar, z_bar[v] +=
// g_bar . zp when zp. Per tile (lane = voxel, all products untransposed, K = N = C):
//   GEMM1 h = x G1^T;  E1: H = gelu(h);  GEMM2 s = H G2^T;  E2: o = base + g_bar sig(s) (stored into the GEMM4
//   accumulator), Q = g_bar x sig(s) (1 - sig(s));  GEMM3 t = Q G2;  E3: G = t gelu'(h);  GEMM4 acc += G G1;  E4: x_bar.
// Roles: warp 0 TMA ring of x and g_bar (two stages; a stage is held until E2 has read it); warp 1 MMA; warps 2-5
// conversion of x into tensor memory; warps 6-9 E1 and E3; warps 10-13 E2 and E4. Tiles go through in pairs, one per
// tensor-memory slot of 4C columns ([x split, then s, then t] [h] [H, then Q, then G] [o + G G1]), and every role
// works through a pair stage by stage (both tiles' GEMM1, both E1, both GEMM2, ...), so that the MMAs of one tile run
// while the epilogue warps work on the other.
template <int C>
__global__ void __launch_bounds__(448, 1)
    k_gate_bwd_ws(const __grid_constant__ CUtensorMap map_x, const __grid_constant__ CUtensorMap map_g,
                  const float* __restrict__ base, long V, const uint8_t* __restrict__ wpack,
                  const float* __restrict__ zp, float* __restrict__ xbar, float* __restrict__ zbar,
                  int* __restrict__ err) {
  static_assert(C == 32 || C == 64, "widths 32 and 64");
  constexpr int GW_TMA = 0, GW_MMA = 1, GW_CVT = 2, GW_E13 = 6, GW_E24 = 10;
  constexpr uint32_t B1 = mat_bytes(C, C);       // each of g1, g2, g2t, g1t
  constexpr uint32_t WB = 4 * B1;
  constexpr int NB = C / 32;
  constexpr uint32_t XB = NB * BOX_BYTES;        // one tensor's FP32 tile
  constexpr uint32_t SB = 2 * XB;                // one ring stage: x, g_bar
  static_assert(WB % 1024 == 0, "the ring must stay 1024-byte aligned (128-byte swizzle)");
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = align1024(smem_raw);
  uint8_t* ring = smem + WB;
  __shared__ uint64_t stg_full[2], stg_empty[2], a_full[2], ra_free[2], d1_full[2], h_full[2], d2_full[2],
      q_full[2], d3_full[2], g_full[2], d4_full[2], wbar;
  __shared__ uint32_t tslot;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (warp == 0) tc::tmem_alloc(&tslot, 512);
  if (threadIdx.x == 0) {
    for (int s = 0; s < 2; ++s) {
      tc::mbar_init(&stg_full[s], 1);
      tc::mbar_init(&stg_empty[s], 128);
      tc::mbar_init(&a_full[s], 128);
      tc::mbar_init(&ra_free[s], 128);
      tc::mbar_init(&d1_full[s], 1);
      tc::mbar_init(&h_full[s], 128);
      tc::mbar_init(&d2_full[s], 1);
      tc::mbar_init(&q_full[s], 128);
      tc::mbar_init(&d3_full[s], 1);
      tc::mbar_init(&g_full[s], 128);
      tc::mbar_init(&d4_full[s], 1);
    }
    tc::mbar_init(&wbar, 1);
    tc::mbar_init_fence();
  }
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  const uint32_t tmem = tslot;
  if (threadIdx.x == 0) {
    tc::mbar_arrive_expect_tx(&wbar, WB);
    for (uint32_t off = 0; off < WB; off += 32768u)
      tc::bulk_g2s(smem + off, wpack + off, WB - off < 32768u ? WB - off : 32768u, &wbar);
  }
  const bool ok = __syncthreads_and(tc::mbar_wait_for(&wbar, 0, WAIT_NS)) != 0;
  if (!ok && threadIdx.x == 0) atomicExch(err, 1);

  const long nt = (V + TM - 1) / TM;
  const int niter = (long)blockIdx.x < nt ? (int)((nt - 1 - blockIdx.x) / gridDim.x + 1) : 0;
  const int npair = (niter + 1) / 2;
  auto tile_of = [&](int i) { return (long)blockIdx.x + (long)i * gridDim.x; };
  // tensor-memory regions of slot t
  auto RA = [&](int t) { return tmem + (uint32_t)(4 * C * t); };
  auto RD1 = [&](int t) { return tmem + (uint32_t)(4 * C * t + C); };
  auto RH = [&](int t) { return tmem + (uint32_t)(4 * C * t + 2 * C); };
  auto RD4 = [&](int t) { return tmem + (uint32_t)(4 * C * t + 3 * C); };

  if (ok && warp == GW_TMA && lane == 0) {
    int issued[2] = {0, 0};
    for (int i = 0; i < niter; ++i) {
      const int s = i & 1;
      const uint32_t n = (uint32_t)i >> 1;
      if (!wait_or_flag(&stg_empty[s], (n & 1u) ^ 1u, err, 3)) break;
      const int row = (int)(tile_of(i) * TM);
      tc::mbar_arrive_expect_tx(&stg_full[s], SB);
      uint8_t* st = ring + s * SB;
#pragma unroll
      for (int b = 0; b < NB; ++b) {
        tc::tma_load_2d(st + b * BOX_BYTES, &map_x, 32 * b, row, &stg_full[s]);
        tc::tma_load_2d(st + XB + b * BOX_BYTES, &map_g, 32 * b, row, &stg_full[s]);
      }
      ++issued[s];
    }
    for (int s = 0; s < 2; ++s)
      if (issued[s]) tc::mbar_wait_for(&stg_full[s], (uint32_t)(issued[s] - 1) & 1u, WAIT_NS);
  } else if (ok && warp == GW_MMA && lane == 0) {
    const uint32_t id = tc::idesc_bf16(128, C);
    const uint32_t g1 = tc::smem_u32(smem), g2 = g1 + B1, g2t = g1 + 2 * B1, g1t = g1 + 3 * B1, LO = B1 / 2;
    auto bd = [&](uint32_t w, int k) { return tc::kmajor_desc(w + 256u * k, 128u, C * 16u); };
    // D (+)= A W^T with A in tensor memory as [hi 8 | lo 8] column pairs per 16-wide k chunk
    auto gemm_il = [&](uint32_t d, uint32_t a, uint32_t w, bool acc) {
#pragma unroll 1
      for (int k = 0; k < C / 16; ++k) mma3_ta(d, a + 16u * k, a + 16u * k + 8u, bd(w, k), bd(w + LO, k), id, acc || k > 0);
    };
    uint64_t* last = nullptr;
    uint32_t last_par = 0;
    bool alive = true;
    for (int p = 0; p < npair && alive; ++p) {
      const uint32_t par = (uint32_t)p & 1u;
      const int nin = (2 * p + 1 < niter) ? 2 : 1;
      for (int t = 0; t < nin && alive; ++t) {   // GEMM1: h = x G1^T (x as [hi C/2 | lo C/2])
        if (!wait_or_flag(&a_full[t], par, err, 4)) { alive = false; break; }
        tc::tc_after_sync();
#pragma unroll 1
        for (int k = 0; k < C / 16; ++k)
          mma3_ta(RD1(t), RA(t) + 8u * k, RA(t) + C / 2 + 8u * k, bd(g1, k), bd(g1 + LO, k), id, k > 0);
        tc::mma_commit(&d1_full[t]);
        last = &d1_full[t];
        last_par = par;
      }
      for (int t = 0; t < nin && alive; ++t) {   // GEMM2: s = H G2^T into the x region
        if (!wait_or_flag(&h_full[t], par, err, 5)) { alive = false; break; }
        tc::tc_after_sync();
        gemm_il(RA(t), RH(t), g2, false);
        tc::mma_commit(&d2_full[t]);
        last = &d2_full[t];
      }
      for (int t = 0; t < nin && alive; ++t) {   // GEMM3: t = Q G2 into the x region
        if (!wait_or_flag(&q_full[t], par, err, 6)) { alive = false; break; }
        tc::tc_after_sync();
        gemm_il(RA(t), RH(t), g2t, false);
        tc::mma_commit(&d3_full[t]);
        last = &d3_full[t];
      }
      for (int t = 0; t < nin && alive; ++t) {   // GEMM4: o += G G1
        if (!wait_or_flag(&g_full[t], par, err, 11)) { alive = false; break; }
        tc::tc_after_sync();
        gemm_il(RD4(t), RH(t), g1t, true);
        tc::mma_commit(&d4_full[t]);
        last = &d4_full[t];
      }
    }
    if (last) tc::mbar_wait_for(last, last_par, WAIT_NS);   // no MMA in flight when tensor memory is freed
  } else if (ok && warp >= GW_CVT && warp < GW_E13) {
    const int q = warp & 3, r = 32 * q + lane;
    const uint32_t lq = (uint32_t)(32 * q) << 16;
    for (int i = 0; i < niter; ++i) {
      const int s = i & 1, t = i & 1;
      const uint32_t n = (uint32_t)i >> 1;
      if (!warp_wait(&stg_full[s], n & 1u, err, 7)) break;
      if (!warp_wait(&ra_free[t], (n & 1u) ^ 1u, err, 8)) break;   // E3 of tile i-2 has read its t
      tc::tc_after_sync();
      const uint8_t* st = ring + s * SB;
      const uint32_t A = RA(t) + lq;
#pragma unroll 1
      for (int bh = 0; bh < 2 * NB; ++bh) {
        const uint8_t* rin = st + (bh >> 1) * BOX_BYTES + r * 128;
        uint32_t hi[8], lo[8];
#pragma unroll
        for (int cc = 0; cc < 4; ++cc) {
          const int c = 4 * (bh & 1) + cc;
          const float4 v = *reinterpret_cast<const float4*>(rin + ((c ^ (r & 7)) << 4));
          tc::split_pack(v.x, v.y, hi[2 * cc], lo[2 * cc]);
          tc::split_pack(v.z, v.w, hi[2 * cc + 1], lo[2 * cc + 1]);
        }
        tc::tmem_st8u(A + (uint32_t)(8 * bh), hi);
        tc::tmem_st8u(A + (uint32_t)(C / 2 + 8 * bh), lo);
      }
      tc::tmem_wait_st();
      tc::tc_before_sync();
      tc::mbar_arrive(&a_full[t]);
    }
  } else if (ok && warp >= GW_E13 && warp < GW_E24) {
    const int q = warp & 3;
    const uint32_t lq = (uint32_t)(32 * q) << 16;
    bool alive = true;
    for (int p = 0; p < npair && alive; ++p) {
      const uint32_t par = (uint32_t)p & 1u;
      const int nin = (2 * p + 1 < niter) ? 2 : 1;
      for (int t = 0; t < nin && alive; ++t) {   // E1: H = gelu(h)
        if (!warp_wait(&d1_full[t], par, err, 9)) { alive = false; break; }
        tc::tc_after_sync();
#pragma unroll 1
        for (int k = 0; k < C / 16; ++k) {
          uint32_t h[16];
          tc::tmem_ld16u(RD1(t) + lq + 16u * k, h);
          tc::tmem_wait_ld();
          uint32_t hi[8], lo[8];
#pragma unroll
          for (int e = 0; e < 8; ++e)
            tc::split_pack(gelu_tc(__uint_as_float(h[2 * e])), gelu_tc(__uint_as_float(h[2 * e + 1])), hi[e], lo[e]);
          tc::tmem_st8u(RH(t) + lq + 16u * k, hi);
          tc::tmem_st8u(RH(t) + lq + 16u * k + 8u, lo);
        }
        tc::tmem_wait_st();
        tc::tc_before_sync();
        tc::mbar_arrive(&h_full[t]);
      }
      for (int t = 0; t < nin && alive; ++t) {   // E3: G = t gelu'(h)
        if (!warp_wait(&d3_full[t], par, err, 12)) { alive = false; break; }
        tc::tc_after_sync();
#pragma unroll 1
        for (int k = 0; k < C / 16; ++k) {
          uint32_t tv[16], h[16];
          tc::tmem_ld16u(RA(t) + lq + 16u * k, tv);
          tc::tmem_ld16u(RD1(t) + lq + 16u * k, h);
          tc::tmem_wait_ld();
          uint32_t hi[8], lo[8];
#pragma unroll
          for (int e = 0; e < 8; ++e)
            tc::split_pack(__uint_as_float(tv[2 * e]) * gelu_grad_tc(__uint_as_float(h[2 * e])),
                           __uint_as_float(tv[2 * e + 1]) * gelu_grad_tc(__uint_as_float(h[2 * e + 1])), hi[e], lo[e]);
          tc::tmem_st8u(RH(t) + lq + 16u * k, hi);
          tc::tmem_st8u(RH(t) + lq + 16u * k + 8u, lo);
        }
        tc::tmem_wait_st();
        tc::tc_before_sync();
        tc::mbar_arrive(&g_full[t]);
        tc::mbar_arrive(&ra_free[t]);
      }
    }
  } else if (ok && warp >= GW_E24) {
    const int q = warp & 3, r = 32 * q + lane;
    const uint32_t lq = (uint32_t)(32 * q) << 16;
    bool alive = true;
    for (int p = 0; p < npair && alive; ++p) {
      const uint32_t par = (uint32_t)p & 1u;
      const int nin = (2 * p + 1 < niter) ? 2 : 1;
      for (int t = 0; t < nin && alive; ++t) {   // E2: the gate's local terms
        const int i = 2 * p + t;
        const long v = tile_of(i) * TM + r;
        const bool live = v < V;
        float bv[C];
#pragma unroll
        for (int c = 0; c < C; c += 8) {
          if (base && live) {
            tc::ld8(base + v * C + c, bv + c);
          } else {
#pragma unroll
            for (int e = 0; e < 8; ++e) bv[c + e] = 0.f;
          }
        }
        if (!warp_wait(&d2_full[t], par, err, 10)) { alive = false; break; }
        // x and g_bar of tile i in its ring stage (i & 1 == t): this warp waits on the stage's TMA barrier itself
        // (its phase cannot move on before this epilogue releases the stage), which makes the copy visible to it
        if (!warp_wait(&stg_full[t], par, err, 14)) { alive = false; break; }
        tc::tc_after_sync();
        const uint8_t* st = ring + t * SB;
        float zs = 0.f;
#pragma unroll
        for (int k = 0; k < C / 16; ++k) {
          uint32_t d[16];
          tc::tmem_ld16u(RA(t) + lq + 16u * k, d);
          tc::tmem_wait_ld();
          float o[16];
          uint32_t hi[8], lo[8];
          const uint8_t* rx = st + (k >> 1) * BOX_BYTES + r * 128;
#pragma unroll
          for (int cc = 0; cc < 4; ++cc) {
            const uint32_t off = (uint32_t)(((4 * (k & 1) + cc) ^ (r & 7)) << 4);
            const float4 xv = *reinterpret_cast<const float4*>(rx + off);
            const float4 gv = *reinterpret_cast<const float4*>(rx + XB + off);
            const float xx[4] = {xv.x, xv.y, xv.z, xv.w}, gg[4] = {gv.x, gv.y, gv.z, gv.w};
            const float* bb = bv + 16 * k + 4 * cc;
            float qv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              const float sg = sigmoid_tc(__uint_as_float(d[4 * cc + u]));
              o[4 * cc + u] = fmaf(gg[u], sg, bb[u]);
              qv[u] = gg[u] * xx[u] * sg * (1.f - sg);
              if (zp) zs = fmaf(gg[u], __ldg(zp + 16 * k + 4 * cc + u), zs);
            }
            tc::split_pack(qv[0], qv[1], hi[2 * cc], lo[2 * cc]);
            tc::split_pack(qv[2], qv[3], hi[2 * cc + 1], lo[2 * cc + 1]);
          }
          tc::tmem_st16(RD4(t) + lq + 16u * k, o);
          tc::tmem_st8u(RH(t) + lq + 16u * k, hi);
          tc::tmem_st8u(RH(t) + lq + 16u * k + 8u, lo);
        }
        tc::tmem_wait_st();
        tc::mbar_arrive(&stg_empty[t]);
        tc::tc_before_sync();
        tc::mbar_arrive(&q_full[t]);
        if (zp && live) zbar[v] += zs;
      }
      for (int t = 0; t < nin && alive; ++t) {   // E4: x_bar
        const int i = 2 * p + t;
        const long v = tile_of(i) * TM + r;
        if (!warp_wait(&d4_full[t], par, err, 13)) { alive = false; break; }
        tc::tc_after_sync();
#pragma unroll
        for (int k = 0; k < C / 16; ++k) {
          uint32_t d[16];
          tc::tmem_ld16u(RD4(t) + lq + 16u * k, d);
          tc::tmem_wait_ld();
          if (v < V) {
            float o[16];
#pragma unroll
            for (int e = 0; e < 16; ++e) o[e] = __uint_as_float(d[e]);
            tc::st8(xbar + v * C + 16 * k, o);
            tc::st8(xbar + v * C + 16 * k + 8, o + 8);
          }
        }
      }
    }
  }
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  if (warp == 0) tc::tmem_free(tmem, 512);
}

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

// [V][C] FP32 rows as [128 voxels][32 channels] boxes with the 128-byte swizzle; rows past V read as zero
bool row_map(CUtensorMap* map, const float* p, long V, int C) {
  const PFN_cuTensorMapEncodeTiled_v12000 encode = tc::tensor_map_encoder();
  if (!encode) return false;
  cuuint64_t gdim[2] = {(cuuint64_t)C, (cuuint64_t)V};
  cuuint64_t gstr[1] = {(cuuint64_t)C * 4};
  cuuint32_t box[2] = {32u, (cuuint32_t)TM};
  cuuint32_t estr[2] = {1u, 1u};
  return encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(p), gdim, gstr, box, estr,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int C>
int launch_mlp2_bwd(const float* a, const float* pb, const float* base, long V, const void* wpack, float* abar,
                    int* err, cudaStream_t s) {
  CUtensorMap ma, mp;
  if (!row_map(&ma, a, V, C) || !row_map(&mp, pb, V, C)) return FFNO_EINVAL;
  const size_t smem = 1024 + 3 * (size_t)mat_bytes(2 * C, C) + 2 * (size_t)(2 * (C / 32) * BOX_BYTES);
  if (!ffno::smem_cap_ok(k_mlp2_bwd_ws<C>, smem))
    return FFNO_ELAUNCH;
  const long nt = (V + TM - 1) / TM;
  const int grid = (int)(nt < sms() ? nt : sms());
  k_mlp2_bwd_ws<C><<<grid, NTHREADS, smem, s>>>(ma, mp, base, V, static_cast<const uint8_t*>(wpack), abar, err);
  return cudaGetLastError() == cudaSuccess ? FFNO_OK : FFNO_ELAUNCH;
}

template <int C, int MODE>
int launch_mlp2_fwd(const float* in, const float* prev, const float* pc, float res, float* xout, long V,
                    const void* wpack, const float* dw, float* pre, double* partials, int nparts, int* err,
                    cudaStream_t s) {
  CUtensorMap mi, mp;
  if (!row_map(&mi, in, V, C)) return FFNO_EINVAL;
  if (MODE != 0 ? !row_map(&mp, prev, V, C) : !row_map(&mp, in, V, C)) return FFNO_EINVAL;
  const size_t smem = 1024 + 2 * (size_t)mat_bytes(2 * C, C) + 2 * (size_t)((MODE == 0 ? 1 : 2) * (C / 32) * BOX_BYTES);
  if (!ffno::smem_cap_ok(k_mlp2_fwd_ws<C, MODE>, smem)) return FFNO_ELAUNCH;
  k_mlp2_fwd_ws<C, MODE><<<nparts, NTHREADS, smem, s>>>(mi, mp, pc, res, xout, V, static_cast<const uint8_t*>(wpack),
                                                         dw, pre, partials, err);
  return cudaGetLastError() == cudaSuccess ? FFNO_OK : FFNO_ELAUNCH;
}

template <int C>
int launch_gate_fwd(const float* x, long V, const void* wpack, const float* zp, const float* z, float* out, int* err,
                    cudaStream_t s) {
  CUtensorMap mx;
  if (!row_map(&mx, x, V, C)) return FFNO_EINVAL;
  const size_t smem = 1024 + 2 * (size_t)mat_bytes(C, C) + 2 * (size_t)((C / 32) * BOX_BYTES);
  if (!ffno::smem_cap_ok(k_gate_fwd_ws<C>, smem))
    return FFNO_ELAUNCH;
  const long nt = (V + TM - 1) / TM;
  const int grid = (int)(nt < sms() ? nt : sms());
  k_gate_fwd_ws<C><<<grid, NTHREADS, smem, s>>>(mx, x, V, static_cast<const uint8_t*>(wpack), zp, z, out, err);
  return cudaGetLastError() == cudaSuccess ? FFNO_OK : FFNO_ELAUNCH;
}

template <int C>
int launch_gate_bwd(const float* x, const float* gbar, const float* base, long V, const void* wpack, const float* zp,
                    float* xbar, float* zbar, int* err, cudaStream_t s) {
  CUtensorMap mx, mg;
  if (!row_map(&mx, x, V, C) || !row_map(&mg, gbar, V, C)) return FFNO_EINVAL;
  const size_t smem = 1024 + 4 * (size_t)mat_bytes(C, C) + 2 * (size_t)(2 * (C / 32) * BOX_BYTES);
  if (!ffno::smem_cap_ok(k_gate_bwd_ws<C>, smem))
    return FFNO_ELAUNCH;
  const long nt = (V + TM - 1) / TM;
  const int grid = (int)(nt < sms() ? nt : sms());
  k_gate_bwd_ws<C><<<grid, 448, smem, s>>>(mx, mg, base, V, static_cast<const uint8_t*>(wpack), zp, xbar, zbar, err);
  return cudaGetLastError() == cudaSuccess ? FFNO_OK : FFNO_ELAUNCH;
}

template <int C>
int launch_fuse2(const float* sp, const float* sc, const float* vp, const float* vc, const float* gates, long V,
                 const void* wpack, const float* dw, float* pre, double* partials, int nparts, int* err,
                 cudaStream_t s) {
  CUtensorMap ms, mv, mg;
  if (!row_map(&ms, sp, V, C) || !row_map(&mv, vp, V, C) || !row_map(&mg, gates, V, 2 * C)) return FFNO_EINVAL;
  const size_t smem = 1024 + (size_t)mat_bytes(2 * C, 2 * C) + mat_bytes(C, 2 * C) + 3 * (size_t)(2 * BOX_BYTES);
  if (!ffno::smem_cap_ok(k_fuse2_ws<C>, smem))
    return FFNO_ELAUNCH;
  k_fuse2_ws<C><<<nparts, NTHREADS, smem, s>>>(ms, mv, mg, sc, vc, V, static_cast<const uint8_t*>(wpack), dw, pre,
                                                partials, err);
  return cudaGetLastError() == cudaSuccess ? FFNO_OK : FFNO_ELAUNCH;
}

template <int C>
int launch_fuse1(const float* x, const float* sp, const float* sc, const float* vp, const float* vc, long V,
                 const void* wpack, const float* bias, float* gates, float* hg, int* err, cudaStream_t s) {
  CUtensorMap mx, ms, mv;
  if (!row_map(&mx, x, V, C) || !row_map(&ms, sp, V, C) || !row_map(&mv, vp, V, C)) return FFNO_EINVAL;
  const size_t smem = 1024 + (size_t)mat_bytes(C, 3 * C) + mat_bytes(2 * C, C) + 4 * (size_t)BOX_BYTES;
  if (!ffno::smem_cap_ok(k_fuse1_ws<C>, smem))
    return FFNO_ELAUNCH;
  const long nt = (V + TM - 1) / TM;
  const int grid = (int)(nt < sms() ? nt : sms());
  k_fuse1_ws<C><<<grid, NTHREADS, smem, s>>>(mx, ms, mv, sc, vc, V, static_cast<const uint8_t*>(wpack), bias, gates,
                                              hg, err);
  return cudaGetLastError() == cudaSuccess ? FFNO_OK : FFNO_ELAUNCH;
}

}  // namespace

namespace ffno {
namespace ws {

// the epilogues read and write a voxel's row 32 bytes per request (rows of 32 or 64 floats keep that alignment)
static bool rows32(const void* p) { return p && reinterpret_cast<uintptr_t>(p) % 32 == 0; }

bool fuse1_supported(int C) { return C == 32 || C == 64; }

int fuse1(const float* x, const float* spec_pre, const float* spec_coefs, const float* vert_pre,
          const float* vert_coefs, long V, int C, const void* wpack, const float* bias, float* gates, float* hg,
          int* err, cudaStream_t stream) {
  if (V < 1 || V > 0x7fffffffL - TM || !bias ||
      (reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(spec_pre) | reinterpret_cast<uintptr_t>(vert_pre) |
       reinterpret_cast<uintptr_t>(gates)) % 16 ||
      (hg && reinterpret_cast<uintptr_t>(hg) % 16) || !rows32(gates) || (hg && !rows32(hg)))
    return FFNO_EINVAL;
  if (C == 64)
    return launch_fuse1<64>(x, spec_pre, spec_coefs, vert_pre, vert_coefs, V, wpack, bias, gates, hg, err, stream);
  if (C == 32)
    return launch_fuse1<32>(x, spec_pre, spec_coefs, vert_pre, vert_coefs, V, wpack, bias, gates, hg, err, stream);
  return FFNO_EINVAL;
}

bool fuse2_supported(int C) { return C == 32 || C == 64; }

int fuse2(const float* spec_pre, const float* spec_coefs, const float* vert_pre, const float* vert_coefs,
          const float* gates, long V, int C, const void* wpack, const float* dw, float* pre, double* partials,
          int nparts, int* err, cudaStream_t stream) {
  if (V < 1 || V > 0x7fffffffL - TM || nparts < 1 ||
      (reinterpret_cast<uintptr_t>(spec_pre) | reinterpret_cast<uintptr_t>(vert_pre) |
       reinterpret_cast<uintptr_t>(gates) | reinterpret_cast<uintptr_t>(pre)) % 16 || !rows32(pre))
    return FFNO_EINVAL;
  if (C == 64)
    return launch_fuse2<64>(spec_pre, spec_coefs, vert_pre, vert_coefs, gates, V, wpack, dw, pre, partials, nparts,
                            err, stream);
  if (C == 32)
    return launch_fuse2<32>(spec_pre, spec_coefs, vert_pre, vert_coefs, gates, V, wpack, dw, pre, partials, nparts,
                            err, stream);
  return FFNO_EINVAL;
}

bool gate_bwd_supported(int C) { return C == 32 || C == 64; }

int gate_bwd(const float* x, const float* g_bar, const float* base, long V, int C, const void* wpack, const float* zp,
             float* x_bar, float* z_bar, int* err, cudaStream_t stream) {
  if (V < 1 || V > 0x7fffffffL - TM ||
      (reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(g_bar) | reinterpret_cast<uintptr_t>(x_bar)) % 16 ||
      (base && reinterpret_cast<uintptr_t>(base) % 16) || !rows32(x_bar) || (base && !rows32(base)))
    return FFNO_EINVAL;
  if (C == 64) return launch_gate_bwd<64>(x, g_bar, base, V, wpack, zp, x_bar, z_bar, err, stream);
  if (C == 32) return launch_gate_bwd<32>(x, g_bar, base, V, wpack, zp, x_bar, z_bar, err, stream);
  return FFNO_EINVAL;
}

bool gate_fwd_supported(int C) { return C == 32 || C == 64; }

int gate_fwd(const float* x, long V, int C, const void* wpack, const float* zp, const float* z, float* out, int* err,
             cudaStream_t stream) {
  if (V < 1 || V > 0x7fffffffL - TM || reinterpret_cast<uintptr_t>(x) % 16 || reinterpret_cast<uintptr_t>(out) % 16 ||
      (zp && reinterpret_cast<uintptr_t>(zp) % 16) || !rows32(x) || !rows32(out))
    return FFNO_EINVAL;
  if (C == 64) return launch_gate_fwd<64>(x, V, wpack, zp, z, out, err, stream);
  if (C == 32) return launch_gate_fwd<32>(x, V, wpack, zp, z, out, err, stream);
  return FFNO_EINVAL;
}

bool mlp2_fwd_supported(int C) { return C == 32 || C == 64; }

int mlp2_fwd(int mode, const float* in, const float* prev_pre, const float* prev_coefs, float res, float* xout, long V,
             int C, const void* wpack, const float* dw, float* pre, double* partials, int nparts, int* err,
             cudaStream_t stream) {
  if (V < 1 || V > 0x7fffffffL - TM || nparts < 1 || reinterpret_cast<uintptr_t>(in) % 16 ||
      (mode && reinterpret_cast<uintptr_t>(prev_pre) % 16) || !rows32(pre) || (mode && !rows32(xout)))
    return FFNO_EINVAL;
#define L(CC, MM)                                                                                                \
  if (C == CC && mode == MM)                                                                                     \
    return launch_mlp2_fwd<CC, MM>(in, prev_pre, prev_coefs, res, xout, V, wpack, dw, pre, partials, nparts, err, \
                                   stream);
  L(64, 0) L(64, 1) L(64, 2) L(32, 0) L(32, 1) L(32, 2)
#undef L
  return FFNO_EINVAL;
}

bool mlp2_bwd_supported(int C) { return C == 32 || C == 64; }

int mlp2_bwd(const float* a, const float* pre_bar, const float* base, long V, int C, const void* wpack, float* a_bar,
             int* err, cudaStream_t stream) {
  if (V < 1 || V > 0x7fffffffL - TM || (reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(pre_bar)) % 16 ||
      !rows32(a_bar) || (base && !rows32(base)))
    return FFNO_EINVAL;
  if (C == 64) return launch_mlp2_bwd<64>(a, pre_bar, base, V, wpack, a_bar, err, stream);
  if (C == 32) return launch_mlp2_bwd<32>(a, pre_bar, base, V, wpack, a_bar, err, stream);
  return FFNO_EINVAL;
}

}  // namespace ws
}  // namespace ffno
