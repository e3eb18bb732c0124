// Tensor-core (tcgen05, split-BF16) versions of the spectral kernels: the batched transform GEMM that carries every
// DFT of the path (same ffno_xform_desc contract as spectral_f32.cu) and the per-frequency channel mixing.
//
// Transform GEMM: out[b][m][n] = sum_k T[m][k] in[b][k][n], computed transposed, D^T [128 data columns][M] = X^T T^T,
// so that tensor-memory lanes are data columns and the stores of a warp cover 32 consecutive columns of one output
// row. Data chunks of 64 rows k are converted from FP32 HBM into split MN-major tiles (the columns are contiguous in
// HBM); the split table is either resident in shared memory (k_xform_rt, tables up to 80 KB: the W and height
// transforms) or streamed per k-chunk next to the data (k_xform_st: the H transforms). Accumulators live in tensor
// memory (<= 256 columns per pipeline).
#include <cudaTypedefs.h>

#include "common.cuh"
#include "tc.cuh"

using namespace ffno;

namespace ffno {
int launch_mix_tc96(const float* in, float* out, long F, long nb, long sf, long sb, long s_im, const void* wpack,
                    const float* g, const float* U, const float* Vm, int rank, int* err, cudaStream_t s);
}

namespace {

constexpr int XT = 512;    // threads of the mixing kernel
constexpr int XKC = 32;    // k per chunk of the streamed table pack (and data rows per chunk of k_xform_st)
constexpr int XMT = 2;     // max m tiles of 128 (a transform call has at most 256 output rows)

// one (m-tile, k-chunk) block of the streamed table pack: 128 rows x kc, split hi + lo
__host__ __device__ constexpr uint32_t a_chunk_bytes(int kc) { return 128u * kc * 2 * 2; }

__device__ __forceinline__ bool bounded(bool ok, int* err, int code) {
  const bool all = __syncthreads_and(ok) != 0;
  if (!all && threadIdx.x == 0) atomicExch(err, code);
  return all;
}

// ------------------------------------------------------------------------------------------- resident table
// The transform GEMM with the whole split table resident in shared memory, in the transposed orientation:
// D^T [128 data columns n][M rows m] = X^T T^T, with X a chunk of 64 data rows k x 128 columns n (A operand, MN-major:
// n contiguous, as in HBM) and T the table [Mp][Kp] (B operand, K-major). The tensor-memory lane is the data column
// n, so the stores of one warp cover 32 consecutive columns of one output row. An item is 128 columns: one n-tile of
// one batch, or 128 / N whole batches when N divides 128 (the W transforms, N = C). Two pipelines of 256 threads per
// CTA take alternate items, each with two data stages (double-buffered against the MMAs), 256 tensor-memory columns
// and its own mbarriers; the table is shared. Every wait is bounded.
constexpr int RT = 256;                     // threads per pipeline
constexpr int RKC = 64;                     // data rows k per chunk
constexpr uint32_t RSB = 128u * RKC * 2;    // one split half of a data stage
constexpr int RT_MAXK = 512;                // largest padded K of a resident table

__device__ __forceinline__ void rt_sync(int pipe) { asm volatile("bar.sync %0, %1;" ::"r"(1 + pipe), "n"(RT) : "memory"); }
__device__ __forceinline__ bool rt_sync_and(int pipe, bool p) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred pi, po;\n setp.ne.u32 pi, %1, 0;\n bar.red.and.pred po, %2, %3, pi;\n selp.u32 %0, 1, 0, po;\n}"
      : "=r"(r)
      : "r"((uint32_t)p), "r"(1 + pipe), "n"(RT)
      : "memory");
  return r != 0;
}

// Fill of one data stage (rows k0 .. k0 + kc of the chunk, 128 columns) from FP32 HBM into the split MN-major tile.
// A piece is 8 consecutive columns of one row (one 32-byte load). Lanes take 8 rows (lane & 7) x 4 column octets
// (lane >> 3) and warps (w & 3) four groups of octets, so a warp reads 8 rows x 128 contiguous bytes, and each 8-lane
// phase of its 16-byte stores covers 8 rows of one octet: 128 contiguous bytes of the tile, free of bank conflicts.
// Row k0 + kr of piece u is kr = 8 (2u + (w >> 2)) + (lane & 7); the columns nf..nf+7 depend on the thread only.
// NP pieces a thread: NP x 32 bytes in flight, the whole chunk of 16 NP rows per pipeline (NP = 4: the 64-row chunks
// of k_xform_rt; NP = 2: the 32-row chunks of k_xform_st). hb: bytes of one split half of the stage.
constexpr int XFB8 = 4;
static_assert(XFB8 * RT * 8 == RKC * 128, "the pieces of a pipeline cover a whole chunk");
static_assert(2 * RT * 8 == XKC * 128, "the pieces of a pipeline cover a whole streamed chunk");

__device__ __forceinline__ int xf_fill_col(int ptid, int lane) { return 8 * (4 * ((ptid >> 5) & 3) + (lane >> 3)); }

template <int NP>
__device__ __forceinline__ void xf_fill_chunk(uint8_t* st, uint32_t hb, const float* fsrc, bool fv,
                                              const long* row_in, int K, int k0, int kc, int ptid, int lane, int nf) {
  const int w = (ptid >> 5) & 7;
  float v[NP][8];
#pragma unroll
  for (int u = 0; u < NP; ++u) {   // every load of the chunk issued before any is converted
    const int kr = 8 * (2 * u + (w >> 2)) + (lane & 7);
    const int k = k0 + kr;
    if (kr < kc && k < K && fv) {
      tc::ld8(fsrc + row_in[k], v[u]);
    } else {
#pragma unroll
      for (int i = 0; i < 8; ++i) v[u][i] = 0.f;
    }
  }
#pragma unroll
  for (int u = 0; u < NP; ++u) {
    const int kr = 8 * (2 * u + (w >> 2)) + (lane & 7);
    if (kr >= kc) break;
    uint32_t h[4], l[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) tc::split_pack(v[u][2 * i], v[u][2 * i + 1], h[i], l[i]);
    const uint32_t o = tc::mnmajor_offset(nf, kr, 128);
    *reinterpret_cast<uint4*>(st + o) = make_uint4(h[0], h[1], h[2], h[3]);
    *reinterpret_cast<uint4*>(st + hb + o) = make_uint4(l[0], l[1], l[2], l[3]);
  }
}

__global__ void __launch_bounds__(2 * RT, 1)
    k_xform_rt(const uint8_t* __restrict__ tpack, int Mp, int Kp, const float* __restrict__ in, float* __restrict__ out,
               ffno_xform_desc d, int nbi, int nshift, long ntn, long items, int accumulate, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = smem_raw + ((1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u);
  const uint32_t TB = (uint32_t)Mp * Kp * 2;                 // one split half of the table
  uint8_t* sT = base;
  uint8_t* sD = base + ((2 * TB + 1023u) & ~1023u);          // [pipe][stage][hi | lo]
  __shared__ uint64_t bar_t, bar_m[2][2];
  __shared__ uint32_t tslot;
  __shared__ long row_in[RT_MAXK], row_out[256];   // element offsets of data row k and output row m
  const int tid = threadIdx.x, pipe = tid / RT, ptid = tid % RT, warp = tid >> 5, lane = tid & 31;
  const int q = warp & 3, half = ptid >> 7;
  for (int k = tid; k < Kp; k += 2 * RT) row_in[k] = (long)(k / d.in_split) * d.in_hi + (long)(k % d.in_split) * d.in_lo;
  for (int m = tid; m < Mp; m += 2 * RT)
    row_out[m] = (long)(m / d.out_split) * d.out_hi + (long)(m % d.out_split) * d.out_lo;
  if (warp == 0) tc::tmem_alloc(&tslot, 512);
  if (tid == 0) {
    tc::mbar_init(&bar_t, 1);
    for (int i = 0; i < 4; ++i) tc::mbar_init(&bar_m[i >> 1][i & 1], 1);
    tc::mbar_init_fence();
    tc::mbar_arrive_expect_tx(&bar_t, 2 * TB);
    for (uint32_t off = 0; off < 2 * TB; off += 32768u)
      tc::bulk_g2s(sT + off, tpack + off, (2 * TB - off) < 32768u ? (2 * TB - off) : 32768u, &bar_t);
  }
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  const uint32_t tmem = tslot + (uint32_t)pipe * 256u;
  const uint32_t lq = (uint32_t)(32 * q) << 16;
  bool ok = __syncthreads_and(tc::mbar_wait(&bar_t, 0)) != 0;
  if (!ok && tid == 0) atomicExch(err, 1);
  const int nch = (Kp + RKC - 1) / RKC;
  const uint32_t idesc = tc::idesc_bf16_ab(128, Mp, true, false);
  const uint32_t t_hi = tc::smem_u32(sT), t_lo = t_hi + TB;
  uint32_t g = 0;                                            // chunks issued by this pipeline
  const int n_ep = 32 * q + lane;                            // epilogue column of this thread
  for (long it = 2L * blockIdx.x + pipe; ok && it < items; it += 2L * gridDim.x) {
    long bfirst, n0;
    if (nbi > 1) {
      bfirst = it * nbi;
      n0 = 0;
    } else {
      bfirst = it / ntn;
      n0 = (it % ntn) * 128;
    }
    // every fill piece of this thread covers the same 8 columns nf..nf+7 (see the piece mapping below)
    const int nf = xf_fill_col(ptid, lane);
    long foff = 0;
    bool fv;
    {
      long b, c;
      if (nbi > 1) {
        b = bfirst + (nf >> nshift);
        c = nf & ((1 << nshift) - 1);
      } else {
        b = bfirst;
        c = n0 + nf;
      }
      fv = b < d.nb && c < d.N;
      if (fv) foff = (b / d.nb2) * d.in_b1 + (b % d.nb2) * d.in_b2 + c;
    }
    const float* fsrc = in + foff;
    for (int ch = 0; ch < nch; ++ch, ++g) {
      const int s = (int)(g & 1u);
      const int k0 = ch * RKC, kc = (Kp - k0) < RKC ? (Kp - k0) : RKC;
      if (g >= 2) {
        const bool w = tc::mbar_wait(&bar_m[pipe][s], ((g - 2) >> 1) & 1u);
        if (!(ok = rt_sync_and(pipe, w))) break;
      }
      uint8_t* st = sD + (uint32_t)(pipe * 2 + s) * 2u * RSB;
      xf_fill_chunk<XFB8>(st, RSB, fsrc, fv, row_in, d.K, k0, kc, ptid, lane, nf);
      tc::fence_async_smem();
      tc::tc_before_sync();
      rt_sync(pipe);
      tc::tc_after_sync();
      if (ptid == 0) {
        const uint32_t x_hi = tc::smem_u32(st), x_lo = x_hi + RSB;
        const uint32_t as[3] = {x_hi, x_hi, x_lo}, bs[3] = {t_hi, t_lo, t_hi};
#pragma unroll
        for (int ps = 0; ps < 3; ++ps)
          for (int kk = 0; kk < kc; kk += 16) {
            const uint64_t ad = tc::mnmajor_desc(as[ps] + (uint32_t)(kk / 8) * 2048u, 2048u, 128u);
            const uint64_t bd = tc::kmajor_desc(bs[ps] + (uint32_t)((k0 + kk) / 8) * 128u, 128u, (uint32_t)Kp * 16u);
            tc::mma_bf16(tmem, ad, bd, idesc, (ch > 0 || ps > 0 || kk > 0) ? 1u : 0u);
          }
        tc::mma_commit(&bar_m[pipe][s]);
      }
    }
    if (!ok) break;
    {
      const uint32_t gl = g - 1;
      const bool w = tc::mbar_wait(&bar_m[pipe][gl & 1u], (gl >> 1) & 1u);
      if (!(ok = rt_sync_and(pipe, w))) break;
      tc::tc_after_sync();
    }
    // epilogue: lane = column n; the two halves of the pipeline take alternate 16-row chunks of m
    long obase = 0;
    bool nv;
    {
      long b, c;
      if (nbi > 1) {
        b = bfirst + (n_ep >> nshift);
        c = n_ep & ((1 << nshift) - 1);
      } else {
        b = bfirst;
        c = n0 + n_ep;
      }
      nv = b < d.nb && c < d.N;
      if (nv) obase = (b / d.nb2) * d.out_b1 + (b % d.nb2) * d.out_b2 + c;
    }
    for (int jj = half; jj < Mp / 16; jj += 2) {
      float v[16];
      tc::tmem_ld16(tmem + lq + 16u * jj, v);
      if (nv) {
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int m = 16 * jj + i;
          if (m < d.M) {
            float* p = out + obase + row_out[m];
            *p = accumulate ? *p + v[i] : v[i];
          }
        }
      }
    }
    tc::tc_before_sync();
    rt_sync(pipe);
    tc::tc_after_sync();
  }
  if (!ok) {   // leave no MMA in flight before freeing tensor memory
    if (g >= 1) tc::mbar_wait(&bar_m[pipe][(g - 1) & 1u], ((g - 1) >> 1) & 1u);
    if (g >= 2) tc::mbar_wait(&bar_m[pipe][g & 1u], ((g - 2) >> 1) & 1u);
  }
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  if (warp == 0) tc::tmem_free(tslot, 512);
}

// ------------------------------------------------------------------------------------------- streamed table
// The transposed transform GEMM of k_xform_rt for tables too large to keep resident (the H transforms, K = M = 2H):
// per 32-row k-chunk the table slice [MT * 128][kc] (from the m-tile / k-chunk pack of ffno_xform_tc) arrives by
// bulk copies into the stage next to the data chunk, both double-buffered against the MMAs. Chunks of 32 rows k keep
// a CTA's stages near 100 KB, so that two CTAs of 256 threads share an SM (each with 256 tensor-memory columns).
constexpr uint32_t SSB = 128u * XKC * 2;    // one split half of a data stage of k_xform_st
__global__ void __launch_bounds__(RT, 2)
    k_xform_st(const uint8_t* __restrict__ tpack, int MT, int Kp, const float* __restrict__ in, float* __restrict__ out,
               ffno_xform_desc d, int nbi, int nshift, long ntn, long items, int accumulate, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = smem_raw + ((1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u);
  const uint32_t TSB = (uint32_t)MT * 128u * XKC * 2;        // one split half of a table stage
  uint8_t* sD = base;                                        // [stage][hi | lo], 2 * SSB each
  uint8_t* sT = base + 4 * SSB;                              // [stage][hi | lo], 2 * TSB each
  __shared__ uint64_t bar_t[2], bar_m[2];
  __shared__ uint32_t tslot;
  __shared__ long row_in[RT_MAXK], row_out[256];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, q = warp & 3, half = tid >> 7;
  const int Mp = MT * 128;
  for (int k = tid; k < Kp; k += RT) row_in[k] = (long)(k / d.in_split) * d.in_hi + (long)(k % d.in_split) * d.in_lo;
  for (int m = tid; m < Mp; m += RT) row_out[m] = (long)(m / d.out_split) * d.out_hi + (long)(m % d.out_split) * d.out_lo;
  if (warp == 0) tc::tmem_alloc(&tslot, 256);
  if (tid == 0) {
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&bar_t[i], 1);
      tc::mbar_init(&bar_m[i], 1);
    }
    tc::mbar_init_fence();
  }
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  const uint32_t tmem = tslot;
  const uint32_t lq = (uint32_t)(32 * q) << 16;
  const int nch = (Kp + XKC - 1) / XKC;
  const uint32_t idesc = tc::idesc_bf16_ab(128, Mp, true, false);
  const uint32_t mt_bytes = (uint32_t)128 * Kp * 2 * 2;
  bool ok = true;
  uint32_t g = 0;
  const int n_ep = 32 * q + lane;
  for (long it = blockIdx.x; ok && it < items; it += gridDim.x) {
    long bfirst, n0;
    if (nbi > 1) {
      bfirst = it * nbi;
      n0 = 0;
    } else {
      bfirst = it / ntn;
      n0 = (it % ntn) * 128;
    }
    const int nf = xf_fill_col(tid, lane);
    long foff = 0;
    bool fv;
    {
      long b, c;
      if (nbi > 1) {
        b = bfirst + (nf >> nshift);
        c = nf & ((1 << nshift) - 1);
      } else {
        b = bfirst;
        c = n0 + nf;
      }
      fv = b < d.nb && c < d.N;
      if (fv) foff = (b / d.nb2) * d.in_b1 + (b % d.nb2) * d.in_b2 + c;
    }
    const float* fsrc = in + foff;
    for (int ch = 0; ch < nch; ++ch, ++g) {
      const int s = (int)(g & 1u);
      const int k0 = ch * XKC, kc = (Kp - k0) < XKC ? (Kp - k0) : XKC;
      if (g >= 2) {
        const bool w = tc::mbar_wait(&bar_m[s], ((g - 2) >> 1) & 1u);
        if (!(ok = bounded(w, err, 3))) break;
      }
      uint8_t* st = sD + (uint32_t)s * 2u * SSB;
      uint8_t* tt = sT + (uint32_t)s * 2u * TSB;
      if (tid == 0) {   // the table slice of this chunk: m-tiles stacked, hi then lo
        const uint32_t part = 128u * kc * 2;
        tc::mbar_arrive_expect_tx(&bar_t[s], 2u * MT * part);
        for (int mt = 0; mt < MT; ++mt) {
          const uint8_t* src = tpack + (size_t)mt * mt_bytes + (size_t)ch * a_chunk_bytes(XKC);
          tc::bulk_g2s(tt + mt * part, src, part, &bar_t[s]);
          tc::bulk_g2s(tt + (uint32_t)MT * part + mt * part, src + part, part, &bar_t[s]);
        }
      }
      xf_fill_chunk<2>(st, SSB, fsrc, fv, row_in, d.K, k0, kc, tid, lane, nf);
      tc::fence_async_smem();
      const bool wt = tc::mbar_wait(&bar_t[s], (g >> 1) & 1u);
      tc::tc_before_sync();
      if (!(ok = bounded(wt, err, 1))) break;
      tc::tc_after_sync();
      if (tid == 0) {
        const uint32_t x_hi = tc::smem_u32(st), x_lo = x_hi + SSB;
        const uint32_t t_hi = tc::smem_u32(tt), t_lo = t_hi + (uint32_t)MT * 128u * kc * 2;
        const uint32_t as[3] = {x_hi, x_hi, x_lo}, bs[3] = {t_hi, t_lo, t_hi};
#pragma unroll
        for (int ps = 0; ps < 3; ++ps)
          for (int kk = 0; kk < kc; kk += 16) {
            const uint64_t ad = tc::mnmajor_desc(as[ps] + (uint32_t)(kk / 8) * 2048u, 2048u, 128u);
            const uint64_t bd = tc::kmajor_desc(bs[ps] + (uint32_t)(kk / 8) * 128u, 128u, (uint32_t)kc * 16u);
            tc::mma_bf16(tmem, ad, bd, idesc, (ch > 0 || ps > 0 || kk > 0) ? 1u : 0u);
          }
        tc::mma_commit(&bar_m[s]);
      }
    }
    if (!ok) break;
    {
      const uint32_t gl = g - 1;
      const bool w = tc::mbar_wait(&bar_m[gl & 1u], (gl >> 1) & 1u);
      if (!(ok = bounded(w, err, 3))) break;
      tc::tc_after_sync();
    }
    long obase = 0;
    bool nv;
    {
      long b, c;
      if (nbi > 1) {
        b = bfirst + (n_ep >> nshift);
        c = n_ep & ((1 << nshift) - 1);
      } else {
        b = bfirst;
        c = n0 + n_ep;
      }
      nv = b < d.nb && c < d.N;
      if (nv) obase = (b / d.nb2) * d.out_b1 + (b % d.nb2) * d.out_b2 + c;
    }
    for (int jj = half; jj < Mp / 16; jj += 2) {
      float v[16];
      tc::tmem_ld16(tmem + lq + 16u * jj, v);
      if (nv) {
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int m = 16 * jj + i;
          if (m < d.M) {
            float* p = out + obase + row_out[m];
            *p = accumulate ? *p + v[i] : v[i];
          }
        }
      }
    }
    tc::tc_before_sync();
    __syncthreads();
    tc::tc_after_sync();
  }
  if (!ok) {   // leave no bulk copy or MMA in flight before freeing tensor memory
    tc::mbar_wait(&bar_t[0], 0);
    tc::mbar_wait(&bar_t[1], 0);
    if (g >= 1) tc::mbar_wait(&bar_m[(g - 1) & 1u], ((g - 1) >> 1) & 1u);
    if (g >= 2) tc::mbar_wait(&bar_m[g & 1u], ((g - 2) >> 1) & 1u);
  }
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  if (warp == 0) tc::tmem_free(tmem, 256);
}

// ---------------------------------------------------------------------------------------------------- mixing
// Per-frequency mixing on tensor cores: out_f = g_f (W x_f) + U_f (V_f x_f) for every row b of frequency f, with
// x = [re | im] (2C values), W the [2C x 2C] channel map and g_f complex. A CTA item = 128 rows b of one frequency;
// the grid is persistent.
//   * The item's FP32 rows arrive by tiled TMA loads (a 4-D tensor map over channel, f, b and re/im, the outer three
//     sorted by stride; 128-byte swizzle) into a staging buffer, issued one item ahead.
//   * The threads split them into X (split BF16, K-major [128 b][2C]) and the item's V_f into a block-diagonal
//     [16][2C] operand (rows 0..7 act on the re half, rows 8..15 on the im half).
//   * MMAs: D^T [2C (padded to 128) x 128 b] = W X^T (W resident in shared memory as the A operand) and the low-rank
//     projections T [128 b x 16] = X Vblk^T, into double-buffered tensor memory, so the epilogue of item i-1 runs
//     while the MMAs of item i do. After that epilogue, T of item i goes back to shared memory as a split K-major
//     tile and the low-rank term D2^T [slots x 128 b] = Ublk T^T (Ublk: U_f block-diagonal by re / im part, K = 16)
//     lands in a third accumulator, read by the epilogue of item i.
//   * Epilogue: thread = output slot p (TMEM lane). W's output rows are packed so that warp quadrant q holds the re
//     parts of channels 16q..16q+15 (lanes 0-15) and their im parts (lanes 16-31): the re and im lanes of a channel
//     swap their values with one shuffle to apply g_f; y = g_f D + D2; 16 warps, each over 32 rows b of its lane
//     quadrant; one warp's stores cover 16 consecutive channels of the re and of the im part.
constexpr int MIX_RANK_TC = 8;   // low-rank terms carried by the tensor-core mixing (larger ranks use k_mix)

struct MixGeom {
  int mul_b, mul_ri;   // staging row of (b, re/im) inside a box: b * mul_b + ri * mul_ri
  int o1, o2, o3;      // logical dimension (0 f, 1 b, 2 re/im) of tensor-map dimensions 1..3
};


template <int C>
__global__ void __launch_bounds__(XT, 1)
    k_mix_tc(const __grid_constant__ CUtensorMap tmap, float* __restrict__ out, long F, long nb, long sf, long sb,
             long s_im, const uint8_t* __restrict__ wpack, const float* __restrict__ g, const float* __restrict__ U,
             const float* __restrict__ Vm, int rank, MixGeom geo, int* __restrict__ err) {
  constexpr int K2 = 2 * C;
  constexpr int CB = C < 32 ? C : 32;       // channels per staging row (one box row)
  constexpr int NH = C / CB;                // boxes per item
  constexpr int CPR = CB / 4;               // 16-byte chunks per staging row
  constexpr uint32_t ROWB = CB * 4;
  constexpr uint32_t HALF = 256u * ROWB;    // one box: 128 rows b x (re, im)
  constexpr bool SWZ = (CB == 32);
  constexpr uint32_t WB = 128u * K2 * 2;    // one split half (hi or lo) of a 128-row operand
  constexpr uint32_t WP = (uint32_t)K2 * K2 * 2;   // one split half of the packed [2C][2C] weight
  constexpr int NT = 16;                    // low-rank operand rows / columns
  constexpr uint32_t LB = 128u * NT * 2;    // one split half of a [128][16] operand
  constexpr uint32_t TD2 = 384;             // tensor-memory column of the low-rank accumulator
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = smem_raw + ((1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u);
  uint8_t* sW = base;                  // hi [0, WB), lo [WB, 2 WB)
  uint8_t* sX = base + 2 * WB;
  uint8_t* sS = base + 4 * WB;         // staging, 1024-byte aligned (WB is a multiple of 1024)
  uint8_t* sV = sS + NH * HALF;        // Vblk [16][K2]: hi, then lo
  uint8_t* sU = sV + 2u * NT * K2 * 2; // Ublk [128 slots][16]: hi, then lo
  uint8_t* sT = sU + 2u * LB;          // T [128 b][16]: hi, then lo
  __shared__ uint64_t bar_w, bar_s, bar_m[2], bar_r;
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, q = warp & 3, wg = warp >> 2;
  if (warp == 0) tc::tmem_alloc(&tslot, 512);
  if (tid == 0) {
    tc::mbar_init(&bar_w, 1);
    tc::mbar_init(&bar_s, 1);
    tc::mbar_init(&bar_m[0], 1);
    tc::mbar_init(&bar_m[1], 1);
    tc::mbar_init(&bar_r, 1);
    tc::mbar_init_fence();
  }
  // zero the padding rows 2C..127 of W (hi and lo); they are contiguous at the end of each half
  for (uint32_t e = 2u * C * K2 * 2 + tid * 16u; e < WB; e += XT * 16u) {
    *reinterpret_cast<uint4*>(sW + e) = make_uint4(0u, 0u, 0u, 0u);
    *reinterpret_cast<uint4*>(sW + WB + e) = make_uint4(0u, 0u, 0u, 0u);
  }
  tc::fence_async_smem();
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  const uint32_t tmem = tslot;
  const uint32_t lq = (uint32_t)(32 * q) << 16;
  const long nbt = (nb + 127) / 128, items = F * nbt;
  auto issue_load = [&](long item) {
    const long f = item / nbt, b0 = (item % nbt) * 128;
    int c[4];
    const int oo[3] = {geo.o1, geo.o2, geo.o3};
#pragma unroll
    for (int k = 0; k < 3; ++k) c[k + 1] = oo[k] == 0 ? (int)f : (oo[k] == 1 ? (int)b0 : 0);
    tc::mbar_arrive_expect_tx(&bar_s, NH * HALF);
#pragma unroll
    for (int h = 0; h < NH; ++h) tc::tma_load_4d(sS + h * HALF, &tmap, h * CB, c[1], c[2], c[3], &bar_s);
  };
  long it = blockIdx.x;
  if (tid == 0) {
    tc::mbar_arrive_expect_tx(&bar_w, 2 * WP);
    tc::bulk_g2s(sW, wpack, WP, &bar_w);
    tc::bulk_g2s(sW + WB, wpack + WP, WP, &bar_w);
    if (it < items) issue_load(it);
  }
  bool ok = bounded(tc::mbar_wait(&bar_w, 0), err, 1);
  bool load_pending = it < items;         // the load of the next item to process is in flight
  uint32_t n1 = 0, n2 = 0;                // commits issued on bar_m (main products) and bar_r (low-rank term)
  long pf = 0, pb0 = 0;
  float pgr = 0.f, pgi = 0.f;
  const int p = 32 * q + lane;            // output slot of this thread in the epilogue (its TMEM lane)
  const bool live = p < 2 * C;
  const int part = lane >> 4, pc = 16 * q + (lane & 15);   // re / im part and channel of slot p

  // y = g_f D + (U_f t) for the rows of item (f, b0) from accumulator buffer buf and the low-rank accumulator
  auto epilogue = [&](uint32_t buf, long f, long b0, float gr, float gi) {
    float* ob = out + f * sf + part * s_im + pc;
    const float ga = gr, gb = part ? gi : -gi;   // y = ga * own + gb * partner
#pragma unroll 1
    for (int cch = 0; cch < 2; ++cch) {
      const int col = 32 * wg + 16 * cch;
      float v[16], w[16], r[16];
      tc::tmem_ld16(tmem + lq + buf * 128u + (uint32_t)col, v);
      if (rank) tc::tmem_ld16(tmem + lq + TD2 + (uint32_t)col, r);
#pragma unroll
      for (int i = 0; i < 16; ++i) w[i] = __shfl_xor_sync(0xffffffffu, v[i], 16);
      if (live) {
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const long b = b0 + col + i;
          if (b < nb) {
            float y = fmaf(ga, v[i], gb * w[i]);
            if (rank) y += r[i];
            ob[b * sb] = y;
          }
        }
      }
    }
    tc::tc_before_sync();
    __syncthreads();
    tc::tc_after_sync();
  };

  // this thread's elements of an item's block-diagonal V_f (pairs e = tid + i XT < NT K2 / 2) and U_f (pairs
  // e = tid + i XT < 128 NT / 2) operands, loaded one item ahead so that their latency stays off the item's path
  static_assert(NT * K2 / 2 <= 2 * XT && 128 * NT / 2 == 2 * XT, "two V_f and two U_f pairs a thread");
  float vn[2][2] = {}, un[2][2] = {};
  auto load_vu = [&](long it2) {
    const long f2 = it2 / nbt;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int e = tid + i * XT;
      const int n = e / (K2 / 2), k = (e % (K2 / 2)) * 2;
      const int kp = k >= C ? 1 : 0, c = k - kp * C;
      const int r = n & 7;
      vn[i][0] = vn[i][1] = 0.f;
      if (e < NT * K2 / 2 && r < rank && (n >> 3) == kp) {
        const float* vr = Vm + (f2 * rank + r) * (long)C + c;
        vn[i][0] = __ldg(vr);
        vn[i][1] = __ldg(vr + 1);
      }
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const int e = tid + i * XT;
      const int ps = e / (NT / 2), k = (e % (NT / 2)) * 2;
      const int sp = (ps & 31) >> 4, sc = 16 * (ps >> 5) + (ps & 15);
      un[i][0] = un[i][1] = 0.f;
      if (ps < 2 * C && (k >> 3) == sp) {
        const int r = k & 7;
        const float* ur = U + (f2 * C + sc) * (long)rank;
        if (r < rank) un[i][0] = __ldg(ur + r);
        if (r + 1 < rank) un[i][1] = __ldg(ur + r + 1);
      }
    }
  };
  if (rank && it < items) load_vu(it);
  uint32_t j = 0;
  for (; ok && it < items; it += gridDim.x, ++j) {
    const long f = it / nbt, b0 = (it % nbt) * 128;
    const uint32_t buf = j & 1u;
    // staged rows of item j; the MMAs of item j-1 (sX free) and its low-rank product (sU, sT free, D2 ready)
    const bool w1 = tc::mbar_wait(&bar_s, j & 1u);
    const bool w2 = n1 ? tc::mbar_wait(&bar_m[(n1 - 1) & 1u], ((n1 - 1) >> 1) & 1u) : true;
    const bool w3 = n2 ? tc::mbar_wait(&bar_r, (n2 - 1) & 1u) : true;
    if (!(ok = bounded(w1 && w2 && w3, err, 2))) break;
    load_pending = false;
    tc::tc_after_sync();
    // split the staged rows into X
    for (int e = tid; e < 128 * NH * CPR; e += XT) {
      const int c4 = e % CPR, rest = e / CPR;
      const int bb = rest & 127, h = rest >> 7;
      const int rre = bb * geo.mul_b, rim = rre + geo.mul_ri;
      const uint8_t* hb = sS + h * HALF;
      const float4 xr = *reinterpret_cast<const float4*>(hb + rre * ROWB + ((SWZ ? (c4 ^ (rre & 7)) : c4) << 4));
      const float4 xi = *reinterpret_cast<const float4*>(hb + rim * ROWB + ((SWZ ? (c4 ^ (rim & 7)) : c4) << 4));
      const int k = h * CB + c4 * 4;
      uint32_t h0, l0, h1, l1;
      tc::split_pack(xr.x, xr.y, h0, l0);
      tc::split_pack(xr.z, xr.w, h1, l1);
      *reinterpret_cast<uint2*>(sX + tc::kmajor_offset(bb, k, K2)) = make_uint2(h0, h1);
      *reinterpret_cast<uint2*>(sX + WB + tc::kmajor_offset(bb, k, K2)) = make_uint2(l0, l1);
      tc::split_pack(xi.x, xi.y, h0, l0);
      tc::split_pack(xi.z, xi.w, h1, l1);
      *reinterpret_cast<uint2*>(sX + tc::kmajor_offset(bb, C + k, K2)) = make_uint2(h0, h1);
      *reinterpret_cast<uint2*>(sX + WB + tc::kmajor_offset(bb, C + k, K2)) = make_uint2(l0, l1);
    }
    if (rank) {
      // block-diagonal V_f: rows 0..r-1 act on the re half, rows 8..8+r-1 on the im half, the others are zero
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int e = tid + i * XT;
        if (e >= NT * K2 / 2) break;
        const int n = e / (K2 / 2), k = (e % (K2 / 2)) * 2;
        uint32_t hi, lo;
        tc::split_pack(vn[i][0], vn[i][1], hi, lo);
        *reinterpret_cast<uint32_t*>(sV + tc::kmajor_offset(n, k, K2)) = hi;
        *reinterpret_cast<uint32_t*>(sV + (uint32_t)NT * K2 * 2 + tc::kmajor_offset(n, k, K2)) = lo;
      }
      // block-diagonal U_f by output slot: slot p (part, channel pc) takes U_f[pc][0..r) in columns 8 part + r
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int e = tid + i * XT;
        const int ps = e / (NT / 2), k = (e % (NT / 2)) * 2;
        uint32_t hi, lo;
        tc::split_pack(un[i][0], un[i][1], hi, lo);
        *reinterpret_cast<uint32_t*>(sU + tc::kmajor_offset(ps, k, NT)) = hi;
        *reinterpret_cast<uint32_t*>(sU + LB + tc::kmajor_offset(ps, k, NT)) = lo;
      }
    }
    tc::fence_async_smem();
    tc::tc_before_sync();
    __syncthreads();
    tc::tc_after_sync();
    load_pending = it + gridDim.x < items;
    if (rank && load_pending) load_vu(it + gridDim.x);   // the next item's V_f and U_f, used after its rows land
    if (tid == 0) {
      if (load_pending) issue_load(it + gridDim.x);
      const uint32_t w_hi = tc::smem_u32(sW), x_hi = tc::smem_u32(sX);
      tc::gemm3_128xN(tmem + buf * 128u, w_hi, w_hi + WB, x_hi, x_hi + WB, K2, 128);
      if (rank) {
        const uint32_t v_hi = tc::smem_u32(sV);
        tc::gemm3_128xN(tmem + 256u + buf * 16u, x_hi, x_hi + WB, v_hi, v_hi + (uint32_t)NT * K2 * 2, K2, NT);
      }
      tc::mma_commit(&bar_m[buf]);
    }
    ++n1;
    if (j) epilogue((j - 1) & 1u, pf, pb0, pgr, pgi);   // ends with a barrier: D2 has been read
    if (rank) {
      // t = X V_f^T of item j (lanes = rows b) into a split K-major tile, then D2 = Ublk T^T
      if (!(ok = bounded(tc::mbar_wait(&bar_m[buf], (j >> 1) & 1u), err, 4))) {
        ++j;
        break;
      }
      tc::tc_after_sync();
      if (wg == 0) {
        float t[16];
        tc::tmem_ld16(tmem + lq + 256u + buf * 16u, t);
        const int bl = 32 * q + lane;
        uint32_t h[8], l[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) tc::split_pack(t[2 * i], t[2 * i + 1], h[i], l[i]);
        const uint32_t o0 = tc::kmajor_offset(bl, 0, NT), o1 = tc::kmajor_offset(bl, 8, NT);
        *reinterpret_cast<uint4*>(sT + o0) = make_uint4(h[0], h[1], h[2], h[3]);
        *reinterpret_cast<uint4*>(sT + o1) = make_uint4(h[4], h[5], h[6], h[7]);
        *reinterpret_cast<uint4*>(sT + LB + o0) = make_uint4(l[0], l[1], l[2], l[3]);
        *reinterpret_cast<uint4*>(sT + LB + o1) = make_uint4(l[4], l[5], l[6], l[7]);
      }
      tc::fence_async_smem();
      tc::tc_before_sync();
      __syncthreads();
      tc::tc_after_sync();
      if (tid == 0) {
        const uint32_t u_hi = tc::smem_u32(sU), t_hi = tc::smem_u32(sT);
        tc::gemm3_128xN(tmem + TD2, u_hi, u_hi + LB, t_hi, t_hi + LB, NT, 128);
        tc::mma_commit(&bar_r);
      }
      ++n2;
    }
    pf = f;
    pb0 = b0;
    pgr = __ldg(g + 2 * f);
    pgi = __ldg(g + 2 * f + 1);
  }
  if (ok && j) {
    const bool w1 = tc::mbar_wait(&bar_m[(n1 - 1) & 1u], ((n1 - 1) >> 1) & 1u);
    const bool w2 = n2 ? tc::mbar_wait(&bar_r, (n2 - 1) & 1u) : true;
    if ((ok = bounded(w1 && w2, err, 3))) {
      tc::tc_after_sync();
      epilogue((j - 1) & 1u, pf, pb0, pgr, pgi);
    }
  }
  if (!ok) {   // leave no bulk copy or MMA in flight before freeing tensor memory
    tc::mbar_wait(&bar_w, 0);
    if (load_pending) tc::mbar_wait(&bar_s, j & 1u);
    if (n1) tc::mbar_wait(&bar_m[(n1 - 1) & 1u], ((n1 - 1) >> 1) & 1u);
    if (n2) tc::mbar_wait(&bar_r, (n2 - 1) & 1u);
  }
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  if (warp == 0) tc::tmem_free(tmem, 512);
}

// ------------------------------------------------------------------------------------------- A B^T split-K
// part[split][i][j] = sum over the split's range of n of A[i][n] B[j][n], A [Ma][N] and B [Mb][N] FP32 rows (the
// gradient of a height-transform table: cotangent rows against transform-input rows, summed over every column and
// channel). One CTA per split, 512 threads. Per chunk of 64 n, the rows of A (TI tiles of 128, rows past Ma zero) and
// of B (NB rows, past Mb zero) are loaded from HBM, split into hi / lo K-major tiles and multiplied on the tensor cores
// into accumulators D_t [128][NB] (tile t at tensor-memory column t NB), which sum over all the split's chunks. With
// two tile buffers (NS = 2) the loads of chunk c + 1 run while the MMAs of chunk c do; a buffer is refilled after the
// mbarrier of its previous MMAs. Element (i, j) of a split's product is stored at part[split so + i si + j sj], so a
// caller can put the longer of its two operands on the M side and store the transpose. Every wait is bounded.
constexpr int OT = 512;    // threads
constexpr int OKC = 64;    // n per chunk
constexpr int OFB = 8;     // loads in flight per thread

__host__ __device__ constexpr uint32_t outer_stage_bytes(int TI, int NB) {
  return (uint32_t)(TI * 128 + NB) * OKC * 2 * 2;
}

__global__ void __launch_bounds__(OT, 1) k_outer_tc(const float* __restrict__ A, long lda, int Ma,
                                                    const float* __restrict__ B, long ldb, int Mb, long N, int TI,
                                                    int NB, int NS, long cps, float* __restrict__ part, long so,
                                                    long si, long sj, int* __restrict__ err) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = smem_raw + ((1024u - (tc::smem_u32(smem_raw) & 1023u)) & 1023u);
  __shared__ uint64_t bar[2];
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int RA = TI * 128, R = RA + NB;     // rows of a stage: A's tiles, then B
  const uint32_t half = (uint32_t)R * OKC * 2, stage = 2 * half;
  uint32_t ncol = 32;
  while (ncol < (uint32_t)(TI * NB)) ncol <<= 1;
  if (warp == 0) tc::tmem_alloc(&tslot, ncol);
  if (tid == 0) {
    tc::mbar_init(&bar[0], 1);
    tc::mbar_init(&bar[1], 1);
    tc::mbar_init_fence();
  }
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  const uint32_t tmem = tslot;
  const long nchunks = (N + OKC - 1) / OKC;
  const long c0 = blockIdx.x * cps, c1 = c0 + cps < nchunks ? c0 + cps : nchunks;
  const long nmine = c1 > c0 ? c1 - c0 : 0;
  const int NE = R * (OKC / 4);             // float4 pieces of a stage
  bool ok = true;
  long c = 0;
  for (; c < nmine; ++c) {
    const uint32_t b = (uint32_t)(c % NS);
    if (c >= NS && !(ok = bounded(tc::mbar_wait(&bar[b], (uint32_t)((c - NS) / NS) & 1u), err, 5))) break;
    uint8_t* hi = base + b * stage;
    uint8_t* lo = hi + half;
    const long n0 = (c0 + c) * OKC;
    for (int e0 = tid; e0 < NE; e0 += OT * OFB) {
      float4 v[OFB];
#pragma unroll
      for (int u = 0; u < OFB; ++u) {   // issue the loads before converting any of them
        // piece e = 4 values at byte e * 8 of the canonical K-major stage (conflict-free 8-byte stores): core matrix
        // e / 16 (8 rows x 8 k), its row (e / 2) % 8 and k half e % 2; a warp reads 8 rows x 64 bytes
        const int e = e0 + u * OT;
        const int cm = e >> 4, r = (cm / (OKC / 8)) * 8 + ((e >> 1) & 7), k = (cm % (OKC / 8)) * 8 + (e & 1) * 4;
        const long n = n0 + k;
        v[u] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (e < NE && n < N) {
          if (r < RA) {
            if (r < Ma) v[u] = __ldg(reinterpret_cast<const float4*>(A + r * lda + n));
          } else if (r - RA < Mb) {
            v[u] = __ldg(reinterpret_cast<const float4*>(B + (r - RA) * ldb + n));
          }
        }
      }
#pragma unroll
      for (int u = 0; u < OFB; ++u) {
        const int e = e0 + u * OT;
        if (e >= NE) break;
        uint32_t h0, l0, h1, l1;
        tc::split_pack(v[u].x, v[u].y, h0, l0);
        tc::split_pack(v[u].z, v[u].w, h1, l1);
        *reinterpret_cast<uint2*>(hi + (size_t)e * 8) = make_uint2(h0, h1);
        *reinterpret_cast<uint2*>(lo + (size_t)e * 8) = make_uint2(l0, l1);
      }
    }
    tc::fence_async_smem();
    tc::tc_before_sync();
    __syncthreads();
    tc::tc_after_sync();
    if (tid == 0) {
      const uint32_t sh = tc::smem_u32(hi), sl = sh + half;
      const uint32_t bo = (uint32_t)RA * OKC * 2;   // B's rows follow A's tiles (a multiple of 8 rows)
      for (int t = 0; t < TI; ++t) {
        const uint32_t ao = (uint32_t)t * 128u * OKC * 2, d = tmem + (uint32_t)(t * NB);
        tc::gemm_128xN(d, sh + ao, sh + bo, OKC, NB, c > 0);
        tc::gemm_128xN(d, sh + ao, sl + bo, OKC, NB, true);
        tc::gemm_128xN(d, sl + ao, sh + bo, OKC, NB, true);
      }
      tc::mma_commit(&bar[b]);
    }
  }
  // the last commit covers every MMA issued before it
  if (ok && nmine > 0) {
    const long l = nmine - 1;
    ok = bounded(tc::mbar_wait(&bar[l % NS], (uint32_t)(l / NS) & 1u), err, 6);
  }
  tc::tc_after_sync();
  if (ok) {
    const int q = warp & 3, g = warp >> 2;
    for (int t = 0; t < TI; ++t) {
      const int i = t * 128 + 32 * q + lane;
      for (int cc = g; cc < NB / 16; cc += 4) {
        float v[16];
        if (nmine > 0) {
          tc::tmem_ld16(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(t * NB + 16 * cc), v);
        } else {
#pragma unroll
          for (int m = 0; m < 16; ++m) v[m] = 0.f;
        }
        if (i < Ma) {
          float* o = part + blockIdx.x * so + i * si;
#pragma unroll
          for (int m = 0; m < 16; ++m)
            if (16 * cc + m < Mb) o[(16 * cc + m) * sj] = v[m];
        }
      }
    }
  } else if (c > 0) {   // leave no MMA in flight before freeing tensor memory
    const long l = c - 1;
    tc::mbar_wait(&bar[l % NS], (uint32_t)(l / NS) & 1u);
  }
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  if (warp == 0) tc::tmem_free(tmem, ncol);
}

// part [nsplit][rows][cols] -> out rows of stride ldo (ldo = cols: out is the contiguous [rows][cols] product)
__global__ void k_outer_tc_reduce(const float* __restrict__ part, long nsplit, long n, long cols, long ldo,
                                  double* __restrict__ out, int accumulate) {
  const long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (e >= n) return;
  double s = 0.0;
#pragma unroll 8
  for (long p = 0; p < nsplit; ++p) s += (double)part[p * n + e];   // loads issued ahead, sums in order
  double* o = out + (e / cols) * ldo + e % cols;
  *o = accumulate ? *o + s : s;
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

}  // namespace

extern "C" {

int ffno_xform_tc_pack_bytes(int M, int K) {
  const int MT = (M + 127) / 128, Kp = (K + 15) / 16 * 16;
  return MT * 128 * Kp * 2 * 2;
}

int ffno_xform_tc(const void* tpack, const float* in, float* out, const ffno_xform_desc* desc, int accumulate, int* err,
                  ffno_stream_t stream) {
  if (!tpack || !in || !out || !desc || !err || (reinterpret_cast<uintptr_t>(tpack) % 16)) return FFNO_EINVAL;
  const ffno_xform_desc& d = *desc;
  if (d.nb < 1 || d.nb2 < 1 || d.K < 1 || d.M < 1 || d.M > 128 * XMT || d.N < 1 || d.in_split < 1 ||
      d.out_split < 1)
    return FFNO_EINVAL;
  if (d.N % 8 || d.in_lo % 8 || d.in_hi % 8 || d.in_b1 % 8 || d.in_b2 % 8) return FFNO_EINVAL;  // 32-byte loads
  if (reinterpret_cast<uintptr_t>(in) % 32) return FFNO_EINVAL;
  const int Kp = (d.K + 15) / 16 * 16;
  if (Kp > RT_MAXK) return FFNO_EINVAL;
  const int MT = (d.M + 127) / 128;
  int nbi = 1, nshift = 0;
  if (d.N < 128 && 128 % d.N == 0) {
    nbi = 128 / (int)d.N;
    while ((1 << nshift) < d.N) ++nshift;
  }
  const long ntn = (d.N + 127) / 128;
  const long items = nbi > 1 ? (d.nb + nbi - 1) / nbi : d.nb * ntn;
  const size_t smem = 1024 + 4 * (size_t)SSB + 2 * 2 * (size_t)MT * 128 * XKC * 2;
  if (!ffno::smem_cap_ok(k_xform_st, smem))
    return FFNO_ELAUNCH;
  const long grid = items < 2L * sms() ? items : 2L * sms();   // two CTAs per SM
  k_xform_st<<<(unsigned)grid, RT, smem, (cudaStream_t)stream>>>(static_cast<const uint8_t*>(tpack), MT, Kp, in, out,
                                                                d, nbi, nshift, ntn, items, accumulate, err);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_xform_tcr(const void* tpack, int Mp, int Kp, const float* in, float* out, const ffno_xform_desc* desc,
                   int accumulate, int* err, ffno_stream_t stream) {
  if (!tpack || !in || !out || !desc || !err || (reinterpret_cast<uintptr_t>(tpack) % 16)) return FFNO_EINVAL;
  const ffno_xform_desc& d = *desc;
  if (d.nb < 1 || d.nb2 < 1 || d.K < 1 || d.M < 1 || d.N < 1 || d.in_split < 1 || d.out_split < 1) return FFNO_EINVAL;
  if (Mp % 16 || Mp < d.M || Mp > 256 || Kp % 16 || Kp < d.K || Kp > RT_MAXK) return FFNO_EINVAL;
  if ((size_t)Mp * Kp * 4 > ffno_xform_tcr_max_table_bytes()) return FFNO_EINVAL;
  if (d.N % 8 || d.in_lo % 8 || d.in_hi % 8 || d.in_b1 % 8 || d.in_b2 % 8) return FFNO_EINVAL;   // 32-byte loads
  if (reinterpret_cast<uintptr_t>(in) % 32) return FFNO_EINVAL;
  int nbi = 1, nshift = 0;
  if (d.N < 128 && 128 % d.N == 0) {
    nbi = 128 / (int)d.N;
    while ((1 << nshift) < d.N) ++nshift;
  }
  const long ntn = (d.N + 127) / 128;
  const long items = nbi > 1 ? (d.nb + nbi - 1) / nbi : d.nb * ntn;
  const size_t smem = 1024 + (((size_t)Mp * Kp * 4 + 1023) & ~(size_t)1023) + 4 * 2 * (size_t)RSB;
  if (!ffno::smem_cap_ok(k_xform_rt, smem))
    return FFNO_ELAUNCH;
  const long pairs = (items + 1) / 2;
  const long grid = pairs < sms() ? pairs : sms();
  k_xform_rt<<<(unsigned)grid, 2 * RT, smem, (cudaStream_t)stream>>>(static_cast<const uint8_t*>(tpack), Mp, Kp, in,
                                                                    out, d, nbi, nshift, ntn, items, accumulate, err);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_xform_tcr_max_table_bytes(void) { return 80 * 1024; }

int ffno_spectral_mix_tc(const float* in, float* out, long F, long nb, long sf, long sb, long s_im, int C,
                         const void* wpack, const float* g, const float* U, const float* Vm, int rank, int* err,
                         ffno_stream_t stream) {
  if (!in || !out || !wpack || !g || !err || F < 1 || nb < 1 || rank < 0 || rank > 16) return FFNO_EINVAL;
  if (rank && (!U || !Vm)) return FFNO_EINVAL;
  if ((reinterpret_cast<uintptr_t>(wpack) % 16) || (reinterpret_cast<uintptr_t>(in) % 16)) return FFNO_EINVAL;
  if (rank > MIX_RANK_TC) return FFNO_EINVAL;
  if (sf < 1 || sb < 1 || s_im < 1 || sf % 4 || sb % 4 || s_im % 4) return FFNO_EINVAL;
  if (F > 0x7fffffffL || nb > 0x7fffffffL) return FFNO_EINVAL;
  if (C == 96)   // the production width: its own row-oriented kernel (pointwise_tc.cu); wpack = [M (2C x 2C)]
    return ffno::launch_mix_tc96(in, out, F, nb, sf, sb, s_im, wpack, g, U, Vm, rank, err, (cudaStream_t)stream);
  if (C != 16 && C != 32 && C != 64) return FFNO_EINVAL;
  // tensor map over (channel, then f / b / re-im sorted by stride); boxes of (min(C, 32), 1, 128, 2)
  struct Dim { int logical; uint64_t extent, stride; uint32_t box; } d[3] = {
      {0, (uint64_t)F, (uint64_t)sf * 4, 1u}, {1, (uint64_t)nb, (uint64_t)sb * 4, 128u}, {2, 2u, (uint64_t)s_im * 4, 2u}};
  for (int i = 1; i < 3; ++i)
    for (int k = i; k > 0 && d[k].stride < d[k - 1].stride; --k) {
      const Dim t = d[k];
      d[k] = d[k - 1];
      d[k - 1] = t;
    }
  const int CB = C < 32 ? C : 32;
  cuuint64_t gdim[4] = {(cuuint64_t)C, d[0].extent, d[1].extent, d[2].extent};
  cuuint64_t gstr[3] = {d[0].stride, d[1].stride, d[2].stride};
  cuuint32_t box[4] = {(cuuint32_t)CB, d[0].box, d[1].box, d[2].box};
  cuuint32_t estr[4] = {1, 1, 1, 1};
  CUtensorMap map;
  const PFN_cuTensorMapEncodeTiled_v12000 encode = tc::tensor_map_encoder();
  if (!encode) return FFNO_ELAUNCH;
  if (encode(&map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<float*>(in), gdim, gstr, box, estr,
                             CU_TENSOR_MAP_INTERLEAVE_NONE,
                             CB == 32 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return FFNO_EINVAL;
  MixGeom geo{};
  int run = 1;
  for (int k = 0; k < 3; ++k) {
    if (d[k].logical == 1) geo.mul_b = run;
    if (d[k].logical == 2) geo.mul_ri = run;
    run *= (int)d[k].box;
  }
  geo.o1 = d[0].logical;
  geo.o2 = d[1].logical;
  geo.o3 = d[2].logical;
  const long items = F * ((nb + 127) / 128);
  const long grid = items < sms() ? items : sms();
  const size_t K2 = 2 * (size_t)C;
  size_t smem = 1024 + 4 * 128 * K2 * 2 + (size_t)(C / CB) * 256 * CB * 4 + 2 * 16 * K2 * 2 + 4 * 128 * 16 * 2;
  if (smem < 120 * 1024) smem = 120 * 1024;   // one CTA per SM: each CTA holds all 512 tensor-memory columns
  cudaStream_t s = (cudaStream_t)stream;
  switch (C) {
#define L(CC)                                                                                                     \
  case CC: {                                                                                                      \
    if (!ffno::smem_cap_ok(k_mix_tc<CC>, smem)) \
      return FFNO_ELAUNCH;                                                                                        \
    k_mix_tc<CC><<<(unsigned)grid, XT, smem, s>>>(map, out, F, nb, sf, sb, s_im, static_cast<const uint8_t*>(wpack), \
                                                 g, U, Vm, rank, geo, err);                                       \
    break;                                                                                                        \
  }
    L(16) L(32) L(64)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_outer_tc(const float* A, long lda, int Ma, const float* B, long ldb, int Mb, long N, float* part, int nsplit,
                  double* out, int accumulate, int* err, ffno_stream_t stream) {
  return ffno_outer_tc_ld(A, lda, Ma, B, ldb, Mb, N, part, nsplit, out, Mb, accumulate, err, stream);
}

int ffno_outer_tc_ld(const float* A, long lda, int Ma, const float* B, long ldb, int Mb, long N, float* part,
                     int nsplit, double* out, long ldo, int accumulate, int* err, ffno_stream_t stream) {
  if (!A || !B || !part || !out || !err || Ma < 1 || Mb < 1 || N < 1 || nsplit < 1 || ldo < Mb) return FFNO_EINVAL;
  if (N % 4 || lda % 4 || ldb % 4 || lda < N || ldb < N || (reinterpret_cast<uintptr_t>(A) % 16) ||
      (reinterpret_cast<uintptr_t>(B) % 16))
    return FFNO_EINVAL;   // float4 loads that never straddle the end of a row
  const bool trans = Mb > Ma;   // the longer operand on the M side (tiles of 128), the shorter as the MMA's N
  const int MA = trans ? Mb : Ma, MB = trans ? Ma : Mb;
  const int TI = (MA + 127) / 128, NB = (MB + 15) / 16 * 16;
  if (NB > 256 || TI * NB > 512) return FFNO_EINVAL;
  const size_t limit = 227 * 1024 - 1024;
  int NS = 2;
  if (1024 + 2 * (size_t)outer_stage_bytes(TI, NB) > limit) NS = 1;
  const size_t smem = 1024 + NS * (size_t)outer_stage_bytes(TI, NB);
  if (smem > limit) return FFNO_EINVAL;
  if (!ffno::smem_cap_ok(k_outer_tc, smem))
    return FFNO_ELAUNCH;
  const long nchunks = (N + OKC - 1) / OKC;
  const long cps = (nchunks + nsplit - 1) / nsplit;
  const long n = (long)Ma * Mb;
  cudaStream_t s = (cudaStream_t)stream;
  if (trans)
    k_outer_tc<<<nsplit, OT, smem, s>>>(B, ldb, Mb, A, lda, Ma, N, TI, NB, NS, cps, part, n, 1, Mb, err);
  else
    k_outer_tc<<<nsplit, OT, smem, s>>>(A, lda, Ma, B, ldb, Mb, N, TI, NB, NS, cps, part, n, Mb, 1, err);
  k_outer_tc_reduce<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(part, nsplit, n, Mb, ldo, out, accumulate);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

}  // extern "C"
