// Tensor-core (tcgen05, split-BF16) versions of the spectral kernels: the batched transform GEMM that carries every
// DFT of the path (same ffno_xform_desc contract as spectral_f32.cu) and the per-frequency channel mixing.
//
// Transform GEMM: out[b][m][n] = sum_k T[m][k] in[b][k][n]. A CTA owns one (batch, 128-column n-tile) and all of M
// (at most two 128-row MMA tiles). K runs in chunks of 64 through a two-stage pipeline: the T chunk (split BF16,
// pre-packed per (m-tile, k-chunk) in the canonical K-major order) arrives by bulk copy while the threads convert the
// FP32 data chunk into a split MN-major tile (n contiguous, as it lies in HBM); the MMAs of chunk c run while chunk
// c + 1 is staged. Accumulators live in tensor memory (<= 2 x 128 columns).
#include "common.cuh"
#include "tc.cuh"

using namespace ffno;

namespace {

constexpr int XT = 256;    // threads
constexpr int XNT = 128;   // n columns per tile
constexpr int XKC = 64;    // k per chunk
constexpr int XMT = 2;     // max m tiles of 128

__host__ __device__ constexpr uint32_t a_chunk_bytes(int kc) { return 128u * kc * 2 * 2; }  // split hi + lo
__host__ __device__ constexpr uint32_t b_chunk_bytes(int kc) { return (uint32_t)XNT * kc * 2 * 2; }

struct XPipe {
  uint64_t* bar_a;    // [2] T chunk arrived
  uint64_t* bar_m;    // [2] MMAs of the chunk in this buffer finished
};

__device__ __forceinline__ bool bounded(bool ok, int* err, int code) {
  const bool all = __syncthreads_and(ok) != 0;
  if (!all && threadIdx.x == 0) atomicExch(err, code);
  return all;
}

__global__ void __launch_bounds__(XT) k_xform_tc(const uint8_t* __restrict__ tpack, const float* __restrict__ in,
                                                 float* __restrict__ out, ffno_xform_desc d, int Kp, long ntn,
                                                 int accumulate, int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  const int MT = (d.M + 127) / 128;
  const int nchunks = (Kp + XKC - 1) / XKC;
  const uint32_t stageA = XMT * a_chunk_bytes(XKC), stageB = b_chunk_bytes(XKC);
  uint8_t* sA[2] = {smem, smem + stageA + stageB};
  uint8_t* sB[2] = {smem + stageA, smem + 2 * stageA + stageB};
  __shared__ uint64_t bars[4];
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x;
  if (tid < 32) tc::tmem_alloc(&tslot, 256);
  if (tid == 0) {
    for (int i = 0; i < 4; ++i) tc::mbar_init(&bars[i], 1);
    tc::mbar_init_fence();
  }
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  const uint32_t tmem = tslot;
  XPipe P{bars, bars + 2};
  const long items = ntn * d.nb;
  long g = 0;  // global chunk counter: buffer g & 1, use (g >> 1) of that buffer
  bool ok = true;
  const int row = tid & 127, wg = tid >> 7;
  const uint32_t lb = (uint32_t)(32 * ((tid >> 5) & 3)) << 16;
  const uint32_t mt_bytes = (uint32_t)128 * Kp * 2 * 2;  // one m-tile of the pack (all chunks)
  for (long it = blockIdx.x; ok && it < items; it += gridDim.x) {
    const long b = it / ntn, tn = it % ntn;
    const long b1 = b / d.nb2, b2 = b % d.nb2;
    const float* ib = in + b1 * d.in_b1 + b2 * d.in_b2;
    float* ob = out + b1 * d.out_b1 + b2 * d.out_b2;
    const long n0 = tn * XNT;
    {  // L2 prefetch of the next item's rows (one row of up to 128 columns per thread)
      const long nx = it + gridDim.x;
      if (nx < items && tid < d.K) {
        const long bn = nx / ntn, tnn = nx % ntn;
        const long nn0 = tnn * XNT, cols = (d.N - nn0) < XNT ? (d.N - nn0) : XNT;
        const float* src = in + (bn / d.nb2) * d.in_b1 + (bn % d.nb2) * d.in_b2 +
                           (long)(tid / d.in_split) * d.in_hi + (long)(tid % d.in_split) * d.in_lo + nn0;
        tc::prefetch_l2(src, (uint32_t)(cols * 4));
      }
    }
    for (int c = 0; c < nchunks; ++c, ++g) {
      const int s = (int)(g & 1);
      const int k0 = c * XKC, kc = (Kp - k0) < XKC ? (Kp - k0) : XKC;
      // buffer s is free once the MMAs of chunk g - 2 are done
      if (g >= 2) {
        const bool w = tc::mbar_wait(&P.bar_m[s], (uint32_t)(((g - 2) >> 1) & 1));
        if (!(ok = bounded(w, err, 3))) break;
      }
      if (tid == 0) {
        const uint32_t bytes = a_chunk_bytes(kc);
        tc::mbar_arrive_expect_tx(&P.bar_a[s], bytes * MT);
        for (int mt = 0; mt < MT; ++mt)
          tc::bulk_g2s(sA[s] + mt * a_chunk_bytes(XKC), tpack + (size_t)mt * mt_bytes + (size_t)c * a_chunk_bytes(XKC),
                       bytes, &P.bar_a[s]);
      }
      // data chunk: rows k0 .. k0 + kc (zero past K), columns n0 .. n0 + 127 (zero past N) -> split MN-major tile;
      // four independent loads in flight per thread before any conversion
      {
        const uint32_t half = (uint32_t)XNT * kc * 2;
        const int ne = kc * XNT / 4;
        for (int e0 = tid; e0 < ne; e0 += 4 * XT) {
          float4 v[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int e = e0 + u * XT;
            const int kk = e / (XNT / 4), nn = 4 * (e % (XNT / 4));
            const int k = k0 + kk;
            const long n = n0 + nn;
            v[u] = make_float4(0.f, 0.f, 0.f, 0.f);
            if (e < ne && k < d.K && n < d.N)
              v[u] = __ldg(reinterpret_cast<const float4*>(ib + (long)(k / d.in_split) * d.in_hi +
                                                           (long)(k % d.in_split) * d.in_lo + n));
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const int e = e0 + u * XT;
            if (e >= ne) break;
            const int kk = e / (XNT / 4), nn = 4 * (e % (XNT / 4));
            uint32_t h0, l0, h1, l1;
            tc::split_pack(v[u].x, v[u].y, h0, l0);
            tc::split_pack(v[u].z, v[u].w, h1, l1);
            const uint32_t off = tc::mnmajor_offset(nn, kk, XNT);
            *reinterpret_cast<uint2*>(sB[s] + off) = make_uint2(h0, h1);
            *reinterpret_cast<uint2*>(sB[s] + half + off) = make_uint2(l0, l1);
          }
        }
      }
      tc::fence_async_smem();
      const bool wa = tc::mbar_wait(&P.bar_a[s], (uint32_t)((g >> 1) & 1));
      tc::tc_before_sync();
      if (!(ok = bounded(wa, err, 1))) break;
      tc::tc_after_sync();
      if (tid == 0) {
        const uint32_t bh = tc::smem_u32(sB[s]), bl = bh + (uint32_t)XNT * kc * 2;
        for (int mt = 0; mt < MT; ++mt) {
          const uint32_t ah = tc::smem_u32(sA[s] + mt * a_chunk_bytes(XKC)), al = ah + 128u * kc * 2;
          const uint32_t dcol = tmem + mt * XNT;
          tc::gemm_128xN_bmn(dcol, ah, bh, kc, XNT, c > 0);
          tc::gemm_128xN_bmn(dcol, ah, bl, kc, XNT, true);
          tc::gemm_128xN_bmn(dcol, al, bh, kc, XNT, true);
        }
        tc::mma_commit(&P.bar_m[s]);
      }
    }
    if (!ok) break;
    // all MMAs of this item: the last chunk's commit covers every earlier MMA of this thread
    {
      const long gl = g - 1;
      const bool w = tc::mbar_wait(&P.bar_m[gl & 1], (uint32_t)((gl >> 1) & 1));
      if (!(ok = bounded(w, err, 3))) break;
      tc::tc_after_sync();
    }
    for (int mt = 0; mt < MT; ++mt) {
      const int m = mt * 128 + row;
      const long off = (long)(m / d.out_split) * d.out_hi + (long)(m % d.out_split) * d.out_lo;
#pragma unroll
      for (int jj = 0; jj < XNT / 16; ++jj) {
        if ((jj & 1) != wg) continue;
        float v[16];
        tc::tmem_ld16(tmem + mt * XNT + lb + 16 * jj, v);
        const long n = n0 + 16 * jj;
        if (m < d.M) {
          float* dst = ob + off + n;
          if (n + 15 < d.N) {
#pragma unroll
            for (int i = 0; i < 16; i += 4) {
              float4 o = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
              if (accumulate) {
                const float4 p = *reinterpret_cast<float4*>(dst + i);
                o.x += p.x;
                o.y += p.y;
                o.z += p.z;
                o.w += p.w;
              }
              *reinterpret_cast<float4*>(dst + i) = o;
            }
          } else {
            for (int i = 0; i < 16 && n + i < d.N; ++i) dst[i] = accumulate ? dst[i] + v[i] : v[i];
          }
        }
      }
    }
    tc::tc_before_sync();
    __syncthreads();
    tc::tc_after_sync();
  }
  // leave no bulk copy or MMA in flight before freeing tensor memory
  if (!ok) {
    tc::mbar_wait(&P.bar_m[0], 0);
    tc::mbar_wait(&P.bar_m[1], 0);
  }
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  if (tid < 32) tc::tmem_free(tmem, 256);
}

// ---------------------------------------------------------------------------------------------------- mixing
// Per-frequency mixing on tensor cores: a CTA item = 128 rows b of one frequency f. A = [re | im] rows (split, K-major
// [128][2C]); B = wbig^T (split, [2C][2C]) resident; D [128][2C] in tensor memory; epilogue: g_f scaling and the
// rank-r term U_f (V_f xhat) from FP32 values.
template <int C>
__global__ void __launch_bounds__(XT) k_mix_tc(const float* __restrict__ in, float* __restrict__ out, long F, long nb,
                                               long sf, long sb, long s_im, const uint8_t* __restrict__ wpack,
                                               const float* __restrict__ g, const float* __restrict__ U,
                                               const float* __restrict__ Vm, int rank, int* __restrict__ err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  constexpr int K2 = 2 * C;
  constexpr uint32_t WB = (uint32_t)K2 * K2 * 2 * 2;
  uint8_t* sW = smem;
  uint8_t* sA = smem + WB;
  float* sT = reinterpret_cast<float*>(sA + 128u * K2 * 2 * 2);   // [128][33] low-rank projections (padded)
  float* sU = sT + 128 * 33;                                      // [C][rank]
  float* sV = sU + C * 16;                                        // [rank][C]
  __shared__ uint64_t bar;
  __shared__ uint32_t tslot;
  const int tid = threadIdx.x, row = tid & 127, wg = tid >> 7;
  if (tid < 32) tc::tmem_alloc(&tslot, K2 <= 32 ? 32 : (K2 <= 64 ? 64 : 128));
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::mbar_init_fence();
  }
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  const uint32_t tmem = tslot;
  const uint32_t lb = (uint32_t)(32 * ((tid >> 5) & 3)) << 16;
  uint32_t phase = 0;
  if (tid == 0) {
    tc::mbar_arrive_expect_tx(&bar, WB);
    for (uint32_t off = 0; off < WB; off += 65536u)
      tc::bulk_g2s(sW + off, wpack + off, (WB - off) < 65536u ? (WB - off) : 65536u, &bar);
  }
  bool ok = bounded(tc::mbar_wait(&bar, phase), err, 1);
  phase ^= 1u;
  const long nbt = (nb + 127) / 128;
  for (long it = blockIdx.x; ok && it < F * nbt; it += gridDim.x) {
    const long f = it / nbt, b0 = (it % nbt) * 128;
    const float* fin = in + f * sf;
    {  // L2 prefetch of the next item's rows (re and im halves)
      const long nx = it + gridDim.x;
      if (nx < F * nbt && tid < 128) {
        const long fn = nx / nbt, bn = (nx % nbt) * 128 + tid;
        if (bn < nb) {
          tc::prefetch_l2(in + fn * sf + bn * sb, C * 4);
          tc::prefetch_l2(in + fn * sf + bn * sb + s_im, C * 4);
        }
      }
    }
    // A tile (split, K-major [128][2C]): row b = [re | im]
    for (int e = tid; e < 128 * K2 / 4; e += XT) {
      const int h = e & 1, r8 = (e >> 1) & 7, q = e >> 4;
      const int kb = q % (K2 / 8), rb = q / (K2 / 8);
      const int r = rb * 8 + r8, k = kb * 8 + h * 4;
      const long b = b0 + r;
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (b < nb) v = __ldg(reinterpret_cast<const float4*>(fin + b * sb + (k < C ? k : s_im + k - C)));
      uint32_t h0, l0, h1, l1;
      tc::split_pack(v.x, v.y, h0, l0);
      tc::split_pack(v.z, v.w, h1, l1);
      *reinterpret_cast<uint2*>(sA + (size_t)e * 8) = make_uint2(h0, h1);
      *reinterpret_cast<uint2*>(sA + 128u * K2 * 2 + (size_t)e * 8) = make_uint2(l0, l1);
    }
    if (rank) {
      for (int e = tid; e < C * rank; e += XT) {
        sU[e] = __ldg(U + f * C * rank + e);
        sV[e] = __ldg(Vm + f * C * rank + e);
      }
    }
    tc::fence_async_smem();
    tc::tc_before_sync();
    __syncthreads();
    tc::tc_after_sync();
    if (tid == 0) {
      const uint32_t ah = tc::smem_u32(sA), al = ah + 128u * K2 * 2;
      const uint32_t bh = tc::smem_u32(sW), bl = bh + (uint32_t)K2 * K2 * 2;
      tc::gemm3_128xN(tmem, ah, al, bh, bl, K2, K2);
      tc::mma_commit(&bar);
    }
    // low-rank projections t[row][q] = sum_i V[r][i] xhat[row][i] (FP32, from the source rows) while the MMA runs
    if (rank) {
      for (int e = tid; e < 128 * 2 * rank; e += XT) {
        const int r = e / (2 * rank), q = e % (2 * rank);
        const int rr = q % rank, part = q / rank;
        const long b = b0 + r;
        float s = 0.f;
        if (b < nb) {
          const float* src = fin + b * sb + (part ? s_im : 0);
          for (int i = 0; i < C; i += 4) {
            const float4 x = __ldg(reinterpret_cast<const float4*>(src + i));
            s = fmaf(sV[rr * C + i], x.x, s);
            s = fmaf(sV[rr * C + i + 1], x.y, s);
            s = fmaf(sV[rr * C + i + 2], x.z, s);
            s = fmaf(sV[rr * C + i + 3], x.w, s);
          }
        }
        sT[r * 33 + q] = s;
      }
    }
    const bool w = tc::mbar_wait(&bar, phase);
    phase ^= 1u;
    tc::tc_before_sync();
    if (!(ok = bounded(w, err, 2))) break;
    tc::tc_after_sync();
    const float gr = __ldg(g + 2 * f), gi = __ldg(g + 2 * f + 1);
    const long b = b0 + row;
    // re chunk j pairs with im chunk j + C/16; warpgroup wg takes j of its parity
#pragma unroll
    for (int j = 0; j < C / 16; ++j) {
      if ((C / 16 > 1) && (j & 1) != wg) continue;
      if ((C / 16 == 1) && wg != 0) continue;
      float ar[16], ai[16];
      tc::tmem_ld16(tmem + lb + 16 * j, ar);
      tc::tmem_ld16(tmem + lb + C + 16 * j, ai);
      if (b < nb) {
        float* fo = out + f * sf + b * sb;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          const int o = 16 * j + i;
          float yr = ar[i] * gr - ai[i] * gi;
          float yi = ar[i] * gi + ai[i] * gr;
          if (rank) {
            float lr = 0.f, li = 0.f;
            for (int r = 0; r < rank; ++r) {
              const float u = sU[o * rank + r];
              lr = fmaf(u, sT[row * 33 + r], lr);
              li = fmaf(u, sT[row * 33 + rank + r], li);
            }
            yr += lr;
            yi += li;
          }
          fo[o] = yr;
          fo[s_im + o] = yi;
        }
      }
    }
    tc::tc_before_sync();
    __syncthreads();
    tc::tc_after_sync();
  }
  if (!ok) tc::mbar_wait(&bar, phase ^ 1u);
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  if (tid < 32) tc::tmem_free(tmem, K2 <= 32 ? 32 : (K2 <= 64 ? 64 : 128));
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
  if (d.N % 4 || d.in_lo % 4 || d.in_hi % 4 || d.in_b1 % 4 || d.in_b2 % 4) return FFNO_EINVAL;  // float4 loads
  if (d.out_lo % 4 || d.out_hi % 4 || d.out_b1 % 4 || d.out_b2 % 4) return FFNO_EINVAL;
  const int Kp = (d.K + 15) / 16 * 16;
  const long ntn = (d.N + XNT - 1) / XNT;
  const long items = ntn * d.nb;
  const size_t smem = 2 * ((size_t)XMT * a_chunk_bytes(XKC) + b_chunk_bytes(XKC));
  if (cudaFuncSetAttribute(k_xform_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return FFNO_ELAUNCH;
  const long grid = items < sms() ? items : sms();
  k_xform_tc<<<(unsigned)grid, XT, smem, (cudaStream_t)stream>>>(static_cast<const uint8_t*>(tpack), in, out, d, Kp,
                                                                 ntn, accumulate, err);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_spectral_mix_tc(const float* in, float* out, long F, long nb, long sf, long sb, long s_im, int C,
                         const void* wpack, const float* g, const float* U, const float* Vm, int rank, int* err,
                         ffno_stream_t stream) {
  if (!in || !out || !wpack || !g || !err || F < 1 || nb < 1 || rank < 0 || rank > 16) return FFNO_EINVAL;
  if (rank && (!U || !Vm)) return FFNO_EINVAL;
  if ((reinterpret_cast<uintptr_t>(wpack) % 16) || sf % 4 || sb % 4 || s_im % 4) return FFNO_EINVAL;
  const long items = F * ((nb + 127) / 128);
  const long grid = items < sms() ? items : sms();
  cudaStream_t s = (cudaStream_t)stream;
  switch (C) {
#define L(CC)                                                                                                     \
  case CC: {                                                                                                      \
    const size_t smem = (size_t)(2 * CC) * (2 * CC) * 4 + 128u * (2 * CC) * 4 + (128 * 33 + 2 * CC * 16) * 4;      \
    if (cudaFuncSetAttribute(k_mix_tc<CC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) \
      return FFNO_ELAUNCH;                                                                                        \
    k_mix_tc<CC><<<(unsigned)grid, XT, smem, s>>>(in, out, F, nb, sf, sb, s_im, static_cast<const uint8_t*>(wpack), \
                                                 g, U, Vm, rank, err);                                            \
    break;                                                                                                        \
  }
    L(16) L(32) L(64)
#undef L
    default:
      return FFNO_EINVAL;
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

}  // extern "C"
