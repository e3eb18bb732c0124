// FP32 kernels of the two spectral operators: the batched transform GEMM that carries every DFT of the path as a
// contraction with a precomputed real table (rfft/irfft along W, complex DFT along H, the Filon height transform and
// its inverse), and the per-frequency complex channel mixing.
#include "common.cuh"

using namespace ffno;

namespace {

constexpr int XM = 64, XN = 64, XK = 16;

// out[b][m][n] (+)= sum_k T[m][k] in[b][k][n]; CTA tile 64 (m) x 64 (n), 256 threads with a 4 x 4 micro-tile
// (rows ty + 16 i, columns tx + 16 j).
__global__ void __launch_bounds__(NT) k_xform(const float* __restrict__ T, const float* __restrict__ in,
                                              float* __restrict__ out, ffno_xform_desc d, long ntn, long ntm,
                                              int accumulate, long t_b) {
  __shared__ float ts[XM][XK + 1];
  __shared__ float is[XK][XN + 4];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  // m tiles vary fastest, so the CTAs that share one slab of `in` run together and read it from L2
  long bid = blockIdx.x;
  const long tm = bid % ntm;
  bid /= ntm;
  const long tn = bid % ntn;
  const long b = bid / ntn;
  const long b1 = b / d.nb2, b2 = b % d.nb2;
  const float* ib = in + b1 * d.in_b1 + b2 * d.in_b2;
  float* ob = out + b1 * d.out_b1 + b2 * d.out_b2;
  T += b * t_b;  // a table per batch element (t_b = 0: one shared table)
  const int m0 = (int)(tm * XM);
  const long n0 = tn * XN;
  float acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
  for (int k0 = 0; k0 < d.K; k0 += XK) {
    // T chunk [64][16]
    for (int e = threadIdx.x; e < XM * XK; e += NT) {
      const int r = e / XK, c = e % XK;
      const int m = m0 + r, k = k0 + c;
      ts[r][c] = (m < d.M && k < d.K) ? __ldg(T + (long)m * d.K + k) : 0.f;
    }
    // in chunk [16][64]
    for (int e = threadIdx.x; e < XK * XN; e += NT) {
      const int r = e / XN, c = e % XN;
      const int k = k0 + r;
      const long n = n0 + c;
      float v = 0.f;
      if (k < d.K && n < d.N) {
        const long off = (long)(k / d.in_split) * d.in_hi + (long)(k % d.in_split) * d.in_lo;
        v = __ldg(ib + off + n);
      }
      is[r][c] = v;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < XK; ++k) {
      float a[4], bb[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = ts[ty + 16 * i][k];
#pragma unroll
      for (int j = 0; j < 4; ++j) bb[j] = is[k][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], bb[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + ty + 16 * i;
    if (m >= d.M) continue;
    const long off = (long)(m / d.out_split) * d.out_hi + (long)(m % d.out_split) * d.out_lo;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const long n = n0 + tx + 16 * j;
      if (n < d.N) {
        if (accumulate)
          ob[off + n] += acc[i][j];
        else
          ob[off + n] = acc[i][j];
      }
    }
  }
}

// Per-frequency mixing, CTA = 64 rows b of one frequency f. xs holds [re | im] of each row (2C columns).
template <int C>
__global__ void __launch_bounds__(NT) k_mix(const float* __restrict__ in, float* __restrict__ out, long F, long nb,
                                            long sf, long sb, long s_im, const float* __restrict__ wbig,
                                            const float* __restrict__ g, const float* __restrict__ U,
                                            const float* __restrict__ Vm, int rank) {
  extern __shared__ float sm[];
  constexpr int LX = 2 * C + 1;
  float* xs = sm;                 // [BM][2C+1]
  float* us = xs + BM * LX;       // [C][rank]
  float* vs = us + C * 16;        // [rank][C]
  float* ts = vs + 16 * C;        // [BM][2*rank]
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const long nbt = (nb + BM - 1) / BM;
  const long f = blockIdx.x / nbt;
  const long b0 = (blockIdx.x % nbt) * BM;
  if (f >= F) return;
  const float* fin = in + f * sf;
  for (int e = threadIdx.x; e < BM * C; e += NT) {
    const int r = e / C, c = e % C;
    const long b = b0 + r;
    float re = 0.f, im = 0.f;
    if (b < nb) {
      re = __ldg(fin + b * sb + c);
      im = __ldg(fin + b * sb + s_im + c);
    }
    xs[r * LX + c] = re;
    xs[r * LX + C + c] = im;
  }
  if (rank) {
    for (int e = threadIdx.x; e < C * rank; e += NT) {
      us[e] = __ldg(U + f * C * rank + e);
      vs[e] = __ldg(Vm + f * C * rank + e);
    }
  }
  __syncthreads();
  if (rank) {
    // t[row][r] = sum_i V[r][i] xhat[row][i], complex (re in t[row][r], im in t[row][rank + r])
    for (int e = threadIdx.x; e < BM * 2 * rank; e += NT) {
      const int row = e / (2 * rank), q = e % (2 * rank);
      const int r = q % rank, part = q / rank;
      const float* xr = xs + row * LX + part * C;
      const float* vr = vs + r * C;
      float s = 0.f;
      for (int i = 0; i < C; ++i) s = fmaf(vr[i], xr[i], s);
      ts[row * 2 * rank + q] = s;
    }
  }
  float acc[4][2 * C / 16];
  tile_mm<2 * C, 2 * C>(xs, LX, wbig, acc);
  __syncthreads();
  const float gr = __ldg(g + 2 * f), gi = __ldg(g + 2 * f + 1);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int row = ty + 16 * i;
    const long b = b0 + row;
#pragma unroll
    for (int j = 0; j < C / 16; ++j) {
      const int o = tx + 16 * j;
      const float ar = acc[i][j], ai = acc[i][j + C / 16];
      float yr = ar * gr - ai * gi;
      float yi = ar * gi + ai * gr;
      if (rank) {
        float lr = 0.f, li = 0.f;
        for (int r = 0; r < rank; ++r) {
          const float u = us[o * rank + r];
          lr = fmaf(u, ts[row * 2 * rank + r], lr);
          li = fmaf(u, ts[row * 2 * rank + rank + r], li);
        }
        yr += lr;
        yi += li;
      }
      if (b < nb) {
        float* fo = out + f * sf + b * sb;
        fo[o] = yr;
        fo[s_im + o] = yi;
      }
    }
  }
}

}  // namespace

extern "C" {

int ffno_xform(const float* T, const float* in, float* out, const ffno_xform_desc* desc, int accumulate,
               ffno_stream_t stream) {
  if (!T || !in || !out || !desc) return FFNO_EINVAL;
  const ffno_xform_desc& d = *desc;
  if (d.nb < 1 || d.nb2 < 1 || d.K < 1 || d.M < 1 || d.N < 1 || d.in_split < 1 || d.out_split < 1)
    return FFNO_EINVAL;
  const long ntn = (d.N + XN - 1) / XN, ntm = (d.M + XM - 1) / XM;
  const long blocks = ntn * ntm * d.nb;
  if (blocks > 0x7fffffffL) return FFNO_EINVAL;
  k_xform<<<(unsigned)blocks, NT, 0, (cudaStream_t)stream>>>(T, in, out, d, ntn, ntm, accumulate, 0L);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_xform_pt(const float* T, long t_b, const float* in, float* out, const ffno_xform_desc* desc, int accumulate,
                  ffno_stream_t stream) {
  if (!T || !in || !out || !desc || t_b < 0) return FFNO_EINVAL;
  const ffno_xform_desc& d = *desc;
  if (d.nb < 1 || d.nb2 < 1 || d.K < 1 || d.M < 1 || d.N < 1 || d.in_split < 1 || d.out_split < 1)
    return FFNO_EINVAL;
  const long ntn = (d.N + XN - 1) / XN, ntm = (d.M + XM - 1) / XM;
  const long blocks = ntn * ntm * d.nb;
  if (blocks > 0x7fffffffL) return FFNO_EINVAL;
  k_xform<<<(unsigned)blocks, NT, 0, (cudaStream_t)stream>>>(T, in, out, d, ntn, ntm, accumulate, t_b);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

// out[col][i][j] (+)= sum_c A[i*rs + col*C + c] * B[j*rs + col*C + c], one CTA per column: the per-column
// height-table gradients. Output tiles of 64 rows of A x 64 rows of B: both row blocks staged in shared memory
// (coalesced row loads, rows padded to C + 1 floats), 4 x 4 outputs a thread summed over the C channels in FP32, then
// added to the FP64 output (which accumulates the blocks of a VJP).
constexpr int OT = 64;

__global__ void __launch_bounds__(256) k_col_outer(const float* __restrict__ A, int Ra, const float* __restrict__ B,
                                                   int Rb, long ncol, int C, long rs, double* __restrict__ out,
                                                   int accumulate) {
  extern __shared__ float osm[];
  const int LD = C + 1;
  float* as = osm;             // [OT][C + 1]
  float* bs = osm + OT * LD;   // [OT][C + 1]
  const long col = blockIdx.x;
  if (col >= ncol) return;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  for (int i0 = 0; i0 < Ra; i0 += OT) {
    for (int j0 = 0; j0 < Rb; j0 += OT) {
      __syncthreads();   // the previous tile's reads are done
      for (int e = threadIdx.x; e < OT * C; e += blockDim.x) {
        const int r = e / C, c = e % C;
        as[r * LD + c] = i0 + r < Ra ? __ldg(A + (long)(i0 + r) * rs + col * C + c) : 0.f;
        bs[r * LD + c] = j0 + r < Rb ? __ldg(B + (long)(j0 + r) * rs + col * C + c) : 0.f;
      }
      __syncthreads();
      float acc[4][4];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
      for (int c = 0; c < C; ++c) {
        float a[4], b[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = as[(ty + 16 * i) * LD + c];
#pragma unroll
        for (int j = 0; j < 4; ++j) b[j] = bs[(tx + 16 * j) * LD + c];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int ii = i0 + ty + 16 * i;
        if (ii >= Ra) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int jj = j0 + tx + 16 * j;
          if (jj >= Rb) continue;
          double* o = out + (col * Ra + ii) * (long)Rb + jj;
          *o = accumulate ? *o + (double)acc[i][j] : (double)acc[i][j];
        }
      }
    }
  }
}

int ffno_col_outer(const float* A, int Ra, const float* B, int Rb, long ncol, int C, long row_stride, double* out,
                   int accumulate, ffno_stream_t stream) {
  if (!A || !B || !out || Ra < 1 || Rb < 1 || ncol < 1 || C < 1 || C > 512 || ncol > 0x7fffffffL) return FFNO_EINVAL;
  const size_t smem = (size_t)2 * OT * (C + 1) * sizeof(float);
  if (smem > 48 * 1024 && !ffno::smem_cap_ok(k_col_outer, smem)) return FFNO_ELAUNCH;
  k_col_outer<<<(unsigned)ncol, 256, smem, (cudaStream_t)stream>>>(A, Ra, B, Rb, ncol, C, row_stride, out,
                                                                  accumulate);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_spectral_mix(const float* in, float* out, long F, long nb, long sf, long sb, long s_im, int C,
                      const float* wbig, const float* g, const float* U, const float* Vm, int rank,
                      ffno_stream_t stream) {
  if (!in || !out || !wbig || !g || F < 1 || nb < 1 || rank < 0 || rank > 16) return FFNO_EINVAL;
  if (rank && (!U || !Vm)) return FFNO_EINVAL;
  const long nbt = (nb + BM - 1) / BM;
  const long blocks = F * nbt;
  if (blocks > 0x7fffffffL) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  switch (C) {
#define L(CC)                                                                                              \
  case CC: {                                                                                               \
    const size_t smem = (BM * (2 * CC + 1) + 2 * CC * 16 + BM * 32) * sizeof(float);                        \
    if (smem > 48 * 1024 &&                                                                                \
        !ffno::smem_cap_ok(k_mix<CC>, smem)) \
      return FFNO_ELAUNCH;                                                                                 \
    k_mix<CC><<<(unsigned)blocks, NT, smem, s>>>(in, out, F, nb, sf, sb, s_im, wbig, g, U, Vm, rank);       \
    break;                                                                                                 \
  }
    L(16) L(32) L(64) L(96)
#undef L
    default:
      return FFNO_EINVAL;
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

}  // extern "C"
