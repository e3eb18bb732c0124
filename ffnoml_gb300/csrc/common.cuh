// Shared device helpers for the FFNO3D kernels: activations, the FP32 SIMT tile GEMM used by the pointwise (1x1x1
// convolution) chains, and the deterministic depth-weighted GroupNorm statistics.
//
// Activation layout: channels last, one row of C floats per voxel, voxel v = (d * H + h) * W + w of one cube.
// A "tile" is BM = 64 consecutive voxels processed by one CTA of NT = 256 threads; thread (ty, tx) = (tid / 16,
// tid % 16) owns rows ty + 16 i (i < 4) and columns tx + 16 j (j < N / 16) of every tile GEMM output.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ffnoml_gb300.h"

namespace ffno {

constexpr int BM = 64;
constexpr int NT = 256;
constexpr int GMAX = 8;  // DepthWeightedGroupNorm uses at most 8 groups (models/ffno_model.py:21-25)

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752440f)); }

// d gelu / dx = Phi(x) + x phi(x)
__device__ __forceinline__ float gelu_grad(float x) {
  const float cdf = 0.5f * (1.f + erff(x * 0.70710678118654752440f));
  const float pdf = 0.39894228040143267794f * expf(-0.5f * x * x);
  return cdf + x * pdf;
}

__device__ __forceinline__ float sigmoid(float x) { return 1.f / (1.f + expf(-x)); }

// Activations of the tensor-core (split-BF16) kernels: the normal CDF from the rational approximation of erfc in
// Abramowitz & Stegun, Handbook of Mathematical Functions, eq. 7.1.26 (|error of erf| <= 1.5e-7), whose exp(-x^2/2)
// factor is also the normal density in the GELU derivative: one exponential and one reciprocal (hardware
// approximations) per element instead of erff and expf. The absolute error of gelu and gelu' stays near 1e-6, well
// below the 2^-16 relative rounding of a split-BF16 operand; the FP32 kernels keep erff / expf.
struct Cdf {
  float cdf, pdf;   // Phi(x), phi(x)
};
__device__ __forceinline__ Cdf cdf_tc(float x) {
  const float u = fabsf(x) * 0.70710678118654752440f;
  const float t = __fdividef(1.f, fmaf(0.3275911f, u, 1.f));
  const float e = __expf(-0.5f * x * x);
  float p = fmaf(t, 1.061405429f, -1.453152027f);
  p = fmaf(t, p, 1.421413741f);
  p = fmaf(t, p, -0.284496736f);
  p = fmaf(t, p, 0.254829592f);
  const float h = 0.5f * (p * t) * e;   // (1 - erf(u)) / 2
  return Cdf{x < 0.f ? h : 1.f - h, 0.39894228040143267794f * e};
}
__device__ __forceinline__ float gelu_tc(float x) { return x * cdf_tc(x).cdf; }
__device__ __forceinline__ float gelu_grad_tc(float x) {
  const Cdf c = cdf_tc(x);
  return fmaf(x, c.pdf, c.cdf);
}
__device__ __forceinline__ float sigmoid_tc(float x) { return __fdividef(1.f, 1.f + __expf(-x)); }

// Math of the level-fraction head in the scalar type of the caller: FP64 (the reference's arithmetic) or FP32.
__device__ __forceinline__ double mexp10(double x) { return exp10(x); }
__device__ __forceinline__ float mexp10(float x) { return exp10f(x); }
__device__ __forceinline__ double mexp(double x) { return exp(x); }
__device__ __forceinline__ float mexp(float x) { return expf(x); }
__device__ __forceinline__ double mlog(double x) { return log(x); }
__device__ __forceinline__ float mlog(float x) { return logf(x); }
__device__ __forceinline__ double msqrt(double x) { return sqrt(x); }
__device__ __forceinline__ float msqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double mtanh(double x) { return tanh(x); }
__device__ __forceinline__ float mtanh(float x) { return tanhf(x); }

// MULTI3D constants, cgs (models/ffno_model.py:111-112)
constexpr double kEE = 1.602189e-12, kBK = 1.380662e-16;
constexpr double kLN10 = 2.302585092994045684;
constexpr double kINV_LN10 = 0.434294481903251827651;

// log(0.5 * (HH / sqrt(2 pi EM) / sqrt(BK))^3) with HH = 6.626176e-27, EM = 9.109534e-28, BK = 1.380662e-16 and
// pi = 3.14159265359: MULTI3D's Saha constant (models/ffno_model.py:112), evaluated once in 40-digit arithmetic (a
// CPU test recomputes it from the formula); as a literal it costs no FP64 log and square roots per voxel
constexpr double kLN_CCON = -36.113482555935598575;

// ------------------------------------------------------------------------------------------ level-fraction head
// One voxel of FFNO3D.head_output after proj2 (models/ffno_model.py:729-748): per species, logits = head channels + the
// LTE Boltzmann/Saha log-weights of (T, ne), log-softmax over the levels, plus the bounded total b tanh(u / b),
// log10 rho and the particle mass; normalised with mean_Y / std_Y. o: the voxel's head channels (species s: its L
// level logits, then its total channel). The LTE math and the log-softmax run in T: double is the reference's FP64
// (torch.log_softmax on float64 logits, :741); float is the split-BF16 path's FP32, where the sum of the max-shifted
// exponentials (each in (0, 1]) is compensated (below), so that the level shares of a voxel add up to 1 within a few
// FP32 roundings. The total term and the final sum of log10 n are FP64 in both.
struct HeadInputs {
  float lt, lne, lrho;   // log10 T, log10 ne (SI), log10 rho of the voxel (denormalised)
};

__device__ __forceinline__ HeadInputs head_inputs(const ffno_head_params& hp, const float* __restrict__ xin, long V,
                                                  long v) {
  const int tc = hp.temperature_channel, ec = hp.ne_channel, rc = hp.rho_channel;
  return HeadInputs{__ldg(xin + (long)tc * V + v), __ldg(xin + (long)ec * V + v), __ldg(xin + (long)rc * V + v)};
}

template <typename T>
struct Lte {
  T lt, lne, conl, dxi, ek_t;
  __device__ __forceinline__ Lte(const ffno_head_params& hp, const HeadInputs& in) {
    const int tc = hp.temperature_channel, ec = hp.ne_channel;
    const T LN10 = (T)kLN10;
    lt = (T)in.lt * (T)hp.std_x[tc] + (T)hp.mean_x[tc];
    lne = (T)in.lne * (T)hp.std_x[ec] + (T)hp.mean_x[ec];
    const T tk = mexp10(lt);
    const T ne = mexp10(lne - (T)6);  // cm^-3
    conl = (T)kLN_CCON + (lne - (T)6) * LN10 - (T)1.5 * lt * LN10;
    dxi = (T)(4.98e-4 * 5040.0) / tk * msqrt(ne * (T)kBK * tk);
    ek_t = (T)(kEE / kBK) / tk;
  }
  // the LTE log-weight of level g
  __device__ __forceinline__ T weight(const ffno_head_params& hp, int g) const {
    return (T)hp.log_g[g] - ek_t * ((T)hp.ev[g] - dxi * (T)hp.ndxi[g]) - (T)hp.dion[g] * conl;
  }
};

// sum_i exp(logit[i] - mx), i < L. FP64: a plain sum (the reference's float64 logsumexp). FP32: Neumaier's
// improved Kahan-Babuska summation (A. Neumaier, "Rundungsfehleranalyse einiger Verfahren zur Summation endlicher
// Summen", ZAMM 54 (1974) 39-51): the rounding error of every addition is carried in c and added once at the end,
// so the result is the exactly rounded sum of the rounded terms up to O(L u^2).
template <typename T>
__device__ __forceinline__ T shifted_exp_sum(const T* logit, int L, T mx) {
  T s = 0;
  for (int i = 0; i < L; ++i) s += mexp(logit[i] - mx);
  return s;
}
template <>
__device__ __forceinline__ float shifted_exp_sum<float>(const float* logit, int L, float mx) {
  float s = 0.f, c = 0.f;
  for (int i = 0; i < L; ++i) {
    const float t = expf(logit[i] - mx);
    const float u = s + t;
    c += fabsf(s) >= fabsf(t) ? (s - u) + t : (t - u) + s;
    s = u;
  }
  return s + c;
}

// Forward: out[g * V + v] = the normalised log10 population of level g.
template <typename T>
__device__ __forceinline__ void head_voxel_fwd(const ffno_head_params& hp, const float* o, const HeadInputs& in,
                                               float* __restrict__ out, long V, long v) {
  const Lte<T> e(hp, in);
  // the total term and the assembly of log10 n (log10 rho - log10 m + s ~ 20, minus mean_Y) stay in FP64 for both
  // T: in FP32 their rounding (~1e-6 dex at that magnitude, and a few ulp of b for tanh) would move every level of
  // the voxel against its total, past the 1e-6 bar on the level shares' sum; they are a handful of FP64 operations
  const double lrho = (double)in.lrho * (double)hp.std_x[hp.rho_channel] + (double)hp.mean_x[hp.rho_channel];
  int hc = 0, lvl = 0;
  for (int s = 0; s < hp.nspecies; ++s) {
    const int L = hp.levels[s];
    T logit[FFNO_MAX_LEVELS];
    T mx = (T)-1e30;
    for (int i = 0; i < L; ++i) {
      logit[i] = (T)o[hc + i] + e.weight(hp, lvl + i);
      mx = fmax(mx, logit[i]);
    }
    const T lse = mlog(shifted_exp_sum<T>(logit, L, mx));
    const double tb = (double)hp.total_bound;
    const double base = lrho - (double)hp.log10_particle_mass[s] + tb * tanh((double)o[hc + L] / tb);
    for (int i = 0; i < L; ++i) {
      const int g = lvl + i;
      const double l10 = base + ((double)(logit[i] - mx) - (double)lse) * kINV_LN10;
      // the large terms cancel in FP64; the difference (a few units) is normalised in FP32
      out[(long)g * V + v] = (float)(l10 - (double)hp.mean_y[g]) / hp.std_y[g];
    }
    hc += L + 1;
    lvl += L;
  }
}

// Backward: with ybar[g * V + v] the cotangent of the normalised output, overwrites o[0..nhp) with the gradient of the
// head channels (zero past the last species) and writes x_in_bar[k * V + v] for every input channel k.
template <typename T>
__device__ __forceinline__ void head_voxel_bwd(const ffno_head_params& hp, float* o, int nhp, const HeadInputs& in,
                                               const float* __restrict__ ybar, long V, long v,
                                               float* __restrict__ xinbar) {
  const Lte<T> e(hp, in);
  const T LN10 = (T)kLN10;
  T gsum = 0, ltb = 0, lneb = 0;
  int hc = 0, lvl = 0;
  for (int s = 0; s < hp.nspecies; ++s) {
    const int L = hp.levels[s];
    T logit[FFNO_MAX_LEVELS], gl[FFNO_MAX_LEVELS];
    T mx = (T)-1e30;
    for (int i = 0; i < L; ++i) {
      logit[i] = (T)o[hc + i] + e.weight(hp, lvl + i);
      mx = fmax(mx, logit[i]);
    }
    const T se = shifted_exp_sum<T>(logit, L, mx);
    T G = 0;
    for (int i = 0; i < L; ++i) {
      gl[i] = (T)__ldg(ybar + (long)(lvl + i) * V + v) / (T)hp.std_y[lvl + i];
      G += gl[i];
    }
    gsum += G;
    const T tb = (T)hp.total_bound;
    const T th = mtanh((T)o[hc + L] / tb);
    const float ubar = (float)(G * ((T)1 - th * th));
    for (int i = 0; i < L; ++i) {
      const int g = lvl + i;
      const T p = mexp(logit[i] - mx) / se;
      const T lb = (gl[i] - p * G) / LN10;
      o[hc + i] = (float)lb;
      ltb += lb * LN10 * (e.ek_t * ((T)hp.ev[g] - (T)1.5 * e.dxi * (T)hp.ndxi[g]) + (T)1.5 * (T)hp.dion[g]);
      lneb += lb * LN10 * ((T)0.5 * e.ek_t * e.dxi * (T)hp.ndxi[g] - (T)hp.dion[g]);
    }
    o[hc + L] = ubar;
    hc += L + 1;
    lvl += L;
  }
  for (int c = hc; c < nhp; ++c) o[c] = 0.f;
  const int tc = hp.temperature_channel, ec = hp.ne_channel, rc = hp.rho_channel;
  for (int k = 0; k < hp.in_channels; ++k) {
    T val = 0;
    if (k == tc) val += ltb * (T)hp.std_x[tc];
    if (k == ec) val += lneb * (T)hp.std_x[ec];
    if (k == rc) val += gsum * (T)hp.std_x[rc];
    xinbar[(long)k * V + v] = (float)val;
  }
}

// acc[i][j] = sum_k A[(ty + 16 i) * lda + k] * W[k * N + tx + 16 j] for i < RM rows per thread (a tile of 16 RM
// rows); A in shared memory, W (row-major K x N) in global memory (read through L1; every CTA reads the same small
// weight matrix).
template <int K, int N, int RM = 4>
__device__ __forceinline__ void tile_mm(const float* __restrict__ A, int lda, const float* __restrict__ W,
                                        float (&acc)[RM][N / 16]) {
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
#pragma unroll
  for (int i = 0; i < RM; ++i)
#pragma unroll
    for (int j = 0; j < N / 16; ++j) acc[i][j] = 0.f;
#pragma unroll 4
  for (int k = 0; k < K; ++k) {
    float a[RM], b[N / 16];
#pragma unroll
    for (int i = 0; i < RM; ++i) a[i] = A[(ty + 16 * i) * lda + k];
#pragma unroll
    for (int j = 0; j < N / 16; ++j) b[j] = __ldg(W + k * N + tx + 16 * j);
#pragma unroll
    for (int i = 0; i < RM; ++i)
#pragma unroll
      for (int j = 0; j < N / 16; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
  }
}

// Copy rows v0 .. v0 + rows - 1 (C floats each, row-major, contiguous) into shared memory with row stride lds; rows at
// or beyond V are zero.
template <int C>
__device__ __forceinline__ void load_rows(float* __restrict__ s, int lds, const float* __restrict__ g, long v0, long V,
                                          int rows = BM) {
  constexpr int Q = C / 4;  // float4 per row
  for (int e = threadIdx.x; e < rows * Q; e += NT) {
    const int r = e / Q, q = e % Q;
    float4 val = make_float4(0.f, 0.f, 0.f, 0.f);
    if (v0 + r < V) val = __ldg(reinterpret_cast<const float4*>(g + (v0 + r) * C) + q);
    float* d = s + r * lds + 4 * q;
    d[0] = val.x; d[1] = val.y; d[2] = val.z; d[3] = val.w;
  }
}

// Running weighted group statistics (total weight, mean, M2) of one CTA, merged tile by tile with Chan's parallel
// update so that no long single-precision sum and no E[x^2] - E[x]^2 cancellation occurs.
struct GroupAcc {
  double w, mean, m2;
};

__device__ __forceinline__ void chan_merge(GroupAcc& a, double wt, double mt, double m2t) {
  if (wt <= 0.0) return;
  const double wn = a.w + wt;
  const double delta = mt - a.mean;
  a.mean += delta * (wt / wn);
  a.m2 += m2t + delta * delta * (a.w * wt / wn);
  a.w = wn;
}

// Scratch (shared memory) for tile_group_stats: colsum [16][N], col [N], gmean [GMAX], gw (1)
template <int N>
struct StatsSmem {
  float part[16 * N];
  float col[N];
  float gmean[GMAX];
  float wsum;
};

// Accumulate the depth-weighted statistics of one tile's values val (rows ty + 16 i, columns tx + 16 j) into acc[g]
// (held by thread g < groups). wr[i] is the weight of row i, zero for rows past the cube. Column c belongs to group
// c / cpg. Deterministic: fixed summation order.
template <int N, int RM = 4>
__device__ __forceinline__ void tile_group_stats(const float (&val)[RM][N / 16], const float (&wr)[RM], int cpg,
                                                 int groups, StatsSmem<N>& sm, GroupAcc& acc) {
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  // tile weight: sum of the row weights (each row counted once: the threads with tx == 0 hold rows ty + 16 i)
  if (tx == 0) {
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < RM; ++i) s += wr[i];
    sm.part[ty] = s;
  }
  __syncthreads();
  if (tid == 0) {
    float s = 0.f;
    for (int t = 0; t < 16; ++t) s += sm.part[t];
    sm.wsum = s;
  }
  __syncthreads();
  // pass 1: weighted sums
#pragma unroll
  for (int j = 0; j < N / 16; ++j) {
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < RM; ++i) s = fmaf(wr[i], val[i][j], s);
    sm.part[ty * N + tx + 16 * j] = s;
  }
  __syncthreads();
  for (int c = tid; c < N; c += NT) {
    float s = 0.f;
    for (int t = 0; t < 16; ++t) s += sm.part[t * N + c];
    sm.col[c] = s;
  }
  __syncthreads();
  if (tid < groups) {
    float s = 0.f;
    for (int c = tid * cpg; c < (tid + 1) * cpg; ++c) s += sm.col[c];
    const float wt = sm.wsum * cpg;
    sm.gmean[tid] = wt > 0.f ? s / wt : 0.f;
  }
  __syncthreads();
  // pass 2: weighted squared deviations from the tile mean
#pragma unroll
  for (int j = 0; j < N / 16; ++j) {
    const float m = sm.gmean[(tx + 16 * j) / cpg];
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < RM; ++i) {
      const float d = val[i][j] - m;
      s = fmaf(wr[i] * d, d, s);
    }
    sm.part[ty * N + tx + 16 * j] = s;
  }
  __syncthreads();
  for (int c = tid; c < N; c += NT) {
    float s = 0.f;
    for (int t = 0; t < 16; ++t) s += sm.part[t * N + c];
    sm.col[c] = s;
  }
  __syncthreads();
  if (tid < groups) {
    float s = 0.f;
    for (int c = tid * cpg; c < (tid + 1) * cpg; ++c) s += sm.col[c];
    chan_merge(acc, (double)sm.wsum * cpg, (double)sm.gmean[tid], (double)s);
  }
  __syncthreads();
}

// Per-group sums of two per-element quantities a, b of one tile (rows ty + 16 i, columns tx + 16 j), added in a fixed
// order into the double accumulators s1, s2 held by thread g < groups. Used by the GroupNorm backward.
template <int N, int RM = 4>
__device__ __forceinline__ void tile_group_sums(const float (&a)[RM][N / 16], const float (&b)[RM][N / 16], int cpg,
                                                int groups, float* part /* [16][N] */, float* col /* [2][N] */,
                                                double& s1, double& s2) {
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
#pragma unroll
  for (int j = 0; j < N / 16; ++j) {
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < RM; ++i) s += a[i][j];
    part[ty * N + tx + 16 * j] = s;
  }
  __syncthreads();
  for (int c = tid; c < N; c += NT) {
    float s = 0.f;
    for (int t = 0; t < 16; ++t) s += part[t * N + c];
    col[c] = s;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < N / 16; ++j) {
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < RM; ++i) s += b[i][j];
    part[ty * N + tx + 16 * j] = s;
  }
  __syncthreads();
  for (int c = tid; c < N; c += NT) {
    float s = 0.f;
    for (int t = 0; t < 16; ++t) s += part[t * N + c];
    col[N + c] = s;
  }
  __syncthreads();
  if (tid < groups) {
    float x = 0.f, y = 0.f;
    for (int c = tid * cpg; c < (tid + 1) * cpg; ++c) {
      x += col[c];
      y += col[N + c];
    }
    s1 += (double)x;
    s2 += (double)y;
  }
  __syncthreads();
}

__device__ __forceinline__ void write_partial(double* partials, int groups, const GroupAcc& acc) {
  const int tid = threadIdx.x;
  if (tid < groups) {
    double* p = partials + ((long)blockIdx.x * groups + tid) * 3;
    p[0] = acc.w;
    p[1] = acc.mean;
    p[2] = acc.m2;
  }
}

// The dynamic shared memory a kernel may take is a process-wide attribute of that kernel. The service launches the
// same kernels from several host threads with different sizes (one request per thread), and a thread that lowered the
// attribute to its own size between another thread's setting and that thread's launch made the launch fail. So the
// attribute is set once per kernel and device, under a lock, to the most the kernel can have there (the opt-in maximum
// per block less the kernel's static shared memory), and each launch only checks its own size against that cap.
bool smem_cap_lookup(const void* kernel, size_t* cap);

template <typename K>
inline bool smem_cap_ok(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return true;
  size_t cap = 0;
  if (!smem_cap_lookup(reinterpret_cast<const void*>(kernel), &cap)) return false;
  return bytes <= cap;
}

}  // namespace ffno

#define FFNO_CHECK_LAUNCH()                                   \
  do {                                                        \
    cudaError_t e_ = cudaGetLastError();                      \
    if (e_ != cudaSuccess) return FFNO_ELAUNCH;               \
  } while (0)
