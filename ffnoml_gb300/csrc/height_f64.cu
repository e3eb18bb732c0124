// Per-column height tables and their gradient, FP64 on the device: the non-shared path of HeightSpectralConv
// (models/ffno_model.py:276-280, 306-308), where every column has its own height grid, so its Filon weights
// (height_fourier_weights, :37-64), inverse phases and taper (cutoff, :239-246) depend on that column's heights.
//
// Column c (heights z_raw[c][0..D), unshifted) at live modes k[0..M') with f[c][m] = factor_m taper_m / length:
//   z = z_raw - min(z_raw);  tzf[c][m][j] = q_re[j][m], tzf[c][M' + m][j] = q_im[j][m]   (Filon weights)
//   tzi[c][j][m] = cos(z_j k_m) f[c][m],  tzi[c][j][M' + m] = -sin(z_j k_m) f[c][m]
// with the Filon weights of the piecewise-linear interpolant: interval (z_j, z_j+1) adds its lower-end term a to node
// j and its upper-end term b to node j + 1. One CTA per column; a thread owns modes m = tid, tid + blockDim, ... and
// walks the column's intervals in order.
//
// The gradient runs the same walk backwards through the Filon weights and phases, adds the taper's dependence on
// the column's median spacing (index med[c] of the D - 1 spacings, as torch.median picks it; df[c][m] = d f / d dz)
// and the shift's (the minimum's gradient shared evenly by tied minima), and adds the result to z_bar. Reductions over
// modes run in a fixed order, so the gradient does not depend on timing.
#include <math.h>

#include "common.cuh"

namespace {

constexpr int HT = 128;    // threads per column
constexpr int HCH = 32;    // intervals per reduction chunk of the gradient

// Lower-end (a) and upper-end (b) Filon terms of interval (za, zb) at wavenumber k (tables.filon, one interval).
struct FilonTerms {
  double a_re, a_im, b_re, b_im;
};

// r = int_0^1 u e^{-i th u} du, l = int_0^1 (1 - u) e^{-i th u} du and their derivatives in th
struct RL {
  double r_re, r_im, l_re, l_im, dr_re, dr_im, dl_re, dl_im;
};

__device__ __forceinline__ RL filon_rl(double th, bool deriv) {
  RL o;
  if (fabs(th) < 1e-2) {
    const double t2 = th * th;
    o.r_re = 0.5 - t2 / 8;
    o.r_im = -th / 3 + t2 * th / 30;
    o.l_re = 0.5 - t2 / 24;
    o.l_im = -th / 6 + t2 * th / 120;
    if (deriv) {
      o.dr_re = -th / 4;
      o.dr_im = -1.0 / 3 + t2 / 10;
      o.dl_re = -th / 12;
      o.dl_im = -1.0 / 6 + t2 / 40;
    }
  } else {
    const double t = th, t2 = t * t;
    double s, c;
    sincos(t, &s, &c);
    o.r_re = (c + t * s - 1) / t2;
    o.r_im = (t * c - s) / t2;
    o.l_re = s / t - o.r_re;
    o.l_im = (c - 1) / t - o.r_im;
    if (deriv) {
      const double t3 = t2 * t;
      o.dr_re = (t2 * c - 2 * (c + t * s - 1)) / t3;
      o.dr_im = (-t2 * s - 2 * (t * c - s)) / t3;
      o.dl_re = (c * t - s) / t2 - o.dr_re;
      o.dl_im = (-s * t - (c - 1)) / t2 - o.dr_im;
    }
  }
  return o;
}

__device__ __forceinline__ FilonTerms filon_terms(double za, double zb, double k) {
  const double lo = fmin(za, zb), h = fabs(zb - za);
  const RL w = filon_rl(h * k, false);
  double sp, cp;
  sincos(lo * k, &sp, &cp);
  const double e_re = h * cp, e_im = -h * sp;
  const double lo_re = e_re * w.l_re - e_im * w.l_im, lo_im = e_re * w.l_im + e_im * w.l_re;
  const double hi_re = e_re * w.r_re - e_im * w.r_im, hi_im = e_re * w.r_im + e_im * w.r_re;
  if (za <= zb) return FilonTerms{lo_re, lo_im, hi_re, hi_im};
  return FilonTerms{hi_re, hi_im, lo_re, lo_im};
}

// d L / d za and d L / d zb of L = ga_re a_re + ga_im a_im + gb_re b_re + gb_im b_im for interval (za, zb).
__device__ __forceinline__ void filon_terms_vjp(double za, double zb, double k, double ga_re, double ga_im,
                                                double gb_re, double gb_im, double& dza, double& dzb) {
  dza = dzb = 0.0;
  if (za == zb) return;   // a zero-length interval: its terms are 0 and so is their gradient (|zb - za|' = 0 there)
  const bool up = za < zb;
  const double lo = up ? za : zb, h = up ? zb - za : za - zb;
  const RL w = filon_rl(h * k, true);
  double sp, cp;
  sincos(lo * k, &sp, &cp);
  const double e_re = h * cp, e_im = -h * sp;
  // the l terms go to the interval's lower end, the r terms to its upper end
  const double wl_re = up ? ga_re : gb_re, wl_im = up ? ga_im : gb_im;
  const double wr_re = up ? gb_re : ga_re, wr_im = up ? gb_im : ga_im;
  const double de_re = wl_re * w.l_re + wl_im * w.l_im + wr_re * w.r_re + wr_im * w.r_im;
  const double de_im = -wl_re * w.l_im + wl_im * w.l_re - wr_re * w.r_im + wr_im * w.r_re;
  const double dl_re = wl_re * e_re + wl_im * e_im, dl_im = -wl_re * e_im + wl_im * e_re;
  const double dr_re = wr_re * e_re + wr_im * e_im, dr_im = -wr_re * e_im + wr_im * e_re;
  const double dth = dl_re * w.dl_re + dl_im * w.dl_im + dr_re * w.dr_re + dr_im * w.dr_im;
  const double dh = de_re * cp - de_im * sp + dth * k;
  const double dlo = (de_re * (-h * sp) + de_im * (-h * cp)) * k;
  if (up) {   // h = zb - za, lo = za
    dza = -dh + dlo;
    dzb = dh;
  } else {    // h = za - zb, lo = zb
    dza = dh;
    dzb = -dh + dlo;
  }
}

// min over the column and its shifted heights in shared memory
__device__ __forceinline__ double shift_column(const double* __restrict__ zr, int D, double* zs, double* red) {
  double mn = INFINITY;
  for (int j = threadIdx.x; j < D; j += blockDim.x) mn = fmin(mn, zr[j]);
#pragma unroll
  for (int o = 16; o; o >>= 1) mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mn;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = red[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmin(m, red[w]);
    red[0] = m;
  }
  __syncthreads();
  const double zmin = red[0];
  for (int j = threadIdx.x; j < D; j += blockDim.x) zs[j] = zr[j] - zmin;
  __syncthreads();
  return zmin;
}

__global__ void __launch_bounds__(HT) k_percol_tables(const double* __restrict__ z_raw, int D, long ncol,
                                                      const double* __restrict__ k, int live,
                                                      const double* __restrict__ f, float* __restrict__ tzf,
                                                      float* __restrict__ tzi, float* __restrict__ tzf_t,
                                                      float* __restrict__ tzi_t) {
  extern __shared__ double zs[];   // [D]
  __shared__ double red[HT / 32];
  const long c = blockIdx.x;
  shift_column(z_raw + c * D, D, zs, red);
  const long M2 = 2L * live;
  float* F = tzf + c * M2 * D;     // [2M'][D]
  float* I = tzi + c * D * M2;     // [D][2M']
  float* Ft = tzf_t + c * D * M2;  // [D][2M']
  float* It = tzi_t + c * M2 * D;  // [2M'][D]
  for (int m = threadIdx.x; m < live; m += blockDim.x) {
    const double km = k[m], fm = f[c * live + m];
    double carry_re = 0.0, carry_im = 0.0;   // the previous interval's upper-end term, into node j
    for (int j = 0; j < D; ++j) {
      double q_re = carry_re, q_im = carry_im;
      if (j + 1 < D) {
        const FilonTerms t = filon_terms(zs[j], zs[j + 1], km);
        q_re = j ? q_re + t.a_re : t.a_re;
        q_im = j ? q_im + t.a_im : t.a_im;
        carry_re = t.b_re;
        carry_im = t.b_im;
      }
      double sn, cs;
      sincos(zs[j] * km, &sn, &cs);
      const float fr = (float)q_re, fi = (float)q_im, ic = (float)(cs * fm), is = (float)(-sn * fm);
      F[(long)m * D + j] = fr;
      F[(long)(live + m) * D + j] = fi;
      Ft[(long)j * M2 + m] = fr;
      Ft[(long)j * M2 + live + m] = fi;
      I[(long)j * M2 + m] = ic;
      I[(long)j * M2 + live + m] = is;
      It[(long)m * D + j] = ic;
      It[(long)(live + m) * D + j] = is;
    }
  }
}

// z_bar[j * ncol + c] += d/dz_raw[c][j] of sum(tzf_bar * tzf) + sum(tzi_bar * tzi) for every column c.
__global__ void __launch_bounds__(HT) k_percol_tables_vjp(const double* __restrict__ z_raw, int D, long ncol,
                                                          const double* __restrict__ k, int live,
                                                          const double* __restrict__ f,
                                                          const double* __restrict__ df, const int* __restrict__ med,
                                                          const double* __restrict__ tzf_bar,
                                                          const double* __restrict__ tzi_bar,
                                                          float* __restrict__ z_bar) {
  extern __shared__ double sh[];
  double* zs = sh;                     // [D] shifted heights
  double* gz = zs + D;                 // [D] gradient w.r.t. the shifted heights
  double* dldf = gz + D;               // [live] d L / d f_m
  double* bufa = dldf + live;          // [HT][HCH + 1] per-thread sums into node j0 + jj (lower ends, tzi)
  double* bufb = bufa + HT * (HCH + 1);   // [HT][HCH + 1] per-thread sums into node j0 + jj + 1 (upper ends)
  __shared__ double red[HT / 32];
  const long c = blockIdx.x;
  const int tid = threadIdx.x;
  const double* zr = z_raw + c * D;
  const double zmin = shift_column(zr, D, zs, red);
  for (int j = tid; j < D; j += HT) gz[j] = 0.0;
  for (int m = tid; m < live; m += HT) dldf[m] = 0.0;
  const long M2 = 2L * live;
  const double* Fb = tzf_bar + c * M2 * D;   // [2M'][D]
  const double* Ib = tzi_bar + c * D * M2;   // [D][2M']
  __syncthreads();
  double* sa = bufa + tid * (HCH + 1);   // this thread's row: its modes' sums, in mode order
  double* sb = bufb + tid * (HCH + 1);
  for (int j0 = 0; j0 < D; j0 += HCH) {
    const int nj = D - j0 < HCH ? D - j0 : HCH;
    for (int jj = 0; jj < HCH; ++jj) sa[jj] = sb[jj] = 0.0;
    for (int m = tid; m < live; m += HT) {
      const double km = k[m], fm = f[c * live + m];
      double dlf = 0.0;
#pragma unroll 1
      for (int jj = 0; jj < nj; ++jj) {
        const int j = j0 + jj;
        // node j's inverse-table entries
        double sn, cs;
        sincos(zs[j] * km, &sn, &cs);
        const double gc = Ib[(long)j * M2 + m], gs = Ib[(long)j * M2 + live + m];
        sa[jj] += fm * km * (-gc * sn - gs * cs);
        dlf += gc * cs - gs * sn;
        // interval (j, j + 1): its lower-end terms sit in node j's table entries, its upper-end terms in node j + 1's
        if (j + 1 < D) {
          double dza, dzb;
          filon_terms_vjp(zs[j], zs[j + 1], km, Fb[(long)m * D + j], Fb[(long)(live + m) * D + j],
                          Fb[(long)m * D + j + 1], Fb[(long)(live + m) * D + j + 1], dza, dzb);
          sa[jj] += dza;
          sb[jj] += dzb;
        }
      }
      dldf[m] += dlf;
    }
    // fixed-order sums over the threads: node j0 + jj gets the lower-end sums, then node j0 + jj + 1 the upper-end
    __syncthreads();
    if (tid < nj) {
      double s = 0.0;
      for (int t = 0; t < HT; ++t) s += bufa[t * (HCH + 1) + tid];
      gz[j0 + tid] += s;
    }
    __syncthreads();
    if (tid < nj && j0 + tid + 1 < D) {
      double s = 0.0;
      for (int t = 0; t < HT; ++t) s += bufb[t * (HCH + 1) + tid];
      gz[j0 + tid + 1] += s;
    }
    __syncthreads();
  }
  if (tid == 0) {
    // the taper through the median spacing |z_p+1 - z_p|
    double g = 0.0;
    for (int m = 0; m < live; ++m) g += dldf[m] * df[c * live + m];
    const int p = med[c];
    const double d = zs[p + 1] - zs[p];
    const double sg = d > 0 ? 1.0 : (d < 0 ? -1.0 : 0.0);
    gz[p + 1] += g * sg;
    gz[p] -= g * sg;
    // the shift by the minimum: its gradient (minus the sum) shared evenly by the tied minima
    double tot = 0.0;
    int nt = 0;
    for (int j = 0; j < D; ++j) {
      tot += gz[j];
      nt += zr[j] == zmin;
    }
    red[0] = tot / nt;
  }
  __syncthreads();
  const double share = red[0];
  for (int j = tid; j < D; j += HT) {
    const double g = gz[j] - (zr[j] == zmin ? share : 0.0);
    z_bar[(long)j * ncol + c] += (float)g;
  }
}

size_t vjp_smem(int D, int live) { return (size_t)(2 * D + live + 2 * HT * (HCH + 1)) * sizeof(double); }

// ---------------------------------------------------------------------------------------- one column, many CTAs
// The same gradient for one column (a shared height grid), spread over the (mode, node) pairs: k_column_terms writes
// every pair's terms (node j's lower-end sum, node j + 1's upper-end term, d L / d f_m) to scratch; k_column_finish
// sums them in a fixed order (per node over the modes, per mode over the nodes) and finishes as k_percol_tables_vjp
// does. scratch: [3][M'][D] doubles.
constexpr int CT1 = 256;

__device__ __forceinline__ double column_min(const double* __restrict__ zr, int D, double* red) {
  double mn = INFINITY;
  for (int j = threadIdx.x; j < D; j += blockDim.x) mn = fmin(mn, zr[j]);
#pragma unroll
  for (int o = 16; o; o >>= 1) mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mn;
  __syncthreads();
  double m = red[0];
  for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmin(m, red[w]);
  return m;
}

__global__ void __launch_bounds__(CT1) k_column_terms(const double* __restrict__ zr, int D,
                                                      const double* __restrict__ k, int live,
                                                      const double* __restrict__ f,
                                                      const double* __restrict__ tzf_bar,
                                                      const double* __restrict__ tzi_bar, double* __restrict__ terms) {
  __shared__ double red[CT1 / 32];
  const double zmin = column_min(zr, D, red);
  const long e = (long)blockIdx.x * CT1 + threadIdx.x;
  if (e >= (long)live * D) return;
  const int m = (int)(e / D), j = (int)(e % D);
  const long M2 = 2L * live;
  const double km = k[m], fm = f[m];
  const double zj = zr[j] - zmin;
  double sn, cs;
  sincos(zj * km, &sn, &cs);
  const double gc = tzi_bar[(long)j * M2 + m], gs = tzi_bar[(long)j * M2 + live + m];
  double lo = fm * km * (-gc * sn - gs * cs), up = 0.0;
  if (j + 1 < D) {
    double dza, dzb;
    filon_terms_vjp(zj, zr[j + 1] - zmin, km, tzf_bar[(long)m * D + j], tzf_bar[(long)(live + m) * D + j],
                    tzf_bar[(long)m * D + j + 1], tzf_bar[(long)(live + m) * D + j + 1], dza, dzb);
    lo += dza;
    up = dzb;
  }
  const long n = (long)live * D;
  terms[e] = lo;
  terms[n + e] = up;
  terms[2 * n + e] = gc * cs - gs * sn;
}

__global__ void __launch_bounds__(CT1) k_column_finish(const double* __restrict__ zr, int D, int live,
                                                       const double* __restrict__ df, int med,
                                                       const double* __restrict__ terms, float* __restrict__ z_bar,
                                                       long z_stride) {
  extern __shared__ double gz[];   // [D]
  __shared__ double red[CT1 / 32];
  __shared__ double share, gtap;
  const double zmin = column_min(zr, D, red);
  const long n = (long)live * D;
  for (int j = threadIdx.x; j < D; j += CT1) {
    double g = 0.0;
    for (int m = 0; m < live; ++m) g += terms[(long)m * D + j];
    if (j > 0)
      for (int m = 0; m < live; ++m) g += terms[n + (long)m * D + j - 1];
    gz[j] = g;
  }
  // d L / d f_m per mode, weighted by d f_m / d dz, summed over the modes in order by one warp
  if (threadIdx.x < 32) {
    double t = 0.0;
    for (int m = threadIdx.x; m < live; m += 32) {
      double dl = 0.0;
      for (int j = 0; j < D; ++j) dl += terms[2 * n + (long)m * D + j];
      t += dl * df[m];
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) gtap = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // the taper through the median spacing |z_p+1 - z_p|
    const double d = zr[med + 1] - zr[med];
    const double sg = d > 0 ? 1.0 : (d < 0 ? -1.0 : 0.0);
    gz[med + 1] += gtap * sg;
    gz[med] -= gtap * sg;
    // the shift by the minimum: its gradient (minus the sum) shared evenly by the tied minima
    double tot = 0.0;
    int nt = 0;
    for (int j = 0; j < D; ++j) {
      tot += gz[j];
      nt += zr[j] == zmin;
    }
    share = tot / nt;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < D; j += CT1) {
    const double g = gz[j] - (zr[j] == zmin ? share : 0.0);
    z_bar[(long)j * z_stride] += (float)g;
  }
}

}  // namespace

extern "C" {

int ffno_percol_tables(const double* z_raw, int D, long ncol, const double* k, int live, const double* f, float* tzf,
                       float* tzi, float* tzf_t, float* tzi_t, ffno_stream_t stream) {
  if (!z_raw || !k || !f || !tzf || !tzi || !tzf_t || !tzi_t || D < 2 || ncol < 1 || live < 1) return FFNO_EINVAL;
  if (D > FFNO_PERCOL_MAX_D || live > FFNO_PERCOL_MAX_LIVE || ncol > 2147483647L) return FFNO_EINVAL;
  const size_t smem = (size_t)D * sizeof(double);
  if (!ffno::smem_cap_ok(k_percol_tables, smem)) return FFNO_ELAUNCH;
  k_percol_tables<<<(unsigned)ncol, HT, smem, (cudaStream_t)stream>>>(z_raw, D, ncol, k, live, f, tzf, tzi, tzf_t,
                                                                     tzi_t);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_column_tables_vjp(const double* z_raw, int D, const double* k, int live, const double* f, const double* df,
                           int med, const double* tzf_bar, const double* tzi_bar, double* scratch, float* z_bar,
                           long z_stride, ffno_stream_t stream) {
  if (!z_raw || !k || !f || !df || !tzf_bar || !tzi_bar || !scratch || !z_bar || D < 2 || live < 1 || z_stride < 1)
    return FFNO_EINVAL;
  if (D > FFNO_PERCOL_MAX_D || live > FFNO_PERCOL_MAX_LIVE || med < 0 || med > D - 2) return FFNO_EINVAL;
  const long n = (long)live * D;
  cudaStream_t s = (cudaStream_t)stream;
  k_column_terms<<<(unsigned)((n + CT1 - 1) / CT1), CT1, 0, s>>>(z_raw, D, k, live, f, tzf_bar, tzi_bar, scratch);
  k_column_finish<<<1, CT1, (size_t)D * sizeof(double), s>>>(z_raw, D, live, df, med, scratch, z_bar, z_stride);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_percol_tables_vjp(const double* z_raw, int D, long ncol, const double* k, int live, const double* f,
                           const double* df, const int* med, const double* tzf_bar, const double* tzi_bar,
                           float* z_bar, ffno_stream_t stream) {
  if (!z_raw || !k || !f || !df || !med || !tzf_bar || !tzi_bar || !z_bar || D < 2 || ncol < 1 || live < 1)
    return FFNO_EINVAL;
  if (D > FFNO_PERCOL_MAX_D || live > FFNO_PERCOL_MAX_LIVE || ncol > 2147483647L) return FFNO_EINVAL;
  const size_t smem = vjp_smem(D, live);
  if (!ffno::smem_cap_ok(k_percol_tables_vjp, smem)) return FFNO_ELAUNCH;
  k_percol_tables_vjp<<<(unsigned)ncol, HT, smem, (cudaStream_t)stream>>>(z_raw, D, ncol, k, live, f, df, med,
                                                                         tzf_bar, tzi_bar, z_bar);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

}  // extern "C"
