// FP32 kernels of the FFNO3D forward-mode derivative (JVP): the tangent of every stage of FFNO3D.forward
// (models/ffno_model.py:524-553, 730-832) along an input tangent, evaluated next to the primal stage it linearises
// (what jvp_local gets from dual tensors carried through the network, ffno_fsdp_runtime.py:350-372). The linear stages
// (the lift convolution, the DFT contractions, the spectral mixing) reuse the forward kernels on the tangent; these are
// the nonlinear ones. The heights are fixed (the depth weights, the height tables and the z_proj term carry no
// tangent).
#include <math.h>

#include "common.cuh"

using namespace ffno;

namespace {

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

int grid_rows(long V, int rows, int per_sm) {
  const long t = (V + rows - 1) / rows;
  const long g = (long)sms() * per_sm;
  return (int)(t < g ? (t > 0 ? t : 1) : g);
}

template <typename K>
bool smem_attr(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return true;
  return ffno::smem_cap_ok(kernel, bytes);
}

bool width_ok(int C) { return C == 16 || C == 32 || C == 64 || C == 96; }

// ------------------------------------------------------------------------------------------------ GroupNorm JVP
// y = gamma (x - mu) r + beta over a group with depth weights w (T = sum of w over the group's elements):
// y' = gamma r (x' - S1 / T - xhat S2 / T), S1 = sum w x', S2 = sum w xhat x' (xhat = (x - mu) r).
// Statistics: per-CTA partial sums [nparts][groups][2] in a fixed order (the layout of ffno_gn_bwd_final).
template <int C>
__global__ void __launch_bounds__(256) k_gn_jvp_stats(const float* __restrict__ pre, const float* __restrict__ ud,
                                                      const double* __restrict__ gst, const float* __restrict__ dw,
                                                      long V, double* __restrict__ partials, int cpg, int groups) {
  constexpr int LPV = C / 4;                       // lanes per voxel (float4 each)
  constexpr int VPW = LPV <= 32 ? 32 / LPV : 1;    // voxels per warp step
  __shared__ float mean[GMAX], rstd[GMAX];
  __shared__ double red[8][GMAX][2];
  if (threadIdx.x < groups) {
    mean[threadIdx.x] = (float)gst[3 * threadIdx.x];
    rstd[threadIdx.x] = (float)gst[3 * threadIdx.x + 1];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sub = lane / LPV, q = lane % LPV;
  const bool active = sub < VPW;
  const int c = 4 * q;
  int grp[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) grp[j] = (c + j) / cpg;
  double d1[4] = {0, 0, 0, 0}, d2[4] = {0, 0, 0, 0};
  float f1[4] = {0, 0, 0, 0}, f2[4] = {0, 0, 0, 0};
  int n = 0;
  const long step = (long)gridDim.x * 8 * VPW;
  for (long v = ((long)blockIdx.x * 8 + warp) * VPW + sub; active && v < V; v += step) {
    const float w = __ldg(dw + v);
    const float4 pu = __ldg(reinterpret_cast<const float4*>(ud + v * C + c));
    const float4 pp = __ldg(reinterpret_cast<const float4*>(pre + v * C + c));
    const float uu[4] = {pu.x, pu.y, pu.z, pu.w}, xx[4] = {pp.x, pp.y, pp.z, pp.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int g = grp[j];
      const float xh = (xx[j] - mean[g]) * rstd[g];
      f1[j] = fmaf(w, uu[j], f1[j]);
      f2[j] = fmaf(w * xh, uu[j], f2[j]);
    }
    if (++n == 16) {
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        d1[j] += f1[j];
        d2[j] += f2[j];
        f1[j] = f2[j] = 0.f;
      }
      n = 0;
    }
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    d1[j] += f1[j];
    d2[j] += f2[j];
  }
  for (int g = 0; g < groups; ++g) {
    double a = 0.0, b = 0.0;
#pragma unroll
    for (int j = 0; j < 4; ++j)
      if (active && grp[j] == g) {
        a += d1[j];
        b += d2[j];
      }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      a += __shfl_xor_sync(0xffffffffu, a, o);
      b += __shfl_xor_sync(0xffffffffu, b, o);
    }
    if (lane == 0) {
      red[warp][g][0] = a;
      red[warp][g][1] = b;
    }
  }
  __syncthreads();
  if (threadIdx.x < groups) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < 8; ++w) {
      a += red[w][threadIdx.x][0];
      b += red[w][threadIdx.x][1];
    }
    partials[((long)blockIdx.x * groups + threadIdx.x) * 2] = a;
    partials[((long)blockIdx.x * groups + threadIdx.x) * 2 + 1] = b;
  }
}

// out = base + res * y' (base may be null; act 1: y' times gelu'(y), a GELU after the GroupNorm)
template <int C>
__global__ void k_gn_jvp_apply(const float* __restrict__ pre, const float* __restrict__ ud,
                               const float* __restrict__ gamma, const float* __restrict__ beta,
                               const double* __restrict__ gst, const double* __restrict__ sums, int act,
                               const float* __restrict__ base, float res, long V, float* __restrict__ out, int cpg,
                               int groups) {
  __shared__ float mean[GMAX], rstd[GMAX], s1[GMAX], s2[GMAX];
  if (threadIdx.x < groups) {
    const int g = threadIdx.x;
    const double it = 1.0 / gst[3 * g + 2];
    mean[g] = (float)gst[3 * g];
    rstd[g] = (float)gst[3 * g + 1];
    s1[g] = (float)(sums[2 * g] * it);
    s2[g] = (float)(sums[2 * g + 1] * it);
  }
  __syncthreads();
  const long n4 = V * (C / 4);
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n4; e += (long)gridDim.x * blockDim.x) {
    const long v = e / (C / 4);
    const int c = (int)(e % (C / 4)) * 4;
    const float4 pp = __ldg(reinterpret_cast<const float4*>(pre + v * C + c));
    const float4 pu = __ldg(reinterpret_cast<const float4*>(ud + v * C + c));
    const float xx[4] = {pp.x, pp.y, pp.z, pp.w}, uu[4] = {pu.x, pu.y, pu.z, pu.w};
    float o[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int g = (c + j) / cpg;
      const float gm = __ldg(gamma + c + j);
      const float xh = (xx[j] - mean[g]) * rstd[g];
      float yd = gm * rstd[g] * (uu[j] - s1[g] - xh * s2[g]);
      if (act) yd *= gelu_grad(fmaf(gm, xh, __ldg(beta + c + j)));
      o[j] = res * yd;
    }
    if (base) {
      const float4 b4 = __ldg(reinterpret_cast<const float4*>(base + v * C + c));
      o[0] += b4.x;
      o[1] += b4.y;
      o[2] += b4.z;
      o[3] += b4.w;
    }
    *reinterpret_cast<float4*>(out + v * C + c) = make_float4(o[0], o[1], o[2], o[3]);
  }
}

// ------------------------------------------------------------------------------------------------ chains
// Tiles of BM voxels, thread (ty, tx) owns rows ty + 16 i and columns tx + 16 j of every tile GEMM (tile_mm).

// Input gate: out = x sigmoid(g), g = gelu(x G1) G2 (+ zp z, constant in x): out' = x' s + x s (1 - s) g',
// g' = (gelu'(x G1) x' G1) G2.
template <int C>
__global__ void __launch_bounds__(NT) k_gate_jvp(const float* __restrict__ x, const float* __restrict__ xd, long V,
                                                 const float* __restrict__ w1, const float* __restrict__ w2,
                                                 float* __restrict__ outd) {
  extern __shared__ float sm[];
  constexpr int L = C + 1;
  float* xs = sm;
  float* xds = xs + BM * L;
  float* hs = xds + BM * L;
  float* hds = hs + BM * L;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const long nt = (V + BM - 1) / BM;
  for (long t = blockIdx.x; t < nt; t += gridDim.x) {
    const long v0 = t * BM;
    __syncthreads();
    load_rows<C>(xs, L, x, v0, V);
    load_rows<C>(xds, L, xd, v0, V);
    __syncthreads();
    {
      float a[4][C / 16], b[4][C / 16];
      tile_mm<C, C>(xs, L, w1, a);
      tile_mm<C, C>(xds, L, w1, b);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < C / 16; ++j) {
          const int r = ty + 16 * i, c = tx + 16 * j;
          hs[r * L + c] = gelu(a[i][j]);
          hds[r * L + c] = gelu_grad(a[i][j]) * b[i][j];
        }
    }
    __syncthreads();
    float a[4][C / 16], b[4][C / 16];
    tile_mm<C, C>(hs, L, w2, a);
    tile_mm<C, C>(hds, L, w2, b);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = ty + 16 * i;
      const long v = v0 + r;
      if (v >= V) continue;
#pragma unroll
      for (int j = 0; j < C / 16; ++j) {
        const int c = tx + 16 * j;
        const float s = sigmoid(a[i][j]);
        outd[v * C + c] = xds[r * L + c] * s + xs[r * L + c] * s * (1.f - s) * b[i][j];
      }
    }
  }
}

// Two-layer MLP C -> 2C -> C: pre' = (gelu'(a W1) a' W1) W2.
template <int C>
__global__ void __launch_bounds__(NT) k_mlp2_jvp(const float* __restrict__ a, const float* __restrict__ ad, long V,
                                                 const float* __restrict__ w1, const float* __restrict__ w2,
                                                 float* __restrict__ outd) {
  extern __shared__ float sm[];
  constexpr int LA = C + 1, LH = 2 * C + 1;
  float* as = sm;
  float* ads = as + BM * LA;
  float* hds = ads + BM * LA;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const long nt = (V + BM - 1) / BM;
  for (long t = blockIdx.x; t < nt; t += gridDim.x) {
    const long v0 = t * BM;
    __syncthreads();
    load_rows<C>(as, LA, a, v0, V);
    load_rows<C>(ads, LA, ad, v0, V);
    __syncthreads();
    {
      float h[4][2 * C / 16], hd[4][2 * C / 16];
      tile_mm<C, 2 * C>(as, LA, w1, h);
      tile_mm<C, 2 * C>(ads, LA, w1, hd);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2 * C / 16; ++j) hds[(ty + 16 * i) * LH + tx + 16 * j] = gelu_grad(h[i][j]) * hd[i][j];
    }
    __syncthreads();
    float o[4][C / 16];
    tile_mm<2 * C, C>(hds, LH, w2, o);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const long v = v0 + ty + 16 * i;
      if (v >= V) continue;
#pragma unroll
      for (int j = 0; j < C / 16; ++j) outd[v * C + tx + 16 * j] = o[i][j];
    }
  }
}

// Gate + fuse (_fuse_branches): A = [x, s, v] with s = gelu(GN(spec_pre)), v likewise (sd, vd: their tangents);
// gates = sigmoid(gelu(A Wg1) Wg2 + b); B = [s gs, v gv]; fused = gelu(B Wf1) Wf2 + (B_s + B_v) / 2 -> fused'.
template <int C, int RM>
__global__ void __launch_bounds__(NT) k_fuse_jvp(const float* __restrict__ x, const float* __restrict__ xd,
                                                 const float* __restrict__ sp, const float* __restrict__ sc,
                                                 const float* __restrict__ vp, const float* __restrict__ vc,
                                                 const float* __restrict__ sd, const float* __restrict__ vd, long V,
                                                 const float* __restrict__ wg1, const float* __restrict__ wg2,
                                                 const float* __restrict__ bg2, const float* __restrict__ wf1,
                                                 const float* __restrict__ wf2, float* __restrict__ outd) {
  extern __shared__ float sm[];
  constexpr int TB = 16 * RM;                     // voxels per tile
  constexpr int LA = 3 * C + 1, LH = C + 1, LB = 2 * C + 1;
  float* A = sm;
  float* Ad = A + TB * LA;
  float* H = Ad + TB * LA;
  float* Hd = H + TB * LH;
  float* Bm = Hd + TB * LH;
  float* Bd = Bm + TB * LB;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const long nt = (V + TB - 1) / TB;
  for (long t = blockIdx.x; t < nt; t += gridDim.x) {
    const long v0 = t * TB;
    __syncthreads();
    for (int e = threadIdx.x; e < TB * C; e += NT) {
      const int r = e / C, c = e % C;
      const long v = v0 + r;
      float a = 0.f, s = 0.f, q = 0.f, ad = 0.f, s_d = 0.f, q_d = 0.f;
      if (v < V) {
        a = __ldg(x + v * C + c);
        s = gelu((__ldg(sp + v * C + c) - __ldg(sc + c)) * __ldg(sc + C + c) + __ldg(sc + 2 * C + c));
        q = gelu((__ldg(vp + v * C + c) - __ldg(vc + c)) * __ldg(vc + C + c) + __ldg(vc + 2 * C + c));
        ad = __ldg(xd + v * C + c);
        s_d = __ldg(sd + v * C + c);
        q_d = __ldg(vd + v * C + c);
      }
      A[r * LA + c] = a;
      A[r * LA + C + c] = s;
      A[r * LA + 2 * C + c] = q;
      Ad[r * LA + c] = ad;
      Ad[r * LA + C + c] = s_d;
      Ad[r * LA + 2 * C + c] = q_d;
    }
    __syncthreads();
    {
      float h[RM][C / 16], hd[RM][C / 16];
      tile_mm<3 * C, C, RM>(A, LA, wg1, h);
      tile_mm<3 * C, C, RM>(Ad, LA, wg1, hd);
#pragma unroll
      for (int i = 0; i < RM; ++i)
#pragma unroll
        for (int j = 0; j < C / 16; ++j) {
          const int r = ty + 16 * i, c = tx + 16 * j;
          H[r * LH + c] = gelu(h[i][j]);
          Hd[r * LH + c] = gelu_grad(h[i][j]) * hd[i][j];
        }
    }
    __syncthreads();
    {
      float q[RM][2 * C / 16], qd[RM][2 * C / 16];
      tile_mm<C, 2 * C, RM>(H, LH, wg2, q);
      tile_mm<C, 2 * C, RM>(Hd, LH, wg2, qd);
#pragma unroll
      for (int i = 0; i < RM; ++i)
#pragma unroll
        for (int j = 0; j < 2 * C / 16; ++j) {
          const int r = ty + 16 * i, n = tx + 16 * j;
          const float g = sigmoid(q[i][j] + __ldg(bg2 + n));
          const float gd = g * (1.f - g) * qd[i][j];
          const float s = A[r * LA + C + n], s_d = Ad[r * LA + C + n];
          Bm[r * LB + n] = s * g;
          Bd[r * LB + n] = s_d * g + s * gd;
        }
    }
    __syncthreads();
    {
      float h[RM][2 * C / 16], hd[RM][2 * C / 16];
      tile_mm<2 * C, 2 * C, RM>(Bm, LB, wf1, h);
      tile_mm<2 * C, 2 * C, RM>(Bd, LB, wf1, hd);
#pragma unroll
      for (int i = 0; i < RM; ++i)
#pragma unroll
        for (int j = 0; j < 2 * C / 16; ++j) A[(ty + 16 * i) * LA + tx + 16 * j] = gelu_grad(h[i][j]) * hd[i][j];
    }
    __syncthreads();
    float o[RM][C / 16];
    tile_mm<2 * C, C, RM>(A, LA, wf2, o);
#pragma unroll
    for (int i = 0; i < RM; ++i) {
      const int r = ty + 16 * i;
      const long v = v0 + r;
      if (v >= V) continue;
#pragma unroll
      for (int j = 0; j < C / 16; ++j) {
        const int c = tx + 16 * j;
        outd[v * C + c] = o[i][j] + 0.5f * (Bd[r * LB + c] + Bd[r * LB + C + c]);
      }
    }
  }
}

// ------------------------------------------------------------------------------------------------ head
// Tangent of head_output (models/ffno_model.py:730-749) along the last block's tangent x' and the input tangent
// x_in': h' = (gelu'(x P1) x' P1) P2; per species, d log10 n_i = d log10 rho + sech^2(h_tot / b) h_tot'
// + (l_i' - sum_j p_j l_j') / ln 10 with l = h + lte (p = softmax(l)); lte' follows MULTI3D's LTE weights through
// log10 T and log10 ne (models/ffno_model.py:131-141).
template <int C, int NHP>
__global__ void __launch_bounds__(NT) k_head_jvp(const float* __restrict__ x, const float* __restrict__ xd,
                                                 const float* __restrict__ xin, const float* __restrict__ xind, long V,
                                                 const float* __restrict__ p1, const float* __restrict__ p2,
                                                 const float* __restrict__ b2, ffno_head_params hp,
                                                 float* __restrict__ outd) {
  extern __shared__ float sm[];
  constexpr int LA = C + 1, LH = 2 * C + 1, LO = NHP + 1;
  float* as = sm;
  float* ads = as + BM * LA;
  float* hs = ads + BM * LA;
  float* hds = hs + BM * LH;
  float* os = hds + BM * LH;
  float* ods = os + BM * LO;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const double lnc = kLN_CCON;
  const long nt = (V + BM - 1) / BM;
  for (long t = blockIdx.x; t < nt; t += gridDim.x) {
    const long v0 = t * BM;
    __syncthreads();
    load_rows<C>(as, LA, x, v0, V);
    load_rows<C>(ads, LA, xd, v0, V);
    __syncthreads();
    {
      float h[4][2 * C / 16], hd[4][2 * C / 16];
      tile_mm<C, 2 * C>(as, LA, p1, h);
      tile_mm<C, 2 * C>(ads, LA, p1, hd);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2 * C / 16; ++j) {
          const int r = ty + 16 * i, c = tx + 16 * j;
          hs[r * LH + c] = gelu(h[i][j]);
          hds[r * LH + c] = gelu_grad(h[i][j]) * hd[i][j];
        }
    }
    __syncthreads();
    {
      float o[4][NHP / 16], od[4][NHP / 16];
      tile_mm<2 * C, NHP>(hs, LH, p2, o);
      tile_mm<2 * C, NHP>(hds, LH, p2, od);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < NHP / 16; ++j) {
          const int r = ty + 16 * i, n = tx + 16 * j;
          os[r * LO + n] = o[i][j] + __ldg(b2 + n);
          ods[r * LO + n] = od[i][j];
        }
    }
    __syncthreads();
    if (threadIdx.x < BM) {
      const int r = threadIdx.x;
      const long v = v0 + r;
      if (v < V) {
        const float* o = os + r * LO;
        const float* od = ods + r * LO;
        const int tc = hp.temperature_channel, ec = hp.ne_channel, rc = hp.rho_channel;
        const double lt = (double)__ldg(xin + (long)tc * V + v) * (double)hp.std_x[tc] + (double)hp.mean_x[tc];
        const double lne = (double)__ldg(xin + (long)ec * V + v) * (double)hp.std_x[ec] + (double)hp.mean_x[ec];
        const double dlt = (double)__ldg(xind + (long)tc * V + v) * (double)hp.std_x[tc];
        const double dlne = (double)__ldg(xind + (long)ec * V + v) * (double)hp.std_x[ec];
        const double dlrho = (double)__ldg(xind + (long)rc * V + v) * (double)hp.std_x[rc];
        const double tk = exp10(lt);
        const double ne = exp10(lne - 6.0);  // cm^-3
        const double conl = lnc + (lne - 6.0) * kLN10 - 1.5 * lt * kLN10;
        const double dxi = 4.98e-4 * 5040.0 / tk * sqrt(ne * kBK * tk);
        const double ek_t = (kEE / kBK) / tk;
        int hc = 0, lvl = 0;
        for (int s = 0; s < hp.nspecies; ++s) {
          const int L = hp.levels[s];
          double logit[FFNO_MAX_LEVELS], dl[FFNO_MAX_LEVELS];
          double mx = -1e300;
          for (int i = 0; i < L; ++i) {
            const int g = lvl + i;
            const double lte = hp.log_g[g] - ek_t * (hp.ev[g] - dxi * hp.ndxi[g]) - hp.dion[g] * conl;
            // d lte / d log10 T and d lte / d log10 ne (through t, the Debye term dxi ~ sqrt(ne / t) and conl)
            const double dT = kLN10 * (ek_t * (hp.ev[g] - 1.5 * dxi * hp.ndxi[g]) + 1.5 * hp.dion[g]);
            const double dN = kLN10 * (0.5 * ek_t * hp.ndxi[g] * dxi - hp.dion[g]);
            logit[i] = (double)o[hc + i] + lte;
            dl[i] = (double)od[hc + i] + dT * dlt + dN * dlne;
            mx = fmax(mx, logit[i]);
          }
          double se = 0.0;
          for (int i = 0; i < L; ++i) se += exp(logit[i] - mx);
          double md = 0.0;
          for (int i = 0; i < L; ++i) md += exp(logit[i] - mx) / se * dl[i];
          const double tb = (double)hp.total_bound;
          const double th = tanh((double)o[hc + L] / tb);
          const double dtot = (1.0 - th * th) * (double)od[hc + L];
          for (int i = 0; i < L; ++i) {
            const int g = lvl + i;
            const double d = dlrho + dtot + (dl[i] - md) / kLN10;
            outd[(long)g * V + v] = (float)(d / (double)hp.std_y[g]);
          }
          hc += L + 1;
          lvl += L;
        }
      }
    }
  }
}

// ------------------------------------------------------------------------------------------------ service units
// Input tangent in the service's SI units (T [K], v [m/s], log10 ne, log10 rho) -> tangent of the normalised model
// inputs (log10 T, v / 1e3, ..., then (x - mean) / std; ffno_fsdp_runtime.py:48-58, 274-280). flags |= 1 on NaN/Inf.
__global__ void k_si_input_tangent(const float* __restrict__ feat, const float* __restrict__ td, long V,
                                   const float* __restrict__ std_x, float* __restrict__ xd, int* __restrict__ flags) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < 6 * V; e += (long)gridDim.x * blockDim.x) {
    const int c = (int)(e / V);
    const float t = td[e];
    if (!isfinite(t)) atomicOr(flags, 1);
    float m;
    if (c == 0)
      m = t / (feat[e] * (float)kLN10);
    else if (c < 4)
      m = t / 1.0e3f;
    else
      m = t;
    xd[e] = m / std_x[c];
  }
}

// Model-output tangent (normalised log10 n, [L][V]) -> population tangent (nz, nx, ny, L) in m^-3: n = 10^clamp(y std
// + mean, +-37), n' = n ln 10 std y' inside the clamp, 0 outside (linear_populations, ffno_fsdp_runtime.py:76-78).
// flags |= 8 on a non-finite tangent.
__global__ void k_si_population_tangent(const float* __restrict__ y, const float* __restrict__ yd, long V, int L,
                                        const float* __restrict__ mean_y, const float* __restrict__ std_y,
                                        float* __restrict__ out, int* __restrict__ flags) {
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < (long)L * V; e += (long)gridDim.x * blockDim.x) {
    const long v = e / L;
    const int l = (int)(e % L);
    const float pl = y[(long)l * V + v] * std_y[l] + mean_y[l];
    float d = 0.f;
    if (pl >= -37.f && pl <= 37.f) d = exp10f(pl) * (float)kLN10 * std_y[l] * yd[(long)l * V + v];
    if (!isfinite(d)) atomicOr(flags, 8);
    out[e] = d;
  }
}

}  // namespace

// ====================================================================================================== C ABI
extern "C" {

int ffno_gn_jvp_stats(const float* pre, const float* pre_dot, const double* gstats, const float* dw, long V, int C,
                      int groups, double* partials, int nparts, ffno_stream_t stream) {
  if (!pre || !pre_dot || !gstats || !dw || !partials || !width_ok(C) || V < 1 || groups < 1 || groups > GMAX ||
      C % groups || nparts < 1)
    return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  const int cpg = C / groups;
  switch (C) {
#define L(CC) case CC: k_gn_jvp_stats<CC><<<nparts, 256, 0, s>>>(pre, pre_dot, gstats, dw, V, partials, cpg, groups); break;
    L(16) L(32) L(64) L(96)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_gn_jvp_apply(const float* pre, const float* pre_dot, const float* gamma, const float* beta,
                      const double* gstats, const double* sums, int act, const float* base, float res, long V, int C,
                      int groups, float* out, ffno_stream_t stream) {
  if (!pre || !pre_dot || !gamma || !beta || !gstats || !sums || !out || !width_ok(C) || V < 1 || groups < 1 ||
      groups > GMAX || C % groups || act < 0 || act > 1)
    return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  const int cpg = C / groups;
  const long n4 = V * (C / 4);
  const int blocks = (int)((n4 + 255) / 256 < 8L * sms() ? (n4 + 255) / 256 : 8L * sms());
  switch (C) {
#define L(CC) case CC: k_gn_jvp_apply<CC><<<blocks, 256, 0, s>>>(pre, pre_dot, gamma, beta, gstats, sums, act, base, res, V, out, cpg, groups); break;
    L(16) L(32) L(64) L(96)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_gate_jvp(const float* x, const float* x_dot, long V, int C, const float* w1, const float* w2, float* out_dot,
                  ffno_stream_t stream) {
  if (!x || !x_dot || !w1 || !w2 || !out_dot || !width_ok(C) || V < 1) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  switch (C) {
#define L(CC)                                                                                 \
  case CC: {                                                                                  \
    const size_t smem = 4 * BM * (CC + 1) * sizeof(float);                                    \
    if (!smem_attr(k_gate_jvp<CC>, smem)) return FFNO_ELAUNCH;                                \
    k_gate_jvp<CC><<<grid_rows(V, BM, 2), NT, smem, s>>>(x, x_dot, V, w1, w2, out_dot);        \
    break;                                                                                    \
  }
    L(16) L(32) L(64) L(96)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_mlp2_jvp(const float* a, const float* a_dot, long V, int C, const float* w1, const float* w2, float* out_dot,
                  ffno_stream_t stream) {
  if (!a || !a_dot || !w1 || !w2 || !out_dot || !width_ok(C) || V < 1) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  switch (C) {
#define L(CC)                                                                                   \
  case CC: {                                                                                    \
    const size_t smem = (2 * BM * (CC + 1) + BM * (2 * CC + 1)) * sizeof(float);                \
    if (!smem_attr(k_mlp2_jvp<CC>, smem)) return FFNO_ELAUNCH;                                  \
    k_mlp2_jvp<CC><<<grid_rows(V, BM, 2), NT, smem, s>>>(a, a_dot, V, w1, w2, out_dot);          \
    break;                                                                                      \
  }
    L(16) L(32) L(64) L(96)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_fuse_jvp(const float* x, const float* x_dot, const float* spec_pre, const float* spec_coefs,
                  const float* vert_pre, const float* vert_coefs, const float* spec_dot, const float* vert_dot, long V,
                  int C, const float* wg1, const float* wg2, const float* bg2, const float* wf1, const float* wf2,
                  float* fused_dot, ffno_stream_t stream) {
  if (!x || !x_dot || !spec_pre || !spec_coefs || !vert_pre || !vert_coefs || !spec_dot || !vert_dot || !wg1 ||
      !wg2 || !bg2 || !wf1 || !wf2 || !fused_dot || !width_ok(C) || V < 1)
    return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  switch (C) {
#define L(CC, RM)                                                                                             \
  case CC: {                                                                                                  \
    const size_t smem = (size_t)16 * RM * (12 * CC + 6) * sizeof(float);                                      \
    if (!smem_attr(k_fuse_jvp<CC, RM>, smem)) return FFNO_ELAUNCH;                                           \
    k_fuse_jvp<CC, RM><<<grid_rows(V, 16 * RM, 1), NT, smem, s>>>(x, x_dot, spec_pre, spec_coefs, vert_pre,    \
                                                                  vert_coefs, spec_dot, vert_dot, V, wg1, wg2, \
                                                                  bg2, wf1, wf2, fused_dot);                   \
    break;                                                                                                    \
  }
    L(16, 4) L(32, 4) L(64, 4) L(96, 2)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_head_jvp(const float* x, const float* x_dot, const float* x_in, const float* x_in_dot, long V, int C,
                  const float* p1, const float* p2, const float* b2, int nhp, const ffno_head_params* params,
                  float* out_dot, ffno_stream_t stream) {
  if (!x || !x_dot || !x_in || !x_in_dot || !p1 || !p2 || !b2 || !params || !out_dot || !width_ok(C) || V < 1)
    return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  switch (C * 1000 + nhp) {
#define L(CC, NN)                                                                                                  \
  case CC * 1000 + NN: {                                                                                           \
    const size_t smem = (2 * BM * (CC + 1) + 2 * BM * (2 * CC + 1) + 2 * BM * (NN + 1)) * sizeof(float);           \
    if (!smem_attr(k_head_jvp<CC, NN>, smem)) return FFNO_ELAUNCH;                                                \
    k_head_jvp<CC, NN><<<grid_rows(V, BM, 2), NT, smem, s>>>(x, x_dot, x_in, x_in_dot, V, p1, p2, b2, *params, out_dot); \
    break;                                                                                                         \
  }
    L(16, 16) L(16, 32) L(32, 16) L(32, 32) L(64, 16) L(64, 32) L(96, 16) L(96, 32)
#undef L
    default:
      return FFNO_EINVAL;
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_si_input_tangent(const float* features, const float* tangent, long V, const float* std_x, float* x_dot,
                          int* flags, ffno_stream_t stream) {
  if (!features || !tangent || !std_x || !x_dot || !flags || V < 1) return FFNO_EINVAL;
  const long n = 6 * V;
  const int blocks = (int)((n + 255) / 256 < 8L * sms() ? (n + 255) / 256 : 8L * sms());
  k_si_input_tangent<<<blocks, 256, 0, (cudaStream_t)stream>>>(features, tangent, V, std_x, x_dot, flags);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_si_population_tangent(const float* y, const float* y_dot, long V, int L, const float* mean_y,
                               const float* std_y, float* out, int* flags, ffno_stream_t stream) {
  if (!y || !y_dot || !mean_y || !std_y || !out || !flags || V < 1 || L < 1) return FFNO_EINVAL;
  const long n = (long)L * V;
  const int blocks = (int)((n + 255) / 256 < 8L * sms() ? (n + 255) / 256 : 8L * sms());
  k_si_population_tangent<<<blocks, 256, 0, (cudaStream_t)stream>>>(y, y_dot, V, L, mean_y, std_y, out, flags);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

}  // extern "C"
