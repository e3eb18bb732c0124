// FP32 kernels of the FFNO3D input VJP (the hand-written replacement of torch.autograd through FFNO3D.forward,
// models/ffno_model.py:536-553, 730-798). Every chain kernel recomputes its tile's forward activations from the
// block's saved inputs instead of storing them.
#include <math.h>

#include <mutex>

#include "common.cuh"
#include "tc.cuh"

using namespace ffno;

namespace {

__host__ __device__ __forceinline__ long ntiles(long V, int rows) { return (V + rows - 1) / rows; }

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

int grid_of(long V, int rows, int per_sm) {
  const long t = ntiles(V, rows);
  const long g = (long)sms() * per_sm;
  return (int)(t < g ? (t > 0 ? t : 1) : g);
}

template <typename K>
bool smem_attr(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return true;
  return ffno::smem_cap_ok(kernel, bytes);
}

bool width_ok(int C) { return C == 16 || C == 32 || C == 64 || C == 96; }

__device__ __forceinline__ float upstream(int mode, float u, float r, float y) {
  // gradient w.r.t. the GroupNorm output y given the upstream u: r u (mode 0), r u gelu'(y) (mode 1: GELU after GN,
  // erf-based), or r u gelu'(y) with the tensor-core kernels' activation (mode 2: the split-BF16 path, whose forward
  // applies that GELU after these GroupNorms)
  if (mode == 2) return r * u * gelu_grad_tc(y);
  return mode ? r * u * gelu_grad(y) : r * u;
}

// ------------------------------------------------------------------------------------------------ GN backward
// Lane layout of the two GroupNorm-backward kernels: each voxel's C channels are held VW at a time by LPV consecutive
// lanes (C = 96: VW = 4 and 24 lanes of a warp); a warp covers VPW voxels per step. The application uses VW = 8 (one
// 32-byte request a lane) for C <= 64; the statistics keep VW = 4, whose per-slot double accumulators would
// otherwise take more registers than two CTAs of an SM have.
template <int C, int W>
struct GnLanes {
  static constexpr int VW = C <= 64 ? W : 4;
  static constexpr int LPV = C / VW;
  static constexpr int VPW = LPV <= 32 ? 32 / LPV : 1;
};

template <int VW>
__device__ __forceinline__ void ldv(const float* p, float (&o)[VW]) {
  if constexpr (VW == 8) {
    ffno::tc::ld8(p, o);
  } else {
    const float4 a = __ldg(reinterpret_cast<const float4*>(p));
    o[0] = a.x, o[1] = a.y, o[2] = a.z, o[3] = a.w;
  }
}
template <int VW>
__device__ __forceinline__ void stv(float* p, const float (&v)[VW]) {
  if constexpr (VW == 8) {
    ffno::tc::st8(p, v);
  } else {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  }
}

// Per-group constants of one GroupNorm, as floats in shared memory: mean, rstd, 1/T, S1, S2, var*rstd^2.
struct GnConst {
  float mean[GMAX], rstd[GMAX], invT[GMAX], s1[GMAX], s2[GMAX], vr2[GMAX];
};

__device__ __forceinline__ void load_gn_const(GnConst& k, const double* gst, const double* sums, int groups,
                                              float eps) {
  if (threadIdx.x < groups) {
    const int g = threadIdx.x;
    const double rs = gst[3 * g + 1];
    k.mean[g] = (float)gst[3 * g];
    k.rstd[g] = (float)rs;
    k.invT[g] = (float)(1.0 / gst[3 * g + 2]);
    k.s1[g] = sums ? (float)sums[2 * g] : 0.f;
    k.s2[g] = sums ? (float)sums[2 * g + 1] : 0.f;
    k.vr2[g] = (float)(1.0 - (double)eps * rs * rs);
  }
  __syncthreads();
}

// Per group: S1 = sum ghat, S2 = sum ghat xhat, ghat = dL/dy * gamma, xhat = (pre - mean) rstd, as per-CTA partials.
template <int C>
__global__ void __launch_bounds__(256) k_gn_bwd_stats(int mode, const float* __restrict__ u, float r,
                                                      const float* __restrict__ pre, const float* __restrict__ gamma,
                                                      const float* __restrict__ beta,
                                                      const double* __restrict__ gst, long V,
                                                      double* __restrict__ partials, int cpg, int groups) {
  using Ln = GnLanes<C, 4>;
  __shared__ GnConst k;
  __shared__ double red[8][GMAX][2];
  load_gn_const(k, gst, nullptr, groups, 0.f);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sub = lane / Ln::LPV, q = lane % Ln::LPV;
  const bool active = sub < Ln::VPW;
  constexpr int VW = Ln::VW;
  const int c = VW * q;
  float gm[VW], bt[VW];
  int grp[VW];
#pragma unroll
  for (int j = 0; j < VW; ++j) {
    gm[j] = active ? __ldg(gamma + c + j) : 0.f;
    bt[j] = active ? __ldg(beta + c + j) : 0.f;
    grp[j] = (c + j) / cpg;
  }
  double d1[VW], d2[VW];   // per element slot (groups of slot j fixed per thread)
  float f1[VW], f2[VW];
#pragma unroll
  for (int j = 0; j < VW; ++j) d1[j] = d2[j] = 0.0, f1[j] = f2[j] = 0.f;
  const long step = (long)gridDim.x * 8 * Ln::VPW;
  // UN voxels a thread are loaded before any is used (128 bytes in flight); float partials go to double every 4
  // rounds
  constexpr int UN = 16 / VW;
  int n = 0;
  for (long v0 = ((long)blockIdx.x * 8 + warp) * Ln::VPW + sub; active && v0 < V; v0 += UN * step) {
    float pu[UN][VW], pp[UN][VW];
#pragma unroll
    for (int e = 0; e < UN; ++e) {
      const long v = v0 + e * step;
      if (v < V) {
        ldv<VW>(u + v * C + c, pu[e]);
        ldv<VW>(pre + v * C + c, pp[e]);
      } else {
#pragma unroll
        for (int j = 0; j < VW; ++j) pu[e][j] = pp[e][j] = 0.f;
      }
    }
#pragma unroll
    for (int e = 0; e < UN; ++e) {
      if (v0 + e * step >= V) break;
#pragma unroll
      for (int j = 0; j < VW; ++j) {
        const int g = grp[j];
        const float xh = (pp[e][j] - k.mean[g]) * k.rstd[g];
        const float gh = upstream(mode, pu[e][j], r, xh * gm[j] + bt[j]) * gm[j];
        f1[j] += gh;
        f2[j] += gh * xh;
      }
    }
    if (++n == 16 / UN) {
#pragma unroll
      for (int j = 0; j < VW; ++j) {
        d1[j] += f1[j];
        d2[j] += f2[j];
        f1[j] = f2[j] = 0.f;
      }
      n = 0;
    }
  }
#pragma unroll
  for (int j = 0; j < VW; ++j) {
    d1[j] += f1[j];
    d2[j] += f2[j];
  }
  // per group: warp reduce (lanes of other groups contribute 0), then warps in order
  for (int g = 0; g < groups; ++g) {
    double a = 0.0, b = 0.0;
#pragma unroll
    for (int j = 0; j < VW; ++j)
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

// The statistics for eight groups and C <= 64 (cpg = C / 8 channels a group): lanes of 8 channels (one 32-byte request
// a lane and tensor), whose channels fall in NG = 8 / cpg groups, so the partials are kept per group (one double pair
// at C = 64) instead of per channel slot. Same partials layout and fixed reduction order as k_gn_bwd_stats.
template <int C>
__global__ void __launch_bounds__(256) k_gn_bwd_stats8(int mode, const float* __restrict__ u, float r,
                                                       const float* __restrict__ pre, const float* __restrict__ gamma,
                                                       const float* __restrict__ beta,
                                                       const double* __restrict__ gst, long V,
                                                       double* __restrict__ partials) {
  static_assert(C == 16 || C == 32 || C == 64, "eight groups of C / 8 channels");
  using Ln = GnLanes<C, 8>;
  constexpr int VW = 8, CPG = C / GMAX, NG = VW / CPG;
  __shared__ GnConst k;
  __shared__ double red[8][GMAX][2];
  load_gn_const(k, gst, nullptr, GMAX, 0.f);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sub = lane / Ln::LPV, q = lane % Ln::LPV;   // every lane is active: LPV divides 32
  const int c = VW * q, g0 = c / CPG;
  float gm[VW], bt[VW];
#pragma unroll
  for (int j = 0; j < VW; ++j) {
    gm[j] = __ldg(gamma + c + j);
    bt[j] = __ldg(beta + c + j);
  }
  double d1[NG], d2[NG];
  float f1[NG], f2[NG];
#pragma unroll
  for (int l = 0; l < NG; ++l) d1[l] = d2[l] = 0.0, f1[l] = f2[l] = 0.f;
  const long step = (long)gridDim.x * 8 * Ln::VPW;
  constexpr int UN = 2;   // voxels a thread loaded before any is used: 128 bytes in flight
  int n = 0;
  for (long v0 = ((long)blockIdx.x * 8 + warp) * Ln::VPW + sub; v0 < V; v0 += UN * step) {
    float pu[UN][VW], pp[UN][VW];
#pragma unroll
    for (int e = 0; e < UN; ++e) {
      const long v = v0 + e * step;
      if (v < V) {
        ffno::tc::ld8(u + v * C + c, pu[e]);
        ffno::tc::ld8(pre + v * C + c, pp[e]);
      } else {
#pragma unroll
        for (int j = 0; j < VW; ++j) pu[e][j] = pp[e][j] = 0.f;
      }
    }
#pragma unroll
    for (int e = 0; e < UN; ++e) {
      if (v0 + e * step >= V) break;
#pragma unroll
      for (int j = 0; j < VW; ++j) {
        const int l = j / CPG, g = g0 + l;
        const float xh = (pp[e][j] - k.mean[g]) * k.rstd[g];
        const float gh = upstream(mode, pu[e][j], r, xh * gm[j] + bt[j]) * gm[j];
        f1[l] += gh;
        f2[l] += gh * xh;
      }
    }
    if (++n == 8) {   // float partials go to double every 16 voxels, as in k_gn_bwd_stats
#pragma unroll
      for (int l = 0; l < NG; ++l) {
        d1[l] += f1[l];
        d2[l] += f2[l];
        f1[l] = f2[l] = 0.f;
      }
      n = 0;
    }
  }
#pragma unroll
  for (int l = 0; l < NG; ++l) {
    d1[l] += f1[l];
    d2[l] += f2[l];
  }
  for (int g = 0; g < GMAX; ++g) {
    double a = 0.0, b = 0.0;
#pragma unroll
    for (int l = 0; l < NG; ++l)
      if (g0 + l == g) {
        a += d1[l];
        b += d2[l];
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
  if (threadIdx.x < GMAX) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < 8; ++w) {
      a += red[w][threadIdx.x][0];
      b += red[w][threadIdx.x][1];
    }
    partials[((long)blockIdx.x * GMAX + threadIdx.x) * 2] = a;
    partials[((long)blockIdx.x * GMAX + threadIdx.x) * 2 + 1] = b;
  }
}

__global__ void k_gn_bwd_final(const double* __restrict__ partials, int nparts, int groups, double* __restrict__ sums) {
  // one warp per group: strided partial sums per lane, then a fixed shuffle tree (deterministic)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int g = warp; g < groups; g += nw) {
    double s1 = 0.0, s2 = 0.0;
    for (int p = lane; p < nparts; p += 32) {
      s1 += partials[((long)p * groups + g) * 2];
      s2 += partials[((long)p * groups + g) * 2 + 1];
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      s1 += __shfl_down_sync(0xffffffffu, s1, off);
      s2 += __shfl_down_sync(0xffffffffu, s2, off);
    }
    if (lane == 0) {
      sums[2 * g] = s1;
      sums[2 * g + 1] = s2;
    }
  }
}

// pre_bar = rstd (ghat - (w / T)(S1 + xhat S2)); w_bar[v] += sum_c (1/T)(-S1 xhat - S2 (xhat^2 - var rstd^2) / 2).
template <int C>
__global__ void __launch_bounds__(256, 4) k_gn_bwd_apply(int mode, const float* __restrict__ u, float r,
                                                      const float* __restrict__ pre, const float* __restrict__ gamma,
                                                      const float* __restrict__ beta,
                                                      const double* __restrict__ gst, const double* __restrict__ sums,
                                                      const float* __restrict__ dw, long V,
                                                      float* __restrict__ pre_bar, float* __restrict__ w_bar, int cpg,
                                                      int groups, float eps) {
  using Ln = GnLanes<C, 8>;
  __shared__ GnConst k;
  load_gn_const(k, gst, sums, groups, eps);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int sub = lane / Ln::LPV, q = lane % Ln::LPV;
  const bool active = sub < Ln::VPW;
  constexpr int VW = Ln::VW;
  const int c = VW * q;
  float gm[VW], bt[VW];
  int grp[VW];
#pragma unroll
  for (int j = 0; j < VW; ++j) {
    gm[j] = active ? __ldg(gamma + c + j) : 0.f;
    bt[j] = active ? __ldg(beta + c + j) : 0.f;
    grp[j] = (c + j) / cpg;
  }
  const long step = (long)gridDim.x * 8 * Ln::VPW;
  const long first = ((long)blockIdx.x * 8 + warp) * Ln::VPW;
  for (long vb = first; vb < V; vb += step) {   // warp-uniform loop
    const long v = vb + sub;
    const bool ok = active && v < V;
    float wc = 0.f;
    if (ok) {
      const float wv = __ldg(dw + v);
      float uu[VW], xx[VW], o[VW];
      ldv<VW>(u + v * C + c, uu);
      ldv<VW>(pre + v * C + c, xx);
#pragma unroll
      for (int j = 0; j < VW; ++j) {
        const int g = grp[j];
        const float xh = (xx[j] - k.mean[g]) * k.rstd[g];
        const float gh = upstream(mode, uu[j], r, xh * gm[j] + bt[j]) * gm[j];
        o[j] = k.rstd[g] * (gh - wv * k.invT[g] * (k.s1[g] + xh * k.s2[g]));
        wc += k.invT[g] * (-k.s1[g] * xh - 0.5f * k.s2[g] * (xh * xh - k.vr2[g]));
      }
      stv<VW>(pre_bar + v * C + c, o);
    }
    // sum over the LPV lanes of this voxel (segments of a power-of-two LPV, or the whole warp for C = 96)
    if (Ln::LPV >= 32 || (Ln::LPV & (Ln::LPV - 1))) {
#pragma unroll
      for (int off = 16; off; off >>= 1) wc += __shfl_xor_sync(0xffffffffu, wc, off);
    } else {
#pragma unroll
      for (int off = Ln::LPV / 2; off; off >>= 1) wc += __shfl_xor_sync(0xffffffffu, wc, off);
    }
    if (ok && q == 0) w_bar[v] += wc;
  }
}

// ------------------------------------------------------------------------------------------------ MLP backward
// pre = gelu(a W1) W2; given pre_bar: a_bar = base + ((pre_bar W2^T) * gelu'(a W1)) W1^T.
template <int C>
__global__ void __launch_bounds__(NT) k_mlp2_bwd(const float* __restrict__ a, const float* __restrict__ pb,
                                                 const float* __restrict__ base, long V, const float* __restrict__ w1,
                                                 const float* __restrict__ w2t, const float* __restrict__ w1t,
                                                 float* __restrict__ abar) {
  extern __shared__ float sm[];
  constexpr int LA = C + 1, LH = 2 * C + 1;
  float* as = sm;
  float* ps = as + BM * LA;
  float* hs = ps + BM * LA;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const long nt = ntiles(V, BM);
  for (long t = blockIdx.x; t < nt; t += gridDim.x) {
    const long v0 = t * BM;
    __syncthreads();
    load_rows<C>(as, LA, a, v0, V);
    load_rows<C>(ps, LA, pb, v0, V);
    __syncthreads();
    {
      float hp[4][2 * C / 16], gb[4][2 * C / 16];
      tile_mm<C, 2 * C>(as, LA, w1, hp);
      tile_mm<C, 2 * C>(ps, LA, w2t, gb);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2 * C / 16; ++j) hs[(ty + 16 * i) * LH + tx + 16 * j] = gb[i][j] * gelu_grad(hp[i][j]);
    }
    __syncthreads();
    float acc[4][C / 16];
    tile_mm<2 * C, C>(hs, LH, w1t, acc);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const long v = v0 + ty + 16 * i;
      if (v >= V) continue;
#pragma unroll
      for (int j = 0; j < C / 16; ++j) {
        const int c = tx + 16 * j;
        abar[v * C + c] = acc[i][j] + (base ? __ldg(base + v * C + c) : 0.f);
      }
    }
  }
}

// ------------------------------------------------------------------------------------------------ fuse backward
// Recomputes the gate/fuse chain of the tile and back-propagates fused_pre_bar (= pb) to x, spec and vert
// (FFNOBlock3dBalanced._fuse_branches, models/ffno_model.py:524-534).
template <int C, int RM>
__global__ void __launch_bounds__(NT) k_fuse_bwd(
    const float* __restrict__ x, const float* __restrict__ sp, const float* __restrict__ sc,
    const float* __restrict__ vp, const float* __restrict__ vc, const float* __restrict__ pb,
    const float* __restrict__ base, long V, const float* __restrict__ wg1, const float* __restrict__ wg2,
    const float* __restrict__ bg2, const float* __restrict__ wf1, const float* __restrict__ wf2t,
    const float* __restrict__ wf1t, const float* __restrict__ wg2t, const float* __restrict__ wg1t,
    float* __restrict__ xbar, float* __restrict__ sbar, float* __restrict__ vbar) {
  extern __shared__ float sm[];
  constexpr int R = 16 * RM;
  constexpr int LA = 3 * C + 1, L1 = C + 1, L2 = 2 * C + 1;
  float* SA = sm;              // [R][3C]  x | spec | vert
  float* SH1 = SA + R * LA;    // [R][C]   branch-gate hidden pre-activation, later its gradient
  float* SG = SH1 + R * L1;    // [R][2C]  gates
  float* SH2 = SG + R * L2;    // [R][2C]  fuse hidden pre-activation, later its gradient
  float* ST = SH2 + R * L2;    // [R][2C]  GEMM operand scratch
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const long nt = ntiles(V, R);
  for (long t = blockIdx.x; t < nt; t += gridDim.x) {
    const long v0 = t * R;
    __syncthreads();
    for (int e = threadIdx.x; e < R * C; e += NT) {
      const int r = e / C, c = e % C;
      const long v = v0 + r;
      float a = 0.f, s = 0.f, q = 0.f, f = 0.f;
      if (v < V) {
        a = __ldg(x + v * C + c);
        s = gelu((__ldg(sp + v * C + c) - sc[c]) * sc[C + c] + sc[2 * C + c]);
        q = gelu((__ldg(vp + v * C + c) - vc[c]) * vc[C + c] + vc[2 * C + c]);
        f = __ldg(pb + v * C + c);
      }
      SA[r * LA + c] = a;
      SA[r * LA + C + c] = s;
      SA[r * LA + 2 * C + c] = q;
      SH2[r * L2 + c] = f;  // fused_pre_bar parked in SH2 until step 4
    }
    __syncthreads();
    // 1. branch-gate hidden
    {
      float acc[RM][C / 16];
      tile_mm<3 * C, C, RM>(SA, LA, wg1, acc);
#pragma unroll
      for (int i = 0; i < RM; ++i)
#pragma unroll
        for (int j = 0; j < C / 16; ++j) {
          const int o = (ty + 16 * i);
          SH1[o * L1 + tx + 16 * j] = acc[i][j];
          ST[o * L2 + tx + 16 * j] = gelu(acc[i][j]);
        }
    }
    __syncthreads();
    // 2. gates
    {
      float acc[RM][2 * C / 16];
      tile_mm<C, 2 * C, RM>(ST, L2, wg2, acc);
#pragma unroll
      for (int i = 0; i < RM; ++i)
#pragma unroll
        for (int j = 0; j < 2 * C / 16; ++j) {
          const int n = tx + 16 * j;
          SG[(ty + 16 * i) * L2 + n] = sigmoid(acc[i][j] + __ldg(bg2 + n));
        }
    }
    __syncthreads();
    // 3. mixed branches B = [spec g_s, vert g_v] -> ST; fused_pre_bar moves to ST's right half is not needed:
    //    keep F in registers of the thread that owns it below
    float fb[RM][C / 16];
#pragma unroll
    for (int i = 0; i < RM; ++i)
#pragma unroll
      for (int j = 0; j < C / 16; ++j) fb[i][j] = SH2[(ty + 16 * i) * L2 + tx + 16 * j];
#pragma unroll
    for (int i = 0; i < RM; ++i)
#pragma unroll
      for (int j = 0; j < 2 * C / 16; ++j) {
        const int r = ty + 16 * i, n = tx + 16 * j;
        ST[r * L2 + n] = SA[r * LA + C + n] * SG[r * L2 + n];
      }
    __syncthreads();
    // 4. fuse hidden pre-activation -> registers; then F (fused_pre_bar) into ST for the next GEMM
    float hf[RM][2 * C / 16];
    tile_mm<2 * C, 2 * C, RM>(ST, L2, wf1, hf);
    __syncthreads();
#pragma unroll
    for (int i = 0; i < RM; ++i)
#pragma unroll
      for (int j = 0; j < C / 16; ++j) ST[(ty + 16 * i) * L2 + tx + 16 * j] = fb[i][j];
    __syncthreads();
    // 5. fuse hidden gradient (times gelu') -> SH2
    {
      float acc[RM][2 * C / 16];
      tile_mm<C, 2 * C, RM>(ST, L2, wf2t, acc);
#pragma unroll
      for (int i = 0; i < RM; ++i)
#pragma unroll
        for (int j = 0; j < 2 * C / 16; ++j) SH2[(ty + 16 * i) * L2 + tx + 16 * j] = acc[i][j] * gelu_grad(hf[i][j]);
    }
    __syncthreads();
    // 6. B_bar = SH2 Wf1^T + 0.5 [F, F]; branch grads (registers) and the gate pre-activation grad -> ST
    float br[RM][2 * C / 16];
    {
      float acc[RM][2 * C / 16];
      tile_mm<2 * C, 2 * C, RM>(SH2, L2, wf1t, acc);
      __syncthreads();
#pragma unroll
      for (int i = 0; i < RM; ++i)
#pragma unroll
        for (int j = 0; j < 2 * C / 16; ++j) {
          const int r = ty + 16 * i, n = tx + 16 * j;
          const float bb = acc[i][j] + 0.5f * fb[i][j % (C / 16)];
          const float g = SG[r * L2 + n];
          br[i][j] = bb * g;                                   // d/d spec (n < C) or vert (n >= C)
          ST[r * L2 + n] = bb * SA[r * LA + C + n] * g * (1.f - g);  // d/d gate pre-activation
        }
    }
    __syncthreads();
    // 7. branch-gate hidden gradient (times gelu') -> SH1
    {
      float acc[RM][C / 16];
      tile_mm<2 * C, C, RM>(ST, L2, wg2t, acc);
#pragma unroll
      for (int i = 0; i < RM; ++i)
#pragma unroll
        for (int j = 0; j < C / 16; ++j) {
          const int o = (ty + 16 * i) * L1 + tx + 16 * j;
          SH1[o] = acc[i][j] * gelu_grad(SH1[o]);
        }
    }
    __syncthreads();
    // 8. A_bar = SH1 Wg1^T: x, spec, vert gradients
    {
      float acc[RM][3 * C / 16];
      tile_mm<C, 3 * C, RM>(SH1, L1, wg1t, acc);
#pragma unroll
      for (int i = 0; i < RM; ++i) {
        const long v = v0 + ty + 16 * i;
        if (v >= V) continue;
#pragma unroll
        for (int j = 0; j < C / 16; ++j) {
          const int c = tx + 16 * j;
          xbar[v * C + c] = acc[i][j] + (base ? __ldg(base + v * C + c) : 0.f);
          sbar[v * C + c] = acc[i][j + C / 16] + br[i][j];
          vbar[v * C + c] = acc[i][j + 2 * C / 16] + br[i][j + C / 16];
        }
      }
    }
  }
}

// ------------------------------------------------------------------------------------------------ gate backward
// x_bar = base + sum over the two branches of d/dx [x * sigmoid(gelu(x G1) G2)] applied to that branch's gradient;
// z_bar += sum_c xv_bar * zp (the z_proj term of the vertical branch, models/ffno_model.py:265).
template <int C>
__global__ void __launch_bounds__(NT) k_gate_bwd(const float* __restrict__ x, const float* __restrict__ xsb,
                                                 const float* __restrict__ xvb, const float* __restrict__ base,
                                                 long V, const float* __restrict__ s1, const float* __restrict__ s2,
                                                 const float* __restrict__ s2t, const float* __restrict__ s1t,
                                                 const float* __restrict__ v1, const float* __restrict__ v2,
                                                 const float* __restrict__ v2t, const float* __restrict__ v1t,
                                                 const float* __restrict__ zp, float* __restrict__ xbar,
                                                 float* __restrict__ zbar) {
  extern __shared__ float sm[];
  constexpr int LD = C + 1;
  float* SX = sm;
  float* SB = SX + BM * LD;
  float* SP = SB + BM * LD;
  float* ST = SP + BM * LD;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const long nt = ntiles(V, BM);
  for (long t = blockIdx.x; t < nt; t += gridDim.x) {
    const long v0 = t * BM;
    float xb[4][C / 16];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < C / 16; ++j) xb[i][j] = 0.f;
    __syncthreads();
    load_rows<C>(SX, LD, x, v0, V);
    for (int br = 0; br < 2; ++br) {
      const float* gbar = br ? xvb : xsb;
      const float* g1 = br ? v1 : s1;
      const float* g2 = br ? v2 : s2;
      const float* g2t = br ? v2t : s2t;
      const float* g1t = br ? v1t : s1t;
      __syncthreads();
      load_rows<C>(SB, LD, gbar, v0, V);
      __syncthreads();
      {
        float acc[4][C / 16];
        tile_mm<C, C>(SX, LD, g1, acc);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < C / 16; ++j) {
            const int o = (ty + 16 * i) * LD + tx + 16 * j;
            SP[o] = acc[i][j];
            ST[o] = gelu(acc[i][j]);
          }
      }
      __syncthreads();
      {
        float acc[4][C / 16];
        tile_mm<C, C>(ST, LD, g2, acc);
        __syncthreads();
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < C / 16; ++j) {
            const int o = (ty + 16 * i) * LD + tx + 16 * j;
            const float g = sigmoid(acc[i][j]);
            const float b = SB[o];
            xb[i][j] += b * g;
            ST[o] = b * SX[o] * g * (1.f - g);
          }
      }
      __syncthreads();
      {
        float acc[4][C / 16];
        tile_mm<C, C>(ST, LD, g2t, acc);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < C / 16; ++j) {
            const int o = (ty + 16 * i) * LD + tx + 16 * j;
            SP[o] = acc[i][j] * gelu_grad(SP[o]);
          }
      }
      __syncthreads();
      {
        float acc[4][C / 16];
        tile_mm<C, C>(SP, LD, g1t, acc);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < C / 16; ++j) xb[i][j] += acc[i][j];
      }
      if (br == 1 && zp) {
        // z_bar[v] += sum_c xv_bar[v][c] zp[c]; the 16 threads of one row are one half-warp
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          float s = 0.f;
#pragma unroll
          for (int j = 0; j < C / 16; ++j) s += SB[(ty + 16 * i) * LD + tx + 16 * j] * __ldg(zp + tx + 16 * j);
          s += __shfl_xor_sync(0xffffffffu, s, 8);
          s += __shfl_xor_sync(0xffffffffu, s, 4);
          s += __shfl_xor_sync(0xffffffffu, s, 2);
          s += __shfl_xor_sync(0xffffffffu, s, 1);
          const long v = v0 + ty + 16 * i;
          if (tx == 0 && v < V) zbar[v] += s;
        }
      }
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const long v = v0 + ty + 16 * i;
      if (v >= V) continue;
#pragma unroll
      for (int j = 0; j < C / 16; ++j) {
        const int c = tx + 16 * j;
        xbar[v * C + c] = xb[i][j] + (base ? __ldg(base + v * C + c) : 0.f);
      }
    }
  }
}

// ------------------------------------------------------------------------------------------------ lift backward
// x_in_bar[k][v] += sum_c pre_bar[v][c] w_lift[k][c]
template <int C>
__global__ void __launch_bounds__(NT) k_lift_bwd(const float* __restrict__ pb, int cin, long V,
                                                 const float* __restrict__ wl, float* __restrict__ xib) {
  __shared__ float ps[BM][C + 1];
  const long nt = ntiles(V, BM);
  for (long t = blockIdx.x; t < nt; t += gridDim.x) {
    const long v0 = t * BM;
    __syncthreads();
    load_rows<C>(&ps[0][0], C + 1, pb, v0, V);
    __syncthreads();
    for (int e = threadIdx.x; e < cin * BM; e += NT) {
      const int k = e / BM, r = e % BM;
      const long v = v0 + r;
      if (v >= V) continue;
      float s = 0.f;
      for (int c = 0; c < C; ++c) s = fmaf(ps[r][c], __ldg(wl + k * C + c), s);
      xib[(long)k * V + v] += s;
    }
  }
}

// ------------------------------------------------------------------------------------------------ head backward

// kLte = false: the VJP of FFNO3D._run_head alone (models/ffno_model.py:790-798); ybar is then the gradient of the
// nh head channels [nh][V] and xin / xinbar are not used.
template <int C, int NHP, typename T, bool kLte = true>
__global__ void __launch_bounds__(NT) k_head_bwd(const float* __restrict__ x, const float* __restrict__ xin,
                                                 const float* __restrict__ ybar, long V, const float* __restrict__ p1,
                                                 const float* __restrict__ p2, const float* __restrict__ b2,
                                                 const float* __restrict__ p2t, const float* __restrict__ p1t,
                                                 const __grid_constant__ ffno_head_params hp, int nh,
                                                 float* __restrict__ xbar, float* __restrict__ xinbar) {
  extern __shared__ float sm[];
  constexpr int LA = C + 1, LH = 2 * C + 1, LO = NHP + 1;
  float* SA = sm;
  float* SP = SA + BM * LA;   // hidden pre-activation
  float* SG = SP + BM * LH;   // gelu(hidden), later the hidden gradient
  float* SO = SG + BM * LH;   // head channels, later their gradient
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const long nt = ntiles(V, BM);
  for (long t = blockIdx.x; t < nt; t += gridDim.x) {
    const long v0 = t * BM;
    __syncthreads();
    load_rows<C>(SA, LA, x, v0, V);
    __syncthreads();
    {
      float acc[4][2 * C / 16];
      tile_mm<C, 2 * C>(SA, LA, p1, acc);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2 * C / 16; ++j) {
          const int o = (ty + 16 * i) * LH + tx + 16 * j;
          SP[o] = acc[i][j];
          SG[o] = gelu(acc[i][j]);
        }
    }
    __syncthreads();
    {
      float acc[4][NHP / 16];
      tile_mm<2 * C, NHP>(SG, LH, p2, acc);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < NHP / 16; ++j) SO[(ty + 16 * i) * LO + tx + 16 * j] = acc[i][j] + __ldg(b2 + tx + 16 * j);
    }
    __syncthreads();
    if (threadIdx.x < BM) {
      const int r = threadIdx.x;
      const long v = v0 + r;
      float* o = SO + r * LO;
      if (v < V) {
        if constexpr (kLte) {
          head_voxel_bwd<T>(hp, o, NHP, head_inputs(hp, xin, V, v), ybar, V, v, xinbar);
        } else {
          for (int c = 0; c < NHP; ++c) o[c] = c < nh ? __ldg(ybar + (long)c * V + v) : 0.f;
        }
      } else {
        for (int c = 0; c < NHP; ++c) o[c] = 0.f;
      }
    }
    __syncthreads();
    {
      float acc[4][2 * C / 16];
      tile_mm<NHP, 2 * C>(SO, LO, p2t, acc);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2 * C / 16; ++j) {
          const int o = (ty + 16 * i) * LH + tx + 16 * j;
          SG[o] = acc[i][j] * gelu_grad(SP[o]);
        }
    }
    __syncthreads();
    {
      float acc[4][C / 16];
      tile_mm<2 * C, C>(SG, LH, p1t, acc);
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const long v = v0 + ty + 16 * i;
        if (v >= V) continue;
#pragma unroll
        for (int j = 0; j < C / 16; ++j) xbar[v * C + tx + 16 * j] = acc[i][j];
      }
    }
  }
}

// VJP of FFNO3D.head_output on precomputed head channels: one thread per voxel; head_bar [nh][V] and x_in_bar
// [cin][V] are written (the T, ne and rho channels carry the LTE and total terms, the others are zero).
template <typename T>
__global__ void __launch_bounds__(256) k_head_output_bwd(const float* __restrict__ head, const float* __restrict__ xin,
                                                         const float* __restrict__ ybar, long V, int nh,
                                                         const __grid_constant__ ffno_head_params hp,
                                                         float* __restrict__ hbar, float* __restrict__ xinbar) {
  float o[FFNO_MAX_LEVELS + FFNO_MAX_SPECIES];
  for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < V; v += (long)gridDim.x * blockDim.x) {
    for (int c = 0; c < nh; ++c) o[c] = __ldg(head + (long)c * V + v);
    head_voxel_bwd<T>(hp, o, nh, head_inputs(hp, xin, V, v), ybar, V, v, xinbar);
    for (int c = 0; c < nh; ++c) hbar[(long)c * V + v] = o[c];
  }
}

// ------------------------------------------------------------------------------------------------ depth weights
// w = t / max(mean_d t, 1e-12), t_d = |z_{d+1} - z_d| / 2 + |z_d - z_{d-1}| / 2 (models/ffno_model.py:28-34, 67-74)
__global__ void k_depth_weights_bwd(const float* __restrict__ z, const float* __restrict__ wb, int D, long HW,
                                    float* __restrict__ zb) {
  const long col = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (col >= HW || D == 1) return;
  auto Z = [&](int d) { return z[(long)d * HW + col]; };
  auto T = [&](int d) {
    float t = 0.f;
    if (d + 1 < D) t += 0.5f * fabsf(Z(d + 1) - Z(d));
    if (d > 0) t += 0.5f * fabsf(Z(d) - Z(d - 1));
    return t;
  };
  float sum = 0.f;
  for (int d = 0; d < D; ++d) sum += T(d);
  const float mraw = sum / (float)D;
  const bool clamped = mraw < 1e-12f;
  const float m = clamped ? 1e-12f : mraw;
  // d/dt_d: wb_d / m - [m not clamped] (sum_j wb_j t_j / m^2) / D
  float corr = 0.f;
  if (!clamped) {
    for (int d = 0; d < D; ++d) corr += wb[(long)d * HW + col] * T(d);
    corr /= m * m * (float)D;
  }
  // segment s_d = z_{d+1} - z_d feeds t_d and t_{d+1} with weight sign(s_d) / 2
  for (int d = 0; d + 1 < D; ++d) {
    const float s = Z(d + 1) - Z(d);
    const float sg = (s > 0.f) ? 1.f : ((s < 0.f) ? -1.f : 0.f);
    const float tb0 = wb[(long)d * HW + col] / m - corr;
    const float tb1 = wb[(long)(d + 1) * HW + col] / m - corr;
    const float sb = 0.5f * sg * (tb0 + tb1);
    zb[(long)(d + 1) * HW + col] += sb;
    zb[(long)d * HW + col] -= sb;
  }
}

// ------------------------------------------------------------------------------------------------ A B^T split-K
// part[split][i][j] = sum_{n in split's range} A[i][n] B[j][n]; CTA tile 64 x 64.
__global__ void __launch_bounds__(NT) k_outer(const float* __restrict__ A, long lda, int Ma,
                                              const float* __restrict__ B, long ldb, int Mb, long N, long chunk,
                                              int ti, int tj, float* __restrict__ part) {
  // 64 x 64 output tile, k in chunks of 64 read as float4 (16 threads per row: 256 contiguous bytes)
  __shared__ float as[64][65];
  __shared__ float bs[64][65];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  long bid = blockIdx.x;
  const int bi = (int)(bid % ti);
  bid /= ti;
  const int bj = (int)(bid % tj);
  const long split = bid / tj;
  const long n0 = split * chunk;
  const long n1 = (n0 + chunk < N) ? n0 + chunk : N;
  float acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.f;
  for (long k0 = n0; k0 < n1; k0 += 64) {
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int e = threadIdx.x + u * NT;
      const int r = e >> 4, c = (e & 15) * 4;
      const long n = k0 + c;
      const int i = bi * 64 + r, j = bj * 64 + r;
      float4 va = make_float4(0.f, 0.f, 0.f, 0.f), vb = va;
      if (n + 3 < n1) {
        if (i < Ma) va = __ldg(reinterpret_cast<const float4*>(A + (long)i * lda + n));
        if (j < Mb) vb = __ldg(reinterpret_cast<const float4*>(B + (long)j * ldb + n));
      } else {
        float ta[4] = {0.f, 0.f, 0.f, 0.f}, tb[4] = {0.f, 0.f, 0.f, 0.f};
        for (int q = 0; q < 4; ++q)
          if (n + q < n1) {
            if (i < Ma) ta[q] = __ldg(A + (long)i * lda + n + q);
            if (j < Mb) tb[q] = __ldg(B + (long)j * ldb + n + q);
          }
        va = make_float4(ta[0], ta[1], ta[2], ta[3]);
        vb = make_float4(tb[0], tb[1], tb[2], tb[3]);
      }
      as[r][c] = va.x;
      as[r][c + 1] = va.y;
      as[r][c + 2] = va.z;
      as[r][c + 3] = va.w;
      bs[r][c] = vb.x;
      bs[r][c + 1] = vb.y;
      bs[r][c + 2] = vb.z;
      bs[r][c + 3] = vb.w;
    }
    __syncthreads();
#pragma unroll 16
    for (int k = 0; k < 64; ++k) {
      float a[4], b[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        a[q] = as[ty + 16 * q][k];
        b[q] = bs[tx + 16 * q][k];
      }
#pragma unroll
      for (int p = 0; p < 4; ++p)
#pragma unroll
        for (int q = 0; q < 4; ++q) acc[p][q] = fmaf(a[p], b[q], acc[p][q]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < 4; ++p) {
    const int i = bi * 64 + ty + 16 * p;
    if (i >= Ma) continue;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int j = bj * 64 + tx + 16 * q;
      if (j < Mb) part[(split * Ma + i) * (long)Mb + j] = acc[p][q];
    }
  }
}

__global__ void k_outer_reduce(const float* __restrict__ part, long nsplit, long n, double* __restrict__ out,
                               int accumulate) {
  const long e = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (e >= n) return;
  double s = 0.0;
  for (long p = 0; p < nsplit; ++p) s += (double)part[p * n + e];
  out[e] = accumulate ? out[e] + s : s;
}

}  // namespace

// ====================================================================================================== C ABI
extern "C" {

int ffno_gn_bwd_stats(int mode, const float* u, float r, const float* pre, const float* gamma, const float* beta,
                      const double* gstats, long V, int C, int groups, double* partials, int nparts,
                      ffno_stream_t stream) {
  if (!u || !pre || !gamma || !beta || !gstats || !partials) return FFNO_EINVAL;
  if (mode < 0 || mode > 2) return FFNO_EINVAL;
  if (!width_ok(C) || V < 1 || groups < 1 || groups > GMAX || C % groups || nparts < 1) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  const int cpg = C / groups;
  if (groups == GMAX && C <= 64 &&
      (reinterpret_cast<uintptr_t>(u) | reinterpret_cast<uintptr_t>(pre)) % 32 == 0) {   // 32-byte lanes
    switch (C) {
#define L(CC) case CC: k_gn_bwd_stats8<CC><<<nparts, 256, 0, s>>>(mode, u, r, pre, gamma, beta, gstats, V, partials); break;
      L(16) L(32) L(64)
#undef L
    }
    FFNO_CHECK_LAUNCH();
    return FFNO_OK;
  }
  switch (C) {
#define L(CC) case CC: k_gn_bwd_stats<CC><<<nparts, 256, 0, s>>>(mode, u, r, pre, gamma, beta, gstats, V, partials, cpg, groups); break;
    L(16) L(32) L(64) L(96)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_gn_bwd_final(const double* partials, int nparts, int groups, double* sums, ffno_stream_t stream) {
  if (!partials || !sums || nparts < 1 || groups < 1 || groups > GMAX) return FFNO_EINVAL;
  k_gn_bwd_final<<<1, 512, 0, (cudaStream_t)stream>>>(partials, nparts, groups, sums);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_gn_bwd_apply(int mode, const float* u, float r, const float* pre, const float* gamma, const float* beta,
                      const double* gstats, const double* sums, const float* dw, long V, int C, int groups, float eps,
                      float* pre_bar, float* w_bar, ffno_stream_t stream) {
  if (!u || !pre || !gamma || !beta || !gstats || !dw || !pre_bar || !w_bar) return FFNO_EINVAL;
  if (mode < 0 || mode > 2) return FFNO_EINVAL;
  if (!width_ok(C) || V < 1 || groups < 1 || groups > GMAX || C % groups) return FFNO_EINVAL;
  // a lane moves 32 bytes of a row per request for C <= 64, 16 bytes for C = 96
  const uintptr_t al = C <= 64 ? 32 : 16;
  if ((reinterpret_cast<uintptr_t>(u) | reinterpret_cast<uintptr_t>(pre) | reinterpret_cast<uintptr_t>(pre_bar)) % al)
    return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  const int cpg = C / groups;
  const int blocks = grid_of(V, 8 * 8, 4);
  switch (C) {
#define L(CC) case CC: k_gn_bwd_apply<CC><<<blocks, 256, 0, s>>>(mode, u, r, pre, gamma, beta, gstats, sums, dw, V, pre_bar, w_bar, cpg, groups, eps); break;
    L(16) L(32) L(64) L(96)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_mlp2_bwd(const float* a, const float* pre_bar, const float* base, long V, int C, const float* w1,
                  const float* w2t, const float* w1t, float* a_bar, ffno_stream_t stream) {
  if (!a || !pre_bar || !w1 || !w2t || !w1t || !a_bar || !width_ok(C) || V < 1) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  switch (C) {
#define L(CC)                                                                                   \
  case CC: {                                                                                    \
    const size_t smem = (2 * BM * (CC + 1) + BM * (2 * CC + 1)) * sizeof(float);                \
    if (!smem_attr(k_mlp2_bwd<CC>, smem)) return FFNO_ELAUNCH;                                  \
    k_mlp2_bwd<CC><<<grid_of(V, BM, 2), NT, smem, s>>>(a, pre_bar, base, V, w1, w2t, w1t, a_bar); \
    break;                                                                                      \
  }
    L(16) L(32) L(64) L(96)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_fuse_bwd(const float* x, const float* spec_pre, const float* spec_coefs, const float* vert_pre,
                  const float* vert_coefs, const float* fused_pre_bar, const float* base, long V, int C,
                  const float* wg1, const float* wg2, const float* bg2, const float* wf1, const float* wf2t,
                  const float* wf1t, const float* wg2t, const float* wg1t, float* x_bar, float* spec_bar,
                  float* vert_bar, ffno_stream_t stream) {
  if (!x || !spec_pre || !spec_coefs || !vert_pre || !vert_coefs || !fused_pre_bar || !wg1 || !wg2 || !bg2 || !wf1 ||
      !wf2t || !wf1t || !wg2t || !wg1t || !x_bar || !spec_bar || !vert_bar)
    return FFNO_EINVAL;
  if (!width_ok(C) || V < 1) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  switch (C) {
#define L(CC, RMV)                                                                                          \
  case CC: {                                                                                                \
    constexpr int R = 16 * RMV;                                                                             \
    const size_t smem = (size_t)R * ((3 * CC + 1) + (CC + 1) + 3 * (2 * CC + 1)) * sizeof(float);          \
    if (!smem_attr(k_fuse_bwd<CC, RMV>, smem)) return FFNO_ELAUNCH;                                         \
    k_fuse_bwd<CC, RMV><<<grid_of(V, R, 2), NT, smem, s>>>(x, spec_pre, spec_coefs, vert_pre, vert_coefs,     \
                                                           fused_pre_bar, base, V, wg1, wg2, bg2, wf1, wf2t,  \
                                                           wf1t, wg2t, wg1t, x_bar, spec_bar, vert_bar);      \
    break;                                                                                                  \
  }
    L(16, 4) L(32, 4) L(64, 4) L(96, 2)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_gate_bwd(const float* x, const float* xs_bar, const float* xv_bar, const float* base, long V, int C,
                  const float* s_w1, const float* s_w2, const float* s_w2t, const float* s_w1t, const float* v_w1,
                  const float* v_w2, const float* v_w2t, const float* v_w1t, const float* zp, float* x_bar,
                  float* z_bar, ffno_stream_t stream) {
  if (!x || !xs_bar || !xv_bar || !s_w1 || !s_w2 || !s_w2t || !s_w1t || !v_w1 || !v_w2 || !v_w2t || !v_w1t || !x_bar)
    return FFNO_EINVAL;
  if (!width_ok(C) || V < 1 || (zp && !z_bar)) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  switch (C) {
#define L(CC)                                                                                              \
  case CC: {                                                                                               \
    const size_t smem = 4 * BM * (CC + 1) * sizeof(float);                                                  \
    if (!smem_attr(k_gate_bwd<CC>, smem)) return FFNO_ELAUNCH;                                             \
    k_gate_bwd<CC><<<grid_of(V, BM, 2), NT, smem, s>>>(x, xs_bar, xv_bar, base, V, s_w1, s_w2, s_w2t, s_w1t, \
                                                       v_w1, v_w2, v_w2t, v_w1t, zp, x_bar, z_bar);          \
    break;                                                                                                 \
  }
    L(16) L(32) L(64) L(96)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_lift_bwd(const float* pre_bar, int cin, long V, int C, const float* w_lift, float* x_in_bar,
                  ffno_stream_t stream) {
  if (!pre_bar || !w_lift || !x_in_bar || !width_ok(C) || V < 1 || cin < 1 || cin > 8) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  switch (C) {
#define L(CC) case CC: k_lift_bwd<CC><<<grid_of(V, BM, 4), NT, 0, s>>>(pre_bar, cin, V, w_lift, x_in_bar); break;
    L(16) L(32) L(64) L(96)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_head_bwd(const float* x, const float* x_in, const float* y_bar, long V, int C, const float* p1,
                  const float* p2, const float* b2, const float* p2t, const float* p1t, int nhp,
                  const ffno_head_params* params, float* x_bar, float* x_in_bar, ffno_stream_t stream) {
  if (!x || !x_in || !y_bar || !p1 || !p2 || !b2 || !p2t || !p1t || !x_bar || !x_in_bar) return FFNO_EINVAL;
  if (!width_ok(C) || V < 1 || !params || (nhp != 16 && nhp != 32)) return FFNO_EINVAL;
  if (params->nspecies < 1 || params->nspecies > FFNO_MAX_SPECIES || params->in_channels > 8) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  switch (C) {
#define L(CC, NN)                                                                                        \
  if (C == CC && nhp == NN) {                                                                            \
    const size_t smem = (BM * (CC + 1) + 2 * BM * (2 * CC + 1) + BM * (NN + 1)) * sizeof(float);         \
    if (params->math32) {                                                                               \
      if (!smem_attr(k_head_bwd<CC, NN, float>, smem)) return FFNO_ELAUNCH;                             \
      k_head_bwd<CC, NN, float><<<grid_of(V, BM, 2), NT, smem, s>>>(x, x_in, y_bar, V, p1, p2, b2, p2t, p1t, \
                                                                    *params, NN, x_bar, x_in_bar);          \
    } else {                                                                                            \
      if (!smem_attr(k_head_bwd<CC, NN, double>, smem)) return FFNO_ELAUNCH;                            \
      k_head_bwd<CC, NN, double><<<grid_of(V, BM, 2), NT, smem, s>>>(x, x_in, y_bar, V, p1, p2, b2, p2t, p1t, \
                                                                     *params, NN, x_bar, x_in_bar);         \
    }                                                                                                   \
  }
    default:
      L(16, 16) L(16, 32) L(32, 16) L(32, 32) L(64, 16) L(64, 32) L(96, 16) L(96, 32)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_depth_weights_bwd(const float* z, const float* w_bar, int D, long HW, float* z_bar, ffno_stream_t stream) {
  if (!z || !w_bar || !z_bar || D < 1 || HW < 1) return FFNO_EINVAL;
  k_depth_weights_bwd<<<(unsigned)((HW + 255) / 256), 256, 0, (cudaStream_t)stream>>>(z, w_bar, D, HW, z_bar);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_outer_parts(int Ma, int Mb, long N) {
  const long tiles = (long)((Ma + 63) / 64) * ((Mb + 63) / 64);
  long nsplit = (4L * sms() + tiles - 1) / tiles;
  const long maxs = (N + 1023) / 1024;
  if (nsplit > maxs) nsplit = maxs;
  if (nsplit < 1) nsplit = 1;
  return (int)nsplit;
}

int ffno_outer(const float* A, long lda, int Ma, const float* B, long ldb, int Mb, long N, float* part, int nsplit,
               double* out, int accumulate, ffno_stream_t stream) {
  if (!A || !B || !part || !out || Ma < 1 || Mb < 1 || N < 1 || nsplit < 1) return FFNO_EINVAL;
  const int ti = (Ma + 63) / 64, tj = (Mb + 63) / 64;
  if (lda % 4 || ldb % 4 || (reinterpret_cast<uintptr_t>(A) % 16) || (reinterpret_cast<uintptr_t>(B) % 16))
    return FFNO_EINVAL;   // float4 loads
  long chunk = (N + nsplit - 1) / nsplit;
  chunk = (chunk + 63) / 64 * 64;
  cudaStream_t s = (cudaStream_t)stream;
  k_outer<<<(unsigned)((long)ti * tj * nsplit), NT, 0, s>>>(A, lda, Ma, B, ldb, Mb, N, chunk, ti, tj, part);
  const long n = (long)Ma * Mb;
  k_outer_reduce<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(part, nsplit, n, out, accumulate);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

// ---------------------------------------------------------------------------------------------- no-allocation variant
// ffno_outer_noalloc: the same product as ffno_outer for hosts that cannot hand this library a scratch buffer on every
// call. A process that binds the C ABI from its own runtime (a Julia, Go or Java host whose device memory belongs to
// that runtime's own pool allocator, or a service that must not grow its footprint after start-up) often has no way to
// call cudaMalloc for us, and the split-K partial sums need somewhere to live. They live here instead: a fixed array in
// the library's own device memory, present on every GPU that loads the library until the process exits.
}  // extern "C"

namespace {

constexpr long kOuterScratchFloats = 4L << 20;  // 16 MiB: Ma * Mb * nsplit partial sums at most
__device__ __align__(256) float g_outer_scratch[kOuterScratchFloats];

std::mutex g_outer_scratch_mutex;
float* g_outer_scratch_ptr[256] = {};  // device address of g_outer_scratch per device ordinal, set on first use

}  // namespace

extern "C" {

int ffno_outer_noalloc(const float* A, long lda, int Ma, const float* B, long ldb, int Mb, long N, double* out,
                       int accumulate, ffno_stream_t stream) {
  if (!A || !B || !out || Ma < 1 || Mb < 1 || N < 1) return FFNO_EINVAL;
  const long n = (long)Ma * Mb;
  if (n > kOuterScratchFloats) return FFNO_ETOOBIG;
  if (lda % 4 || ldb % 4 || (reinterpret_cast<uintptr_t>(A) % 16) || (reinterpret_cast<uintptr_t>(B) % 16))
    return FFNO_EINVAL;   // k_outer reads float4
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return FFNO_EINVAL;
  float* scratch = nullptr;
  {
    // The host-side name g_outer_scratch is not a device address: ask the runtime for it once per device, with that
    // device current.
    std::lock_guard<std::mutex> lock(g_outer_scratch_mutex);
    if (!g_outer_scratch_ptr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_outer_scratch) != cudaSuccess || !p) return FFNO_ELAUNCH;
      g_outer_scratch_ptr[dev] = static_cast<float*>(p);
    }
    scratch = g_outer_scratch_ptr[dev];
  }
  long nsplit = ffno_outer_parts(Ma, Mb, N);
  if (nsplit > kOuterScratchFloats / n) nsplit = kOuterScratchFloats / n;
  const int ti = (Ma + 63) / 64, tj = (Mb + 63) / 64;
  long chunk = (N + nsplit - 1) / nsplit;
  chunk = (chunk + 63) / 64 * 64;
  cudaStream_t s = (cudaStream_t)stream;
  // every partial sum the reduction reads is written first by k_outer: nothing in the scratch has to start at zero
  k_outer<<<(unsigned)((long)ti * tj * nsplit), NT, 0, s>>>(A, lda, Ma, B, ldb, Mb, N, chunk, ti, tj, scratch);
  k_outer_reduce<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(scratch, nsplit, n, out, accumulate);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_proj_bwd(const float* x, const float* head_bar, long V, int C, const float* p1, const float* p2,
                  const float* b2, const float* p2t, const float* p1t, int nh, int nhp, float* x_bar,
                  ffno_stream_t stream) {
  if (!x || !head_bar || !p1 || !p2 || !b2 || !p2t || !p1t || !x_bar) return FFNO_EINVAL;
  if (!width_ok(C) || V < 1 || (nhp != 16 && nhp != 32) || nh < 1 || nh > nhp) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  ffno_head_params none{};
  switch (C) {
#define L(CC, NN)                                                                                        \
  if (C == CC && nhp == NN) {                                                                            \
    const size_t smem = (BM * (CC + 1) + 2 * BM * (2 * CC + 1) + BM * (NN + 1)) * sizeof(float);         \
    if (!smem_attr(k_head_bwd<CC, NN, float, false>, smem)) return FFNO_ELAUNCH;                         \
    k_head_bwd<CC, NN, float, false><<<grid_of(V, BM, 2), NT, smem, s>>>(x, nullptr, head_bar, V, p1, p2, b2, \
                                                                         p2t, p1t, none, nh, x_bar, nullptr); \
  }
    default:
      L(16, 16) L(16, 32) L(32, 16) L(32, 32) L(64, 16) L(64, 32) L(96, 16) L(96, 32)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_head_output_bwd(const float* head, const float* x_in, const float* y_bar, long V, int nh,
                         const ffno_head_params* params, float* head_bar, float* x_in_bar, ffno_stream_t stream) {
  if (!head || !x_in || !y_bar || !params || !head_bar || !x_in_bar) return FFNO_EINVAL;
  if (V < 1 || params->nspecies < 1 || params->nspecies > FFNO_MAX_SPECIES || params->in_channels > 8)
    return FFNO_EINVAL;
  int tot = 0, lv = 0;
  for (int s = 0; s < params->nspecies; ++s) {
    if (params->levels[s] < 1) return FFNO_EINVAL;
    tot += params->levels[s] + 1;
    lv += params->levels[s];
  }
  if (tot != nh || lv > FFNO_MAX_LEVELS) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  const long want = (V + 255) / 256, cap = 8L * sms();   // 8 CTAs of 256 threads per SM, grid-stride
  const long blocks = want < cap ? want : cap;
  if (params->math32)
    k_head_output_bwd<float><<<(unsigned)blocks, 256, 0, s>>>(head, x_in, y_bar, V, nh, *params, head_bar, x_in_bar);
  else
    k_head_output_bwd<double><<<(unsigned)blocks, 256, 0, s>>>(head, x_in, y_bar, V, nh, *params, head_bar,
                                                               x_in_bar);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

}  // extern "C"
