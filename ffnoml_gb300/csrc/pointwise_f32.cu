// FP32 pointwise kernels of the FFNO3D forward: lift, input gates, the 2-layer channel MLPs with fused residual
// prologues and GroupNorm-statistics epilogues, the branch-gate/fuse chain and the projection + level-fraction head.
// Every kernel is persistent over 64-voxel tiles (grid-stride), so the GroupNorm partials it writes have one row per
// CTA and a fixed summation order.
#include <math.h>

#include "common.cuh"

using namespace ffno;

namespace {

int g_num_sms = 0;

int num_sms() {
  if (!g_num_sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 152;
  }
  return g_num_sms;
}

__host__ __device__ __forceinline__ long ntiles_of(long V) { return (V + BM - 1) / BM; }

int grid_for(long V, int per_sm) {
  long t = ntiles_of(V);
  long g = (long)num_sms() * per_sm;
  return (int)(t < g ? (t > 0 ? t : 1) : g);
}

template <typename K>
bool set_smem(K kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return true;
  return ffno::smem_cap_ok(kernel, bytes);
}

// ------------------------------------------------------------------------------------------------ depth weights
__global__ void k_depth_weights(const float* __restrict__ z, int D, long HW, float* __restrict__ w) {
  const long col = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (col >= HW) return;
  if (D == 1) {
    w[col] = 1.f;
    return;
  }
  float sum = 0.f;
  float prev = z[col];
  float half_prev = 0.f;
  for (int d = 0; d < D; ++d) {
    float half_next = 0.f;
    if (d + 1 < D) {
      const float nx = z[(long)(d + 1) * HW + col];
      half_next = 0.5f * fabsf(nx - prev);
      prev = nx;
    }
    const float t = half_prev + half_next;
    w[(long)d * HW + col] = t;
    sum += t;
    half_prev = half_next;
  }
  const float mean = fmaxf(sum / (float)D, 1e-12f);
  for (int d = 0; d < D; ++d) w[(long)d * HW + col] /= mean;
}

// ------------------------------------------------------------------------------------------------ column info
__global__ void k_column_info(const float* __restrict__ z, int D, long HW, unsigned int* __restrict__ flags) {
  // flags[0]: 1 while every column equals column 0 (each shifted by its own minimum); flags[1]: float bits of the
  // largest span (non-negative floats order as unsigned ints)
  const long col = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (col >= HW) return;
  float mn = z[col], mx = z[col], mn0 = z[0];
  for (int d = 1; d < D; ++d) {
    const float v = z[(long)d * HW + col];
    mn = fminf(mn, v);
    mx = fmaxf(mx, v);
    mn0 = fminf(mn0, z[(long)d * HW]);
  }
  bool same = true;
  for (int d = 0; d < D && same; ++d) same = (z[(long)d * HW + col] - mn) == (z[(long)d * HW] - mn0);
  if (!same) atomicAnd(flags, 0u);
  atomicMax(flags + 1, __float_as_uint(mx - mn));
}

__global__ void k_column_info_init(unsigned int* flags) {
  flags[0] = 1u;
  flags[1] = 0u;
}

__global__ void k_column_info_final(unsigned int* flags) {
  float* out = reinterpret_cast<float*>(flags);
  const unsigned int s = flags[0];
  out[0] = s ? 1.f : 0.f;  // flags[1] already holds the span's float bits
}

// ------------------------------------------------------------------------------------------------ lift
template <int C>
__global__ void __launch_bounds__(NT) k_lift(const float* __restrict__ xin, int cin, long V,
                                             const float* __restrict__ wl, const float* __restrict__ dw,
                                             float* __restrict__ pre, double* __restrict__ partials, int cpg,
                                             int groups) {
  __shared__ float xs[8][BM];
  __shared__ StatsSmem<C> st;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  GroupAcc acc{0.0, 0.0, 0.0};
  const long nt = ntiles_of(V);
  for (long t = blockIdx.x; t < nt; t += gridDim.x) {
    const long v0 = t * BM;
    __syncthreads();
    for (int e = threadIdx.x; e < cin * BM; e += NT) {
      const int k = e / BM, r = e % BM;
      xs[k][r] = (v0 + r < V) ? __ldg(xin + (long)k * V + v0 + r) : 0.f;
    }
    __syncthreads();
    float val[4][C / 16], wr[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = ty + 16 * i;
      const long v = v0 + r;
      wr[i] = v < V ? __ldg(dw + v) : 0.f;
#pragma unroll
      for (int j = 0; j < C / 16; ++j) {
        const int c = tx + 16 * j;
        float s = 0.f;
        for (int k = 0; k < cin; ++k) s = fmaf(xs[k][r], __ldg(wl + k * C + c), s);
        val[i][j] = s;
        if (v < V) pre[v * C + c] = s;
      }
    }
    tile_group_stats<C>(val, wr, cpg, groups, st, acc);
  }
  write_partial(partials, groups, acc);
}

// ------------------------------------------------------------------------------------------------ GN finalize
__global__ void k_gn_finalize(const double* __restrict__ partials, int nparts, int C, int groups,
                              const float* __restrict__ gamma, const float* __restrict__ beta, float eps,
                              float* __restrict__ coefs, double* __restrict__ gstats) {
  __shared__ double gm[GMAX], gr[GMAX];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  // one warp per group: lane l merges partials l, l + 32, ... in order, then a fixed shuffle tree (deterministic)
  for (int g = warp; g < groups; g += nw) {
    GroupAcc a{0.0, 0.0, 0.0};
    for (int p = lane; p < nparts; p += 32) {
      const double* q = partials + ((long)p * groups + g) * 3;
      chan_merge(a, q[0], q[1], q[2]);
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const double w = __shfl_down_sync(0xffffffffu, a.w, off);
      const double m = __shfl_down_sync(0xffffffffu, a.mean, off);
      const double m2 = __shfl_down_sync(0xffffffffu, a.m2, off);
      if (lane < off) chan_merge(a, w, m, m2);
    }
    if (lane == 0) {
      const double var = a.w > 0.0 ? a.m2 / a.w : 0.0;
      const double rstd = 1.0 / sqrt(var + (double)eps);
      gm[g] = a.mean;
      gr[g] = rstd;
      if (gstats) {
        gstats[3 * g] = a.mean;
        gstats[3 * g + 1] = rstd;
        gstats[3 * g + 2] = a.w;
      }
    }
  }
  __syncthreads();
  const int cpg = C / groups;
  for (int c = tid; c < C; c += blockDim.x) {
    const int g = c / cpg;
    coefs[c] = (float)gm[g];
    coefs[C + c] = (float)((double)gamma[c] * gr[g]);
    coefs[2 * C + c] = beta[c];
  }
}

// ------------------------------------------------------------------------------------------------ elementwise
// y = GN(pre) from the finalized coefficients, 4 channels a thread (float4), two float4 in flight per round; the
// channel index from a 32-bit modulo (n / 4 < 2^31 is checked by the launchers).
__device__ __forceinline__ float4 gn4(float4 p, const float* __restrict__ cf, int C, int c) {
  const float4 m = __ldg(reinterpret_cast<const float4*>(cf + c));
  const float4 sc = __ldg(reinterpret_cast<const float4*>(cf + C + c));
  const float4 b = __ldg(reinterpret_cast<const float4*>(cf + 2 * C + c));
  return make_float4((p.x - m.x) * sc.x + b.x, (p.y - m.y) * sc.y + b.y, (p.z - m.z) * sc.z + b.z,
                     (p.w - m.w) * sc.w + b.w);
}

__global__ void k_gn_act(const float* __restrict__ pre, const float* __restrict__ coefs, unsigned n4, int C, int act,
                         float* __restrict__ out) {
  const unsigned C4 = (unsigned)C / 4, stride = gridDim.x * blockDim.x;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += 2 * stride) {
    const unsigned i2 = i + stride;
    const float4 p0 = __ldg(reinterpret_cast<const float4*>(pre) + i);
    const float4 p1 = i2 < n4 ? __ldg(reinterpret_cast<const float4*>(pre) + i2) : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 y = gn4(p0, coefs, C, (int)(i % C4) * 4);
    if (act) y = make_float4(gelu(y.x), gelu(y.y), gelu(y.z), gelu(y.w));
    reinterpret_cast<float4*>(out)[i] = y;
    if (i2 < n4) {
      y = gn4(p1, coefs, C, (int)(i2 % C4) * 4);
      if (act) y = make_float4(gelu(y.x), gelu(y.y), gelu(y.z), gelu(y.w));
      reinterpret_cast<float4*>(out)[i2] = y;
    }
  }
}

__global__ void k_resid_out(const float* __restrict__ x2, const float* __restrict__ pre,
                            const float* __restrict__ coefs, float res, unsigned n4, int C, float* __restrict__ out) {
  const unsigned C4 = (unsigned)C / 4, stride = gridDim.x * blockDim.x;
  for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += 2 * stride) {
    const unsigned i2 = i + stride;
    const bool two = i2 < n4;
    const float4 p0 = __ldg(reinterpret_cast<const float4*>(pre) + i);
    const float4 a0 = __ldg(reinterpret_cast<const float4*>(x2) + i);
    const float4 p1 = two ? __ldg(reinterpret_cast<const float4*>(pre) + i2) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 a1 = two ? __ldg(reinterpret_cast<const float4*>(x2) + i2) : make_float4(0.f, 0.f, 0.f, 0.f);
    float4 y = gn4(p0, coefs, C, (int)(i % C4) * 4);
    reinterpret_cast<float4*>(out)[i] =
        make_float4(fmaf(res, y.x, a0.x), fmaf(res, y.y, a0.y), fmaf(res, y.z, a0.z), fmaf(res, y.w, a0.w));
    if (two) {
      y = gn4(p1, coefs, C, (int)(i2 % C4) * 4);
      reinterpret_cast<float4*>(out)[i2] =
          make_float4(fmaf(res, y.x, a1.x), fmaf(res, y.y, a1.y), fmaf(res, y.z, a1.z), fmaf(res, y.w, a1.w));
    }
  }
}

// ------------------------------------------------------------------------------------------------ input gate
template <int C>
__global__ void __launch_bounds__(NT) k_gate(const float* __restrict__ x, long V, const float* __restrict__ w1,
                                             const float* __restrict__ w2, const float* __restrict__ zp,
                                             const float* __restrict__ z, float* __restrict__ out) {
  extern __shared__ float sm[];
  constexpr int LD = C + 1;
  float* xs = sm;
  float* hs = xs + BM * LD;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const long nt = ntiles_of(V);
  for (long t = blockIdx.x; t < nt; t += gridDim.x) {
    const long v0 = t * BM;
    __syncthreads();
    load_rows<C>(xs, LD, x, v0, V);
    __syncthreads();
    float acc[4][C / 16];
    tile_mm<C, C>(xs, LD, w1, acc);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < C / 16; ++j) hs[(ty + 16 * i) * LD + tx + 16 * j] = gelu(acc[i][j]);
    __syncthreads();
    tile_mm<C, C>(hs, LD, w2, acc);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = ty + 16 * i;
      const long v = v0 + r;
      if (v >= V) continue;
      const float zv = zp ? __ldg(z + v) : 0.f;
#pragma unroll
      for (int j = 0; j < C / 16; ++j) {
        const int c = tx + 16 * j;
        float o = xs[r * LD + c] * sigmoid(acc[i][j]);
        if (zp) o += __ldg(zp + c) * zv;
        out[v * C + c] = o;
      }
    }
  }
}

// ------------------------------------------------------------------------------------------------ 2-layer MLP
template <int C, int MODE>
__global__ void __launch_bounds__(NT) k_mlp2(const float* __restrict__ in, const float* __restrict__ prev_pre,
                                             const float* __restrict__ pc, float res, float* __restrict__ xout,
                                             long V, const float* __restrict__ w1, const float* __restrict__ w2,
                                             const float* __restrict__ dw, float* __restrict__ pre,
                                             double* __restrict__ partials, int cpg, int groups) {
  extern __shared__ float sm[];
  constexpr int LA = C + 1, LH = 2 * C + 1;
  float* as = sm;
  float* hs = as + BM * LA;
  StatsSmem<C>& st = *reinterpret_cast<StatsSmem<C>*>(hs + BM * LH);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  GroupAcc acc_g{0.0, 0.0, 0.0};
  const long nt = ntiles_of(V);
  for (long t = blockIdx.x; t < nt; t += gridDim.x) {
    const long v0 = t * BM;
    __syncthreads();
    load_rows<C>(as, LA, in, v0, V);
    if (MODE != 0) {
      __syncthreads();
      for (int e = threadIdx.x; e < BM * C; e += NT) {
        const int r = e / C, c = e % C;
        const long v = v0 + r;
        if (v >= V) continue;
        float y = (__ldg(prev_pre + v * C + c) - pc[c]) * pc[C + c] + pc[2 * C + c];
        if (MODE == 1) y = gelu(y);
        const float a = as[r * LA + c] + res * y;
        as[r * LA + c] = a;
        xout[v * C + c] = a;
      }
    }
    __syncthreads();
    {
      float acc[4][2 * C / 16];
      tile_mm<C, 2 * C>(as, LA, w1, acc);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2 * C / 16; ++j) hs[(ty + 16 * i) * LH + tx + 16 * j] = gelu(acc[i][j]);
    }
    __syncthreads();
    float acc[4][C / 16], wr[4];
    tile_mm<2 * C, C>(hs, LH, w2, acc);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const long v = v0 + ty + 16 * i;
      wr[i] = v < V ? __ldg(dw + v) : 0.f;
      if (v < V) {
#pragma unroll
        for (int j = 0; j < C / 16; ++j) pre[v * C + tx + 16 * j] = acc[i][j];
      }
    }
    tile_group_stats<C>(acc, wr, cpg, groups, st, acc_g);
  }
  write_partial(partials, groups, acc_g);
}

// ------------------------------------------------------------------------------------------------ gate + fuse
template <int C>
__global__ void __launch_bounds__(NT) k_fuse(const float* __restrict__ x, const float* __restrict__ sp,
                                             const float* __restrict__ sc, const float* __restrict__ vp,
                                             const float* __restrict__ vc, long V, const float* __restrict__ wg1,
                                             const float* __restrict__ wg2, const float* __restrict__ bg2,
                                             const float* __restrict__ wf1, const float* __restrict__ wf2,
                                             const float* __restrict__ dw, float* __restrict__ pre,
                                             double* __restrict__ partials, int cpg, int groups) {
  extern __shared__ float sm[];
  constexpr int LA = 3 * C + 1, LH = 2 * C + 1;
  float* as = sm;
  float* hs = as + BM * LA;
  StatsSmem<C>& st = *reinterpret_cast<StatsSmem<C>*>(hs + BM * LH);
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  GroupAcc acc_g{0.0, 0.0, 0.0};
  const long nt = ntiles_of(V);
  for (long t = blockIdx.x; t < nt; t += gridDim.x) {
    const long v0 = t * BM;
    __syncthreads();
    for (int e = threadIdx.x; e < BM * C; e += NT) {
      const int r = e / C, c = e % C;
      const long v = v0 + r;
      float a = 0.f, s = 0.f, q = 0.f;
      if (v < V) {
        a = __ldg(x + v * C + c);
        s = gelu((__ldg(sp + v * C + c) - sc[c]) * sc[C + c] + sc[2 * C + c]);
        q = gelu((__ldg(vp + v * C + c) - vc[c]) * vc[C + c] + vc[2 * C + c]);
      }
      as[r * LA + c] = a;
      as[r * LA + C + c] = s;
      as[r * LA + 2 * C + c] = q;
    }
    __syncthreads();
    {
      float acc[4][C / 16];
      tile_mm<3 * C, C>(as, LA, wg1, acc);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < C / 16; ++j) hs[(ty + 16 * i) * LH + tx + 16 * j] = gelu(acc[i][j]);
    }
    __syncthreads();
    {
      float acc[4][2 * C / 16];
      tile_mm<C, 2 * C>(hs, LH, wg2, acc);
      // gates multiply spec (columns C..2C) and vert (2C..3C) in place: column n of the gates -> as[:, C + n]
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2 * C / 16; ++j) {
          const int n = tx + 16 * j;
          as[(ty + 16 * i) * LA + C + n] *= sigmoid(acc[i][j] + __ldg(bg2 + n));
        }
    }
    __syncthreads();
    {
      float acc[4][2 * C / 16];
      tile_mm<2 * C, 2 * C>(as + C, LA, wf1, acc);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2 * C / 16; ++j) hs[(ty + 16 * i) * LH + tx + 16 * j] = gelu(acc[i][j]);
    }
    __syncthreads();
    float acc[4][C / 16], wr[4];
    tile_mm<2 * C, C>(hs, LH, wf2, acc);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int r = ty + 16 * i;
      const long v = v0 + r;
      wr[i] = v < V ? __ldg(dw + v) : 0.f;
#pragma unroll
      for (int j = 0; j < C / 16; ++j) {
        const int c = tx + 16 * j;
        acc[i][j] += 0.5f * (as[r * LA + C + c] + as[r * LA + 2 * C + c]);
        if (v < V) pre[v * C + c] = acc[i][j];
      }
    }
    tile_group_stats<C>(acc, wr, cpg, groups, st, acc_g);
  }
  write_partial(partials, groups, acc_g);
}

// ------------------------------------------------------------------------------------------------ head

// kLte = false: FFNO3D._run_head alone (models/ffno_model.py:790-798), the head channels into head_out, no LTE head.
template <int C, int NHP, typename T, bool kLte = true>
__global__ void __launch_bounds__(NT) k_head(const float* __restrict__ x, const float* __restrict__ xin, long V,
                                             const float* __restrict__ p1, const float* __restrict__ p2,
                                             const float* __restrict__ b2, int nh,
                                             const __grid_constant__ ffno_head_params hp, float* __restrict__ out,
                                             float* __restrict__ head_out) {
  extern __shared__ float sm[];
  constexpr int LA = C + 1, LH = 2 * C + 1, LO = NHP + 1;
  float* as = sm;
  float* hs = as + BM * LA;
  float* os = hs + BM * LH;
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const long nt = ntiles_of(V);
  for (long t = blockIdx.x; t < nt; t += gridDim.x) {
    const long v0 = t * BM;
    __syncthreads();
    load_rows<C>(as, LA, x, v0, V);
    __syncthreads();
    {
      float acc[4][2 * C / 16];
      tile_mm<C, 2 * C>(as, LA, p1, acc);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 2 * C / 16; ++j) hs[(ty + 16 * i) * LH + tx + 16 * j] = gelu(acc[i][j]);
    }
    __syncthreads();
    {
      float acc[4][NHP / 16];
      tile_mm<2 * C, NHP>(hs, LH, p2, acc);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < NHP / 16; ++j) os[(ty + 16 * i) * LO + tx + 16 * j] = acc[i][j] + __ldg(b2 + tx + 16 * j);
    }
    __syncthreads();
    if (threadIdx.x < BM) {
      const int r = threadIdx.x;
      const long v = v0 + r;
      if (v < V) {
        const float* o = os + r * LO;
        if (head_out)
          for (int c = 0; c < nh; ++c) head_out[(long)c * V + v] = o[c];
        if constexpr (kLte) head_voxel_fwd<T>(hp, o, head_inputs(hp, xin, V, v), out, V, v);
      }
    }
  }
}

// FFNO3D.head_output on head channels that are already computed (models/ffno_model.py:730-749): one thread per voxel,
// the head channels read channels-first (consecutive voxels of one channel plane per warp: coalesced), the levels
// written channels-first. Bound by HBM: (nh + 3 + levels) * 4 bytes a voxel.
template <typename T>
__global__ void __launch_bounds__(256) k_head_output(const float* __restrict__ head, const float* __restrict__ xin,
                                                     long V, int nh, const __grid_constant__ ffno_head_params hp,
                                                     float* __restrict__ out) {
  float o[FFNO_MAX_LEVELS + FFNO_MAX_SPECIES];
  for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < V; v += (long)gridDim.x * blockDim.x) {
    for (int c = 0; c < nh; ++c) o[c] = __ldg(head + (long)c * V + v);
    head_voxel_fwd<T>(hp, o, head_inputs(hp, xin, V, v), out, V, v);
  }
}

bool width_ok(int C) { return C == 16 || C == 32 || C == 64 || C == 96; }

}  // namespace

// ====================================================================================================== C ABI
extern "C" {

const char* ffno_version(void) { return "ffnoml_gb300 0.1 (sm_103a)"; }

int ffno_stats_parts(long V) { return grid_for(V, 2); }

int ffno_depth_weights(const float* z, int D, long HW, float* w, ffno_stream_t stream) {
  if (!z || !w || D < 1 || HW < 1) return FFNO_EINVAL;
  k_depth_weights<<<(unsigned)((HW + 255) / 256), 256, 0, (cudaStream_t)stream>>>(z, D, HW, w);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_column_info(const float* z, int D, long HW, float* out, ffno_stream_t stream) {
  if (!z || !out || D < 1 || HW < 1) return FFNO_EINVAL;
  unsigned int* flags = reinterpret_cast<unsigned int*>(out);
  k_column_info_init<<<1, 1, 0, (cudaStream_t)stream>>>(flags);
  k_column_info<<<(unsigned)((HW + 255) / 256), 256, 0, (cudaStream_t)stream>>>(z, D, HW, flags);
  k_column_info_final<<<1, 1, 0, (cudaStream_t)stream>>>(flags);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_lift_fwd(const float* x_in, int cin, long V, int C, const float* w_lift, const float* dw, float* pre,
                  double* partials, int nparts, int groups, ffno_stream_t stream) {
  if (!x_in || !w_lift || !dw || !pre || !partials) return FFNO_EINVAL;
  if (!width_ok(C) || cin < 1 || cin > 8 || V < 1 || groups < 1 || groups > GMAX || C % groups) return FFNO_EINVAL;
  if (nparts != ffno_stats_parts(V)) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  const int cpg = C / groups;
  switch (C) {
#define L(CC) case CC: k_lift<CC><<<nparts, NT, 0, s>>>(x_in, cin, V, w_lift, dw, pre, partials, cpg, groups); break;
    L(16) L(32) L(64) L(96)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_gn_finalize(const double* partials, int nparts, int C, int groups, const float* gamma, const float* beta,
                     float eps, float* coefs, double* gstats, ffno_stream_t stream) {
  if (!partials || !gamma || !beta || !coefs) return FFNO_EINVAL;
  if (nparts < 1 || C < 1 || groups < 1 || groups > GMAX || C % groups) return FFNO_EINVAL;
  k_gn_finalize<<<1, 512, 0, (cudaStream_t)stream>>>(partials, nparts, C, groups, gamma, beta, eps, coefs, gstats);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

bool elementwise_ok(long V, int C, const void* a, const void* b, const void* c) {
  return V >= 1 && C >= 4 && C % 4 == 0 && V * (long)C / 4 < 0x7fffffffL &&
         ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b) | reinterpret_cast<uintptr_t>(c)) % 16) == 0;
}

int elementwise_blocks(long n4) {
  const long want = (n4 + 511) / 512, cap = (long)num_sms() * 8;
  return (int)(want < cap ? (want > 0 ? want : 1) : cap);
}

int ffno_gn_act(const float* pre, const float* coefs, long V, int C, int act, float* out, ffno_stream_t stream) {
  if (!pre || !coefs || !out || !elementwise_ok(V, C, pre, coefs, out)) return FFNO_EINVAL;
  const long n4 = V * C / 4;
  k_gn_act<<<elementwise_blocks(n4), 256, 0, (cudaStream_t)stream>>>(pre, coefs, (unsigned)n4, C, act, out);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_resid_out(const float* x2, const float* pre, const float* coefs, float res, long V, int C, float* out,
                   ffno_stream_t stream) {
  if (!x2 || !pre || !coefs || !out || !elementwise_ok(V, C, x2, pre, out) ||
      reinterpret_cast<uintptr_t>(coefs) % 16)
    return FFNO_EINVAL;
  const long n4 = V * C / 4;
  k_resid_out<<<elementwise_blocks(n4), 256, 0, (cudaStream_t)stream>>>(x2, pre, coefs, res, (unsigned)n4, C, out);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_gate_fwd(const float* x, long V, int C, const float* w1, const float* w2, const float* zp, const float* z,
                  float* out, ffno_stream_t stream) {
  if (!x || !w1 || !w2 || !out || !width_ok(C) || V < 1 || (zp && !z)) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t smem = 2 * BM * (C + 1) * sizeof(float);
  switch (C) {
#define L(CC)                                                                   \
  case CC:                                                                      \
    if (!set_smem(k_gate<CC>, smem)) return FFNO_ELAUNCH;                       \
    k_gate<CC><<<grid_for(V, 2), NT, smem, s>>>(x, V, w1, w2, zp, z, out);      \
    break;
    L(16) L(32) L(64) L(96)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_mlp2_fwd(int mode, const float* in, const float* prev_pre, const float* prev_coefs, float res, float* xout,
                  long V, int C, const float* w1, const float* w2, const float* dw, float* pre, double* partials,
                  int nparts, int groups, ffno_stream_t stream) {
  if (!in || !w1 || !w2 || !dw || !pre || !partials) return FFNO_EINVAL;
  if (!width_ok(C) || V < 1 || mode < 0 || mode > 2 || groups < 1 || groups > GMAX || C % groups) return FFNO_EINVAL;
  if (mode && (!prev_pre || !prev_coefs || !xout)) return FFNO_EINVAL;
  if (nparts != ffno_stats_parts(V)) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  const int cpg = C / groups;
  switch (C) {
#define L(CC)                                                                                          \
  case CC: {                                                                                           \
    const size_t smem = (BM * (CC + 1) + BM * (2 * CC + 1)) * sizeof(float) + sizeof(StatsSmem<CC>);   \
    if (mode == 0) {                                                                                   \
      if (!set_smem(k_mlp2<CC, 0>, smem)) return FFNO_ELAUNCH;                                         \
      k_mlp2<CC, 0><<<nparts, NT, smem, s>>>(in, prev_pre, prev_coefs, res, xout, V, w1, w2, dw, pre,   \
                                             partials, cpg, groups);                                   \
    } else if (mode == 1) {                                                                            \
      if (!set_smem(k_mlp2<CC, 1>, smem)) return FFNO_ELAUNCH;                                         \
      k_mlp2<CC, 1><<<nparts, NT, smem, s>>>(in, prev_pre, prev_coefs, res, xout, V, w1, w2, dw, pre,   \
                                             partials, cpg, groups);                                   \
    } else {                                                                                           \
      if (!set_smem(k_mlp2<CC, 2>, smem)) return FFNO_ELAUNCH;                                         \
      k_mlp2<CC, 2><<<nparts, NT, smem, s>>>(in, prev_pre, prev_coefs, res, xout, V, w1, w2, dw, pre,   \
                                             partials, cpg, groups);                                   \
    }                                                                                                  \
    break;                                                                                             \
  }
    L(16) L(32) L(64) L(96)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_fuse_fwd(const float* x, const float* spec_pre, const float* spec_coefs, const float* vert_pre,
                  const float* vert_coefs, long V, int C, const float* wg1, const float* wg2, const float* bg2,
                  const float* wf1, const float* wf2, const float* dw, float* pre, double* partials, int nparts,
                  int groups, ffno_stream_t stream) {
  if (!x || !spec_pre || !spec_coefs || !vert_pre || !vert_coefs || !wg1 || !wg2 || !bg2 || !wf1 || !wf2 || !dw ||
      !pre || !partials)
    return FFNO_EINVAL;
  if (!width_ok(C) || V < 1 || groups < 1 || groups > GMAX || C % groups) return FFNO_EINVAL;
  if (nparts != ffno_stats_parts(V)) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  const int cpg = C / groups;
  switch (C) {
#define L(CC)                                                                                                \
  case CC: {                                                                                                 \
    const size_t smem = (BM * (3 * CC + 1) + BM * (2 * CC + 1)) * sizeof(float) + sizeof(StatsSmem<CC>);     \
    if (!set_smem(k_fuse<CC>, smem)) return FFNO_ELAUNCH;                                                    \
    k_fuse<CC><<<nparts, NT, smem, s>>>(x, spec_pre, spec_coefs, vert_pre, vert_coefs, V, wg1, wg2, bg2, wf1, \
                                        wf2, dw, pre, partials, cpg, groups);                                \
    break;                                                                                                   \
  }
    L(16) L(32) L(64) L(96)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_head_fwd(const float* x, const float* x_in, long V, int C, const float* p1, const float* p2, const float* b2,
                  int nh, int nhp, const ffno_head_params* params, float* out, float* head_out,
                  ffno_stream_t stream) {
  if (!x || !x_in || !p1 || !p2 || !b2 || !out) return FFNO_EINVAL;
  if (!width_ok(C) || V < 1 || !params || (nhp != 16 && nhp != 32) || nh > nhp) return FFNO_EINVAL;
  if (params->nspecies < 1 || params->nspecies > FFNO_MAX_SPECIES) return FFNO_EINVAL;
  int tot = 0;
  for (int s = 0; s < params->nspecies; ++s) tot += params->levels[s] + 1;
  if (tot != nh) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  switch (C) {
#define L(CC, NN)                                                                                       \
  if (C == CC && nhp == NN) {                                                                           \
    const size_t smem = (BM * (CC + 1) + BM * (2 * CC + 1) + BM * (NN + 1)) * sizeof(float);            \
    if (params->math32) {                                                                               \
      if (!set_smem(k_head<CC, NN, float>, smem)) return FFNO_ELAUNCH;                                  \
      k_head<CC, NN, float><<<grid_for(V, 2), NT, smem, s>>>(x, x_in, V, p1, p2, b2, nh, *params, out, head_out); \
    } else {                                                                                            \
      if (!set_smem(k_head<CC, NN, double>, smem)) return FFNO_ELAUNCH;                                 \
      k_head<CC, NN, double><<<grid_for(V, 2), NT, smem, s>>>(x, x_in, V, p1, p2, b2, nh, *params, out, head_out); \
    }                                                                                                   \
  }
    default:
      L(16, 16) L(16, 32) L(32, 16) L(32, 32) L(64, 16) L(64, 32) L(96, 16) L(96, 32)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_proj_fwd(const float* x, long V, int C, const float* p1, const float* p2, const float* b2, int nh, int nhp,
                  float* head, ffno_stream_t stream) {
  if (!x || !p1 || !p2 || !b2 || !head) return FFNO_EINVAL;
  if (!width_ok(C) || V < 1 || (nhp != 16 && nhp != 32) || nh < 1 || nh > nhp) return FFNO_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  ffno_head_params none{};
  switch (C) {
#define L(CC, NN)                                                                                       \
  if (C == CC && nhp == NN) {                                                                           \
    const size_t smem = (BM * (CC + 1) + BM * (2 * CC + 1) + BM * (NN + 1)) * sizeof(float);            \
    if (!set_smem(k_head<CC, NN, float, false>, smem)) return FFNO_ELAUNCH;                             \
    k_head<CC, NN, float, false><<<grid_for(V, 2), NT, smem, s>>>(x, nullptr, V, p1, p2, b2, nh, none,  \
                                                                  nullptr, head);                       \
  }
    default:
      L(16, 16) L(16, 32) L(32, 16) L(32, 32) L(64, 16) L(64, 32) L(96, 16) L(96, 32)
#undef L
  }
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_head_output(const float* head, const float* x_in, long V, int nh, const ffno_head_params* params,
                     float* out, ffno_stream_t stream) {
  if (!head || !x_in || !out || !params) return FFNO_EINVAL;
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
  const long want = (V + 255) / 256, cap = 8L * num_sms();   // 8 CTAs of 256 threads per SM, grid-stride
  const long blocks = want < cap ? want : cap;
  if (params->math32)
    k_head_output<float><<<(unsigned)blocks, 256, 0, s>>>(head, x_in, V, nh, *params, out);
  else
    k_head_output<double><<<(unsigned)blocks, 256, 0, s>>>(head, x_in, V, nh, *params, out);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

}  // extern "C"
