// Service-level conversions around the model (ffno_fsdp_runtime.py): SI features -> normalised model inputs
// (_model_inputs + normalisation, :48-58, :265-281), normalised log10 populations -> linear populations in the wire
// layout (linear_populations, _canonical_populations, :76-78, :283-292), and the matching VJP conversions. Each
// kernel also raises a device-side flag for non-finite or out-of-domain values, which the host turns into the
// reference's ValueError / RuntimeError.
#include <math.h>

#include "common.cuh"

namespace {

constexpr float kLn10 = 2.302585092994046f;
constexpr float kLog10Limit = 37.f;  // LOG10_POPULATION_LIMIT (ffno_fsdp_runtime.py:46)

// feat [6][V] SI (T [K], vx, vy, vz [m/s], log10 ne, log10 rho), z_m [V] metres -> x [6][V] normalised model inputs,
// z_mm [V] Mm. flags[0] |= 1 on a non-finite input, |= 2 on T <= 0.
__global__ void k_si_inputs(const float* __restrict__ feat, const float* __restrict__ zm, long V,
                            const float* __restrict__ mean_x, const float* __restrict__ std_x, float* __restrict__ x,
                            float* __restrict__ zmm, int* __restrict__ flags) {
  int bad = 0;
  for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < V; v += (long)gridDim.x * blockDim.x) {
    for (int c = 0; c < 6; ++c) {
      const float f = feat[(long)c * V + v];
      if (!isfinite(f)) bad |= 1;
      float m;
      if (c == 0) {
        if (!(f > 0.f)) bad |= 2;
        m = log10f(f);
      } else if (c < 4) {
        m = f / 1.0e3f;
      } else {
        m = f;
      }
      x[(long)c * V + v] = (m - mean_x[c]) / std_x[c];
    }
    const float z = zm[v];
    if (!isfinite(z)) bad |= 1;
    zmm[v] = z / 1.0e6f;
  }
  if (bad) atomicOr(flags, bad);
}

// y [L][V] normalised log10 n -> pop [V][L] = 10^clamp(y std + mean, +-37); flags |= 4 if a population is not
// positive and finite.
__global__ void k_si_populations(const float* __restrict__ y, long V, int L, const float* __restrict__ mean_y,
                                 const float* __restrict__ std_y, float* __restrict__ pop, int* __restrict__ flags) {
  int bad = 0;
  for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < V; v += (long)gridDim.x * blockDim.x) {
    for (int l = 0; l < L; ++l) {
      const float s = y[(long)l * V + v] * std_y[l] + mean_y[l];
      const float p = exp10f(fminf(fmaxf(s, -kLog10Limit), kLog10Limit));
      if (!(p > 0.f) || !isfinite(p)) bad |= 4;
      pop[v * L + l] = p;
    }
  }
  if (bad) atomicOr(flags, bad);
}

// cotangent on the populations pbar [V][L] -> ybar [L][V] on the normalised model output: pbar p ln10 std_y where the
// clamp is inactive; flags |= 1 on a non-finite cotangent.
__global__ void k_si_population_cotangent(const float* __restrict__ y, const float* __restrict__ pbar, long V, int L,
                                          const float* __restrict__ mean_y, const float* __restrict__ std_y,
                                          float* __restrict__ ybar, int* __restrict__ flags) {
  int bad = 0;
  for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < V; v += (long)gridDim.x * blockDim.x) {
    for (int l = 0; l < L; ++l) {
      const float s = y[(long)l * V + v] * std_y[l] + mean_y[l];
      const float b = pbar[v * L + l];
      if (!isfinite(b)) bad |= 1;
      const bool inside = s >= -kLog10Limit && s <= kLog10Limit;
      const float p = exp10f(fminf(fmaxf(s, -kLog10Limit), kLog10Limit));
      ybar[(long)l * V + v] = inside ? b * p * kLn10 * std_y[l] : 0.f;
    }
  }
  if (bad) atomicOr(flags, bad);
}

// gradients on the normalised inputs -> gradients on the SI features and heights; flags |= 8 if not finite.
__global__ void k_si_input_grads(const float* __restrict__ feat, const float* __restrict__ xbar,
                                 const float* __restrict__ zbar_mm, long V, const float* __restrict__ std_x,
                                 float* __restrict__ feat_bar, float* __restrict__ zbar_m, int* __restrict__ flags) {
  int bad = 0;
  for (long v = blockIdx.x * (long)blockDim.x + threadIdx.x; v < V; v += (long)gridDim.x * blockDim.x) {
    for (int c = 0; c < 6; ++c) {
      float g = xbar[(long)c * V + v] / std_x[c];
      if (c == 0)
        g = g / (feat[v] * kLn10);
      else if (c < 4)
        g = g / 1.0e3f;
      if (!isfinite(g)) bad |= 8;
      feat_bar[(long)c * V + v] = g;
    }
    const float zg = zbar_mm[v] / 1.0e6f;
    if (!isfinite(zg)) bad |= 8;
    zbar_m[v] = zg;
  }
  if (bad) atomicOr(flags, bad);
}

// out = in with its four axes reversed: in C-order [s0][s1][s2][s3], out C-order [s3][s2][s1][s0], i.e. the same
// array in Fortran order (the layout of the protocol's arrays, FFNOInversion.jl/src/FSDPService.jl). For a fixed i1
// the input is a [s0][s2 s3] matrix (rows contiguous) and the output, for each (i3, i2), a run of s0 contiguous
// values: a 32 x 32 shared-memory tile over (i0, k = i2 s3 + i3) reads and writes whole warp-wide runs.
__global__ void __launch_bounds__(256) k_reverse4(const float* __restrict__ in, long s0, long s1, long s2, long s3,
                                                  float* __restrict__ out) {
  __shared__ float tile[32][33];
  const long K = s2 * s3;
  const long k0 = (long)blockIdx.x * 32, r0 = (long)blockIdx.y * 32, i1 = blockIdx.z;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int r = ty; r < 32; r += 8) {
    const long i0 = r0 + r, k = k0 + tx;
    if (i0 < s0 && k < K) tile[r][tx] = in[(i0 * s1 + i1) * K + k];
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const long k = k0 + r, i0 = r0 + tx;
    if (i0 < s0 && k < K) {
      const long i2 = k / s3, i3 = k - i2 * s3;
      out[((i3 * s2 + i2) * s1 + i1) * s0 + i0] = tile[tx][r];
    }
  }
}

unsigned grid1d(long n) {
  long b = (n + 255) / 256;
  return (unsigned)(b < 4096 ? (b > 0 ? b : 1) : 4096);
}

}  // namespace

extern "C" {

int ffno_si_inputs(const float* features, const float* z_m, long V, const float* mean_x, const float* std_x,
                   float* x, float* z_mm, int* flags, ffno_stream_t stream) {
  if (!features || !z_m || !mean_x || !std_x || !x || !z_mm || !flags || V < 1) return FFNO_EINVAL;
  k_si_inputs<<<grid1d(V), 256, 0, (cudaStream_t)stream>>>(features, z_m, V, mean_x, std_x, x, z_mm, flags);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_si_populations(const float* y, long V, int L, const float* mean_y, const float* std_y, float* pop,
                        int* flags, ffno_stream_t stream) {
  if (!y || !mean_y || !std_y || !pop || !flags || V < 1 || L < 1) return FFNO_EINVAL;
  k_si_populations<<<grid1d(V), 256, 0, (cudaStream_t)stream>>>(y, V, L, mean_y, std_y, pop, flags);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_si_population_cotangent(const float* y, const float* pop_bar, long V, int L, const float* mean_y,
                                 const float* std_y, float* y_bar, int* flags, ffno_stream_t stream) {
  if (!y || !pop_bar || !mean_y || !std_y || !y_bar || !flags || V < 1 || L < 1) return FFNO_EINVAL;
  k_si_population_cotangent<<<grid1d(V), 256, 0, (cudaStream_t)stream>>>(y, pop_bar, V, L, mean_y, std_y, y_bar,
                                                                         flags);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_si_input_grads(const float* features, const float* x_bar, const float* z_bar_mm, long V, const float* std_x,
                        float* features_bar, float* z_bar_m, int* flags, ffno_stream_t stream) {
  if (!features || !x_bar || !z_bar_mm || !std_x || !features_bar || !z_bar_m || !flags || V < 1) return FFNO_EINVAL;
  k_si_input_grads<<<grid1d(V), 256, 0, (cudaStream_t)stream>>>(features, x_bar, z_bar_mm, V, std_x, features_bar,
                                                                z_bar_m, flags);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_reverse_axes4(const float* in, long s0, long s1, long s2, long s3, float* out, ffno_stream_t stream) {
  if (!in || !out || in == out || s0 < 1 || s1 < 1 || s2 < 1 || s3 < 1) return FFNO_EINVAL;
  const long kt = (s2 * s3 + 31) / 32, rt = (s0 + 31) / 32;
  if (kt > 0x7fffffffL || rt > 65535 || s1 > 65535) return FFNO_EINVAL;
  k_reverse4<<<dim3((unsigned)kt, (unsigned)rt, (unsigned)s1), 256, 0, (cudaStream_t)stream>>>(in, s0, s1, s2, s3, out);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

// Strided host <-> device block copy (rows of width bytes, each pitch apart on either side) on a stream: the slab and
// row-slab transfers of the host-RAM streaming forward (ffno_batched_backend.py:147-157 moves the same blocks with
// tensor slicing).
int ffno_copy2d(void* dst, long dpitch, const void* src, long spitch, long width, long rows, ffno_stream_t stream) {
  if (!dst || !src || width < 0 || rows < 0 || dpitch < width || spitch < width) return FFNO_EINVAL;
  if (!width || !rows) return FFNO_OK;
  if (cudaMemcpy2DAsync(dst, (size_t)dpitch, src, (size_t)spitch, (size_t)width, (size_t)rows, cudaMemcpyDefault,
                        (cudaStream_t)stream) != cudaSuccess)
    return FFNO_ELAUNCH;
  return FFNO_OK;
}

}  // extern "C"
