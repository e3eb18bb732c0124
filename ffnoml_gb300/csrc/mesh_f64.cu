// Population-mesh maps in FP64 (FFNOInversion.jl/src/PopulationMesh.jl): a log-tau column's atmosphere interpolated
// onto the height mesh the FFNO runs on, and the mesh populations interpolated back to the column's heights, with
// the transposes (VJP) and tangents (JVP) of both maps. The reference runs these per column on the host; here a
// thread takes a (column, mesh point) or a (column, height) pair, and the scatters of the transposes take a whole
// column per thread, in the reference's loop order, so every sum is deterministic.
//
// Layouts (the reference's column-major Julia arrays read row-major; col = x + nx y):
//   atm [6][ncol][nz]  T, vx, vy, vz, log10 ne, log10 rho (the service's features); z [ncol][nz] heights, top first
//   mesh [nm]          heights, top first;           f, fm_bar, fm_dot [ncol][nm][6]  T, vx, vy, vz, log10 ne, log10 rho
//   kind [ncol][nm]    0 inside, 1 above the top (values held), 2 below the bottom, 3 corona (left to the caller)
//   pm, pm_bar, pm_dot [L][ncol][nm];  pop, pop_bar, pop_dot [L][ncol][nz];  feature_bar / feature_dot [ncol][nz][6]
// Points below a column's bottom (and above its top when a corona temperature is set) follow hydrostatic
// extensions on the HSEMHS equation-of-state table (PopulationMesh.jl:122-180); the kernels mark them and leave their
// features, and their share of the transposes, to the caller.
#include <math.h>

#include "common.cuh"

namespace {

// interpolation variables of point k: ln T, vx, vy, vz, log10 ne, log10 rho (PopulationMesh.jl:182-190)
__device__ __forceinline__ double var(const double* atm, long plane, long i, int c) {
  const double v = atm[c * plane + i];
  return c == 0 ? log(v) : v;
}

// (kind, k, w) of height zeta in column zc (top first): the smallest k with zc[k+1] <= zeta (PopulationMesh.jl:192-198)
__device__ __forceinline__ int locate(const double* zc, int nz, double zeta, int& k, double& w) {
  if (zeta >= zc[0]) {
    k = 0;
    w = 0.0;
    return 1;
  }
  if (zeta < zc[nz - 1]) {
    k = nz - 1;
    w = 0.0;
    return 2;
  }
  int lo = 0, hi = nz - 2;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (zc[mid + 1] <= zeta)
      hi = mid;
    else
      lo = mid + 1;
  }
  k = lo;
  w = (zc[k] - zeta) / (zc[k] - zc[k + 1]);
  return 0;
}

// (j0, j1, u) with mesh[j0] >= zeta >= mesh[j1], clamped to the ends (PopulationMesh.jl:335-341)
__device__ __forceinline__ void bracket(const double* mesh, int nm, double zeta, int& j0, int& j1, double& u) {
  if (zeta >= mesh[0]) {
    j0 = j1 = 0;
    u = 0.0;
    return;
  }
  if (zeta <= mesh[nm - 1]) {
    j0 = j1 = nm - 1;
    u = 0.0;
    return;
  }
  int lo = 0, hi = nm - 1;   // the last j with mesh[j] >= zeta
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (mesh[mid] >= zeta)
      lo = mid;
    else
      hi = mid - 1;
  }
  j0 = lo;
  j1 = lo + 1;
  u = (mesh[j0] - zeta) / (mesh[j0] - mesh[j1]);
}

__device__ __forceinline__ int point_kind(int kd, bool corona, double zeta, double ztop) {
  return (kd == 1 && corona && zeta > ztop) ? 3 : kd;
}

__global__ void k_mesh_features(const double* __restrict__ atm, const double* __restrict__ z, long ncol, int nz,
                                const double* __restrict__ mesh, int nm, int corona, double* __restrict__ f,
                                int8_t* __restrict__ kind) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncol * nm) return;
  const long col = i / nm;
  const int m = (int)(i % nm);
  const double* zc = z + col * nz;
  int k;
  double w;
  const int kd = point_kind(locate(zc, nz, mesh[m], k, w), corona != 0, mesh[m], zc[0]);
  kind[i] = (int8_t)kd;
  double* o = f + i * 6;
  const long plane = ncol * nz, base = col * nz;
  for (int c = 0; c < 6; ++c) {
    double v = 0.0;
    if (kd == 1)
      v = var(atm, plane, base, c);
    else if (kd == 0)
      v = (1 - w) * var(atm, plane, base + k, c) + w * var(atm, plane, base + k + 1, c);
    o[c] = (c == 0 && kd <= 1) ? exp(v) : v;
  }
}

__global__ void k_mesh_features_jvp(const double* __restrict__ atm, const double* __restrict__ z, long ncol, int nz,
                                    const double* __restrict__ mesh, int nm, int corona, const double* __restrict__ f,
                                    const double* __restrict__ fd, double* __restrict__ out) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncol * nm) return;
  const long col = i / nm;
  const int m = (int)(i % nm);
  const double* zc = z + col * nz;
  int k;
  double w;
  const int kd = point_kind(locate(zc, nz, mesh[m], k, w), corona != 0, mesh[m], zc[0]);
  double* o = out + i * 6;
  const long base = col * nz;
  // tangents of (ln T, v, log10 ne, log10 rho) at point kk
  auto ad = [&](int c, int kk) {
    const double t = fd[(base + kk) * 6 + c];
    return c == 0 ? t / atm[base + kk] : t;
  };
  for (int c = 0; c < 6; ++c) {
    double v = 0.0;
    if (kd == 1)
      v = ad(c, 0);
    else if (kd == 0)
      v = (1 - w) * ad(c, k) + w * ad(c, k + 1);
    o[c] = (c == 0 && kd <= 1) ? v * f[i * 6] : v;
  }
}

// one thread per column: the transpose of the interpolation in mesh-point order (PopulationMesh.jl:522-541, 567-573)
__global__ void k_mesh_features_vjp(const double* __restrict__ atm, const double* __restrict__ z, long ncol, int nz,
                                    const double* __restrict__ mesh, int nm, int corona, const double* __restrict__ f,
                                    const double* __restrict__ fb, double* __restrict__ fbar,
                                    double* __restrict__ z_bar) {
  const long col = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const double* zc = z + col * nz;
  const long plane = ncol * nz, base = col * nz;
  double* ab = fbar + base * 6;        // accumulates a_bar [k][c], converted to feature_bar at the end
  double* zb = z_bar + base;
  for (int e = 0; e < nz * 6; ++e) ab[e] = 0.0;
  for (int k = 0; k < nz; ++k) zb[k] = 0.0;
  for (int m = 0; m < nm; ++m) {
    int k;
    double w;
    const int kd = point_kind(locate(zc, nz, mesh[m], k, w), corona != 0, mesh[m], zc[0]);
    if (kd >= 2) continue;
    const double* g = fb + (col * nm + m) * 6;
    const double f0 = f[(col * nm + m) * 6];
    if (kd == 1) {
      for (int c = 0; c < 6; ++c) ab[c] += g[c] * (c == 0 ? f0 : 1.0);
      continue;
    }
    double w_bar = 0.0;
    for (int c = 0; c < 6; ++c) {
      const double G = g[c] * (c == 0 ? f0 : 1.0);
      ab[k * 6 + c] += G * (1 - w);
      ab[(k + 1) * 6 + c] += G * w;
      w_bar += G * (var(atm, plane, base + k + 1, c) - var(atm, plane, base + k, c));
    }
    const double d = zc[k] - zc[k + 1];
    zb[k] += w_bar * (1 - w) / d;
    zb[k + 1] += w_bar * w / d;
  }
  for (int k = 0; k < nz; ++k) ab[k * 6] /= atm[base + k];
}

__global__ void k_mesh_backmap(const double* __restrict__ pm, const double* __restrict__ mesh, int nm,
                               const double* __restrict__ z, long ncol, int nz, int L, double* __restrict__ out) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncol * nz) return;
  const long col = i / nz;
  int j0, j1;
  double u;
  bracket(mesh, nm, z[i], j0, j1, u);
  for (int l = 0; l < L; ++l) {
    const double* p = pm + ((long)l * ncol + col) * nm;
    out[(long)l * ncol * nz + i] = exp((1 - u) * log(p[j0]) + u * log(p[j1]));
  }
}

__global__ void k_mesh_backmap_jvp(const double* __restrict__ pm, const double* __restrict__ pm_dot,
                                   const double* __restrict__ mesh, int nm, const double* __restrict__ z, long ncol,
                                   int nz, int L, double* __restrict__ out) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncol * nz) return;
  const long col = i / nz;
  int j0, j1;
  double u;
  bracket(mesh, nm, z[i], j0, j1, u);
  for (int l = 0; l < L; ++l) {
    const long o = ((long)l * ncol + col) * nm;
    const double p = exp((1 - u) * log(pm[o + j0]) + u * log(pm[o + j1]));
    out[(long)l * ncol * nz + i] = p * ((1 - u) * pm_dot[o + j0] / pm[o + j0] + u * pm_dot[o + j1] / pm[o + j1]);
  }
}

// one thread per column, heights ascending then levels (PopulationMesh.jl:371-381)
__global__ void k_mesh_backmap_vjp(const double* __restrict__ pm, const double* __restrict__ mesh, int nm,
                                   const double* __restrict__ z, long ncol, int nz, int L,
                                   const double* __restrict__ pop_bar, double* __restrict__ pm_bar,
                                   double* __restrict__ z_bar) {
  const long col = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  for (int l = 0; l < L; ++l)
    for (int m = 0; m < nm; ++m) pm_bar[((long)l * ncol + col) * nm + m] = 0.0;
  for (int k = 0; k < nz; ++k) {
    const long i = col * nz + k;
    int j0, j1;
    double u;
    bracket(mesh, nm, z[i], j0, j1, u);
    double zb = 0.0;
    for (int l = 0; l < L; ++l) {
      const long o = ((long)l * ncol + col) * nm;
      const double lp0 = log(pm[o + j0]), lp1 = log(pm[o + j1]);
      const double g = pop_bar[(long)l * ncol * nz + i] * exp((1 - u) * lp0 + u * lp1);
      pm_bar[o + j0] += g * (1 - u) / pm[o + j0];
      pm_bar[o + j1] += g * u / pm[o + j1];
      if (j0 != j1) zb -= g * (lp1 - lp0) / (mesh[j0] - mesh[j1]);
    }
    z_bar[i] = zb;
  }
}

unsigned blocks_for(long n) { return (unsigned)((n + 255) / 256); }

bool dims_ok(long ncol, int nz, int nm) {
  return ncol >= 1 && nz >= 2 && nm >= 1 && ncol * (long)(nz > nm ? nz : nm) < (long)0x7fffffff * 256L;
}

}  // namespace

extern "C" {

int ffno_mesh_features(const double* atm, const double* z, long ncol, int nz, const double* mesh, int nm, int corona,
                       double* f, int8_t* kind, ffno_stream_t stream) {
  if (!atm || !z || !mesh || !f || !kind || !dims_ok(ncol, nz, nm)) return FFNO_EINVAL;
  k_mesh_features<<<blocks_for(ncol * nm), 256, 0, (cudaStream_t)stream>>>(atm, z, ncol, nz, mesh, nm, corona, f,
                                                                             kind);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_mesh_features_jvp(const double* atm, const double* z, long ncol, int nz, const double* mesh, int nm,
                           int corona, const double* f, const double* feature_dot, double* fm_dot,
                           ffno_stream_t stream) {
  if (!atm || !z || !mesh || !f || !feature_dot || !fm_dot || !dims_ok(ncol, nz, nm)) return FFNO_EINVAL;
  k_mesh_features_jvp<<<blocks_for(ncol * nm), 256, 0, (cudaStream_t)stream>>>(atm, z, ncol, nz, mesh, nm, corona, f,
                                                                                 feature_dot, fm_dot);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_mesh_features_vjp(const double* atm, const double* z, long ncol, int nz, const double* mesh, int nm,
                           int corona, const double* f, const double* fm_bar, double* feature_bar, double* z_bar,
                           ffno_stream_t stream) {
  if (!atm || !z || !mesh || !f || !fm_bar || !feature_bar || !z_bar || !dims_ok(ncol, nz, nm)) return FFNO_EINVAL;
  k_mesh_features_vjp<<<blocks_for(ncol), 256, 0, (cudaStream_t)stream>>>(atm, z, ncol, nz, mesh, nm, corona, f,
                                                                            fm_bar, feature_bar, z_bar);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_mesh_backmap(const double* pm, const double* mesh, int nm, const double* z, long ncol, int nz, int L,
                      double* pop, ffno_stream_t stream) {
  if (!pm || !mesh || !z || !pop || L < 1 || !dims_ok(ncol, nz, nm)) return FFNO_EINVAL;
  k_mesh_backmap<<<blocks_for(ncol * nz), 256, 0, (cudaStream_t)stream>>>(pm, mesh, nm, z, ncol, nz, L, pop);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_mesh_backmap_jvp(const double* pm, const double* pm_dot, const double* mesh, int nm, const double* z,
                          long ncol, int nz, int L, double* pop_dot, ffno_stream_t stream) {
  if (!pm || !pm_dot || !mesh || !z || !pop_dot || L < 1 || !dims_ok(ncol, nz, nm)) return FFNO_EINVAL;
  k_mesh_backmap_jvp<<<blocks_for(ncol * nz), 256, 0, (cudaStream_t)stream>>>(pm, pm_dot, mesh, nm, z, ncol, nz, L,
                                                                                pop_dot);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_mesh_backmap_vjp(const double* pm, const double* mesh, int nm, const double* z, long ncol, int nz, int L,
                          const double* pop_bar, double* pm_bar, double* z_bar, ffno_stream_t stream) {
  if (!pm || !mesh || !z || !pop_bar || !pm_bar || !z_bar || L < 1 || !dims_ok(ncol, nz, nm)) return FFNO_EINVAL;
  k_mesh_backmap_vjp<<<blocks_for(ncol), 256, 0, (cudaStream_t)stream>>>(pm, mesh, nm, z, ncol, nz, L, pop_bar,
                                                                           pm_bar, z_bar);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

}  // extern "C"
