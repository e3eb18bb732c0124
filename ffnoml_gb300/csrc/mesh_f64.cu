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

// ------------------------------------------------------------------------------------------------ adaptive mesh
// The spacing each probe interval needs (adaptive_population_mesh, FFNOInversion.jl/src/PopulationMesh.jl:213-262):
// for column c and interval i of features f [ncol][n][6] (T, v, log10 ne, log10 rho on probe heights dz apart),
// r = max(|ln(T_i / T_{i+1})| / lnT_step, |d log10 ne| / log_ne_step, |d log10 rho| / log_rho_step, |d v| / v_step),
// and need[i] = min(need[i], dz / r) over the columns with r > 0. The minimum of positive doubles is taken on their
// bit patterns (which order as the values), so the result does not depend on the order of the columns.
__global__ void k_mesh_refine(const double* __restrict__ f, long ncol, int n, double dz, double lnT_step,
                              double ne_step, double rho_step, double v_step, unsigned long long* __restrict__ need) {
  const long total = ncol * (long)(n - 1);
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < total; e += (long)gridDim.x * blockDim.x) {
    const long col = e / (n - 1);
    const int i = (int)(e - col * (n - 1));
    const double* a = f + (col * n + i) * 6;
    const double* b = a + 6;
    double r = fabs(log(a[0] / b[0])) / lnT_step;
    r = fmax(r, fabs(a[4] - b[4]) / ne_step);
    r = fmax(r, fabs(a[5] - b[5]) / rho_step);
    for (int v = 1; v <= 3; ++v) r = fmax(r, fabs(a[v] - b[v]) / v_step);
    if (r > 0.0) atomicMin(need + i, (unsigned long long)__double_as_longlong(dz / r));
  }
}

// ------------------------------------------------------------------------------------------------ inclined views
// The periodic bilinear shear of an inclined view between Cartesian mesh columns and the footprint rays
// (FFNOInversion.jl/src/ViewAngle.jl:93-145): level k of A [nz][nx][ny] is read at the fractional cell offset
// (i0[k] + wx[k], j0[k] + wy[k]), the same for every cell of the level:
//   out[k][i][j] = (1 - wy)((1 - wx) A[k][ia][ja] + wx A[k][ib][ja]) + wy((1 - wx) A[k][ia][jb] + wx A[k][ib][jb]),
//   ia = (i + i0) mod nx, ib = (ia + 1) mod nx, ja = (j + j0) mod ny, jb = (ja + 1) mod ny.
// Its transpose (ViewAngle.jl:147-162, a scatter there) is a gather here, one thread per output value and no atomics:
//   out[k][p][q] = (1 - wy)(1 - wx) A[k][p - i0][q - j0] + (1 - wy) wx A[k][p - 1 - i0][q - j0]
//                + wy (1 - wx) A[k][p - i0][q - 1 - j0] + wy wx A[k][p - 1 - i0][q - 1 - j0]   (indices mod nx, ny).
__device__ __forceinline__ long pmod(long a, long n) {
  const long r = a % n;
  return r < 0 ? r + n : r;
}

__global__ void k_shear_levels(const double* __restrict__ A, int nz, long nx, long ny, const int* __restrict__ i0,
                               const int* __restrict__ j0, const double* __restrict__ wx,
                               const double* __restrict__ wy, int transpose, double* __restrict__ out) {
  const long n = (long)nz * nx * ny;
  for (long e = blockIdx.x * (long)blockDim.x + threadIdx.x; e < n; e += (long)gridDim.x * blockDim.x) {
    const long j = e % ny, t = e / ny, i = t % nx;
    const int k = (int)(t / nx);
    const double ax = wx[k], ay = wy[k];
    const double* a = A + (long)k * nx * ny;
    double v;
    if (!transpose) {
      const long ia = pmod(i + i0[k], nx), ib = (ia + 1) % nx, ja = pmod(j + j0[k], ny), jb = (ja + 1) % ny;
      v = (1.0 - ay) * ((1.0 - ax) * a[ia * ny + ja] + ax * a[ib * ny + ja]) +
          ay * ((1.0 - ax) * a[ia * ny + jb] + ax * a[ib * ny + jb]);
    } else {
      const long pa = pmod(i - i0[k], nx), pb = pmod(i - 1 - i0[k], nx), qa = pmod(j - j0[k], ny),
                 qb = pmod(j - 1 - j0[k], ny);
      v = (1.0 - ay) * ((1.0 - ax) * a[pa * ny + qa] + ax * a[pb * ny + qa]) +
          ay * ((1.0 - ax) * a[pa * ny + qb] + ax * a[pb * ny + qb]);
    }
    out[e] = v;
  }
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

int ffno_shear_levels(const double* A, int nz, long nx, long ny, const int* i0, const int* j0, const double* wx,
                      const double* wy, int transpose, double* out, ffno_stream_t stream) {
  if (!A || !i0 || !j0 || !wx || !wy || !out || A == out || nz < 1 || nx < 1 || ny < 1) return FFNO_EINVAL;
  const long n = (long)nz * nx * ny;
  const long blocks = (n + 255) / 256 < 8L * 152 ? (n + 255) / 256 : 8L * 152;
  k_shear_levels<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(A, nz, nx, ny, i0, j0, wx, wy, transpose, out);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

int ffno_mesh_refine(const double* f, long ncol, int n, double dz, double lnT_step, double log_ne_step,
                     double log_rho_step, double velocity_step, double* need, ffno_stream_t stream) {
  if (!f || !need || ncol < 1 || n < 2 || !(dz > 0) || !(lnT_step > 0) || !(log_ne_step > 0) || !(log_rho_step > 0) ||
      !(velocity_step > 0))
    return FFNO_EINVAL;
  const long total = ncol * (long)(n - 1);
  const long blocks = (total + 255) / 256 < 8L * 152 ? (total + 255) / 256 : 8L * 152;
  k_mesh_refine<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(f, ncol, n, dz, lnT_step, log_ne_step, log_rho_step,
                                                                    velocity_step,
                                                                    reinterpret_cast<unsigned long long*>(need));
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}

}  // extern "C"
