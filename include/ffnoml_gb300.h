/* ffnoml_gb300 — C ABI of the GB300 (sm_103a) FFNO3D forward and input-VJP kernels.
 *
 * The reference (harshmathur1990/FFNOML) exposes this path only as the PyTorch module FFNO3D
 * (models/ffno_model.py:614-832) behind ffno_model_factory.create_ffno3d (ffno_model_factory.py:6-19) and the
 * protocol-v2 service (ffno_fsdp_service.py). Each entry point below replaces one stage of FFNO3D.forward / its
 * autograd backward; the comment on each names the reference code it stands for. The Python host code in
 * ffnoml_gb300/ (module, executor, service) calls these through ctypes.
 *
 * Conventions
 *  - Every pointer is a device pointer unless noted; every call is asynchronous on `stream` (a cudaStream_t, NULL =
 *    legacy default stream) and allocates nothing: all workspace is passed in by the caller.
 *  - Activations are channels-last: one contiguous row of C floats per voxel, voxel v = (d*H + h)*W + w of one cube,
 *    V = D*H*W voxels. The model input x_in and the output are channels-first [channels][V], as FFNO3D's [B,C,D,H,W].
 *  - Weight matrices are row-major [K][N] (input channel k, output channel n): the transpose of a Conv3d weight
 *    [N][K][1][1][1].
 *  - GroupNorm coefficients `coefs` are [3][C] floats: per channel the group mean, gamma*rstd and beta; the
 *    normalised value is (x - coefs[0][c]) * coefs[1][c] + coefs[2][c].
 *  - GroupNorm partial statistics `partials` are [nparts][groups][3] doubles (total weight, mean, M2), one row per
 *    CTA of the producing kernel, which is launched with exactly nparts CTAs.
 *  - Return value: FFNO_OK (0) or an error code; no call traps, aborts or throws.
 *  - Supported widths C: 16, 32, 64, 96.
 */
#ifndef FFNOML_GB300_H
#define FFNOML_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FFNO_OK 0
#define FFNO_EINVAL 1      /* unsupported size, null pointer, inconsistent arguments */
#define FFNO_ELAUNCH 2     /* a kernel launch failed (cudaGetLastError) */
#define FFNO_ENOMEM 3      /* the caller's workspace is too small */
#define FFNO_ETIMEOUT 4    /* a bounded device wait ran out */
#define FFNO_ETOOBIG 5     /* the request exceeds the fixed capacity of a non-allocating entry point */

typedef void* ffno_stream_t; /* cudaStream_t */

/* Level-fraction head constants (FFNO3D.head_output, models/ffno_model.py:730-749; MULTI3D tables :116-141). */
#define FFNO_MAX_LEVELS 32
#define FFNO_MAX_SPECIES 4
typedef struct {
  int nspecies;
  int levels[FFNO_MAX_SPECIES];
  int rho_channel, temperature_channel, ne_channel;
  int in_channels;
  float total_bound;
  float log10_particle_mass[FFNO_MAX_SPECIES];
  float mean_x[8], std_x[8];
  float mean_y[FFNO_MAX_LEVELS], std_y[FFNO_MAX_LEVELS];
  double log_g[FFNO_MAX_LEVELS], ev[FFNO_MAX_LEVELS], ndxi[FFNO_MAX_LEVELS], dion[FFNO_MAX_LEVELS];
  int math32; /* nonzero: the LTE weights and log-softmax in FP32 with a compensated (Neumaier) sum of the level
                 exponentials, so that a voxel's level shares add up to 1 within 1e-6 (the split-BF16 path);
                 0: all of it in FP64, as the reference computes it */
} ffno_head_params;

/* library version string */
const char* ffno_version(void);

/* Number of CTAs the statistics-producing kernels use for V voxels (= nparts of their partials). */
int ffno_stats_parts(long V);

/* depth_weights (models/ffno_model.py:28-34, 67-74): z [D][HW] heights (any units) -> w [D][HW] trapezoid |dz| over
 * the column mean. */
int ffno_depth_weights(const float* z, int D, long HW, float* w, ffno_stream_t stream);

/* Column analysis for HeightSpectralConv.box/shared-grid check (models/ffno_model.py:248-259, 266-269): out[0] = 1.0f
 * if every column shifted by its own minimum equals column 0 shifted by its minimum (exact float equality), else 0;
 * out[1] = the largest column span max - min. out is 2 floats of device memory. */
int ffno_column_info(const float* z, int D, long HW, float* out, ffno_stream_t stream);

/* lift: pre = x_in (channels-first [cin][V]) @ w_lift [cin][C] (FFNO3D.lift[0], models/ffno_model.py:688-692),
 * with the depth-weighted GroupNorm partials of pre (lift[1]). */
int ffno_lift_fwd(const float* x_in, int cin, long V, int C, const float* w_lift, const float* dw, float* pre,
                  double* partials, int nparts, int groups, ffno_stream_t stream);

/* DepthWeightedGroupNorm statistics (models/ffno_model.py:77-95): partials -> coefs [3][C] and, if gstats is not
 * NULL, gstats [groups][3] doubles (mean, rstd, total weight T). */
int ffno_gn_finalize(const double* partials, int nparts, int C, int groups, const float* gamma, const float* beta,
                     float eps, float* coefs, double* gstats, ffno_stream_t stream);

/* out = act(GroupNorm(pre)), act 0 = identity, 1 = GELU (lift[1:3], models/ffno_model.py:782-783). */
int ffno_gn_act(const float* pre, const float* coefs, long V, int C, int act, float* out, ffno_stream_t stream);

/* Input gate of both branches (SpectralConv2dFull.input_gate :336-341, HeightSpectralConv.input_gate :205-210 and
 * z_proj :211, :265): out = x * sigmoid(gelu(x @ w1) @ w2) [+ zp[c] * z[v]] (zp, z may be NULL). */
int ffno_gate_fwd(const float* x, long V, int C, const float* w1, const float* w2, const float* zp, const float* z,
                  float* out, ffno_stream_t stream);

/* Pointwise 2-layer MLP C -> 2C -> C (post :367-373, :221-225; pw :489-493; mlp :495) with a residual prologue and
 * the GroupNorm partials of its output:
 *   mode 0: a = in
 *   mode 1: a = in + res * gelu(GN(prev_pre))    (x1 = x + res_fused * fused, :545)
 *   mode 2: a = in + res * GN(prev_pre)          (x2 = x1 + res_pw * pw, :548)
 * modes 1 and 2 also write a to xout. pre = gelu(a @ w1) @ w2. */
int ffno_mlp2_fwd(int mode, const float* in, const float* prev_pre, const float* prev_coefs, float res, float* xout,
                  long V, int C, const float* w1, const float* w2, const float* dw, float* pre, double* partials,
                  int nparts, int groups, ffno_stream_t stream);

/* Branch gate + fuse (FFNOBlock3dBalanced._fuse_branches, models/ffno_model.py:524-534) on
 * spec = gelu(GN_spec(spec_pre)), vert = gelu(GN_vert(vert_pre)):
 *   gates = sigmoid(gelu([x, spec, vert] @ wg1) @ wg2 + bg2); smix = spec*gates[:C]; vmix = vert*gates[C:]
 *   pre = gelu([smix, vmix] @ wf1) @ wf2 + 0.5 (smix + vmix), with the GroupNorm partials of pre. */
int ffno_fuse_fwd(const float* x, const float* spec_pre, const float* spec_coefs, const float* vert_pre,
                  const float* vert_coefs, long V, int C, const float* wg1, const float* wg2, const float* bg2,
                  const float* wf1, const float* wf2, const float* dw, float* pre, double* partials, int nparts,
                  int groups, ffno_stream_t stream);

/* Block output out = x2 + res * GN(pre) (models/ffno_model.py:550-551). */
int ffno_resid_out(const float* x2, const float* pre, const float* coefs, float res, long V, int C, float* out,
                   ffno_stream_t stream);

/* Projection + level-fraction head (FFNO3D._run_head + head_output, models/ffno_model.py:790-798, 730-749):
 * h = gelu(x @ p1) @ p2 + b2 (p2, b2 padded to nhp = 16 or 32 columns), then per voxel the MULTI3D LTE weights of
 * T, ne from x_in, per-species log-softmax and total correction -> out channels-first [levels][V], normalised
 * log10 n. If head_out is not NULL the raw head channels are also written there channels-first [nh][V]. */
int ffno_head_fwd(const float* x, const float* x_in, long V, int C, const float* p1, const float* p2, const float* b2,
                  int nh, int nhp, const ffno_head_params* params, float* out, float* head_out, ffno_stream_t stream);

/* FFNO3D._run_head alone (models/ffno_model.py:790-798; the drop-in module's _run_head): head [nh][V] channels-first
 * = gelu(x @ p1) @ p2 + b2 for x [V][C]; p2, b2 padded to nhp = 16 or 32 columns, nh <= nhp. */
int ffno_proj_fwd(const float* x, long V, int C, const float* p1, const float* p2, const float* b2, int nh, int nhp,
                  float* head, ffno_stream_t stream);

/* FFNO3D.head_output (models/ffno_model.py:730-749) on head channels that are already computed: head [nh][V]
 * channels-first (per species its level logits, then its total channel), x_in [cin][V] the normalised inputs ->
 * out [levels][V] normalised log10 n. One thread per voxel: coalesced loads and stores of the channel planes. */
int ffno_head_output(const float* head, const float* x_in, long V, int nh, const ffno_head_params* params,
                     float* out, ffno_stream_t stream);

/* Batched transform GEMM: out[b][m][n] = sum_k T[m][k] * in[b][k][n], the DFT-as-contraction of both spectral
 * operators (rfft2/irfft2 of SpectralConv2dFull.forward :441-448; the Filon height transform and its inverse of
 * HeightSpectralConv.forward :270-275, :303-305). Batch b = b1 * nb2 + b2; a row index r of in (k) or out (m) is
 * addressed as (r / split) * s_hi + (r % split) * s_lo. n is contiguous. */
typedef struct {
  long nb, nb2;
  long in_b1, in_b2, out_b1, out_b2;
  int K, M;
  long N;
  int in_split;
  long in_hi, in_lo;
  int out_split;
  long out_hi, out_lo;
} ffno_xform_desc;
int ffno_xform(const float* T, const float* in, float* out, const ffno_xform_desc* desc, int accumulate,
               ffno_stream_t stream);
/* ffno_xform with a table per batch element: batch b uses T + b * t_b (b = b1 * nb2 + b2): the per-column Filon
 * transforms of HeightSpectralConv when the columns' height grids differ (models/ffno_model.py:276-280, 306-308). */
int ffno_xform_pt(const float* T, long t_b, const float* in, float* out, const ffno_xform_desc* desc, int accumulate,
                  ffno_stream_t stream);
/* Per-column table gradients: out [ncol][Ra][Rb] (double; = or +=) with out[col][i][j] = sum_c A[i][col][c] *
 * B[j][col][c], A and B laid [rows][ncol][C] with row stride row_stride floats; each sum over the C <= 512 channels
 * in FP32, added to out in FP64. */
int ffno_col_outer(const float* A, int Ra, const float* B, int Rb, long ncol, int C, long row_stride, double* out,
                   int accumulate, ffno_stream_t stream);

/* Per-frequency complex channel mixing (SpectralConv2dFull.mix_spectrum :394-429; HeightSpectralConv mode mixing
 * :282-300): for each frequency f < F and row b < nb, with xhat = re + i im at offset f*sf + b*sb (im at +s_im):
 *   out = g_f * (xhat @ (w_re + i w_im)) + U_f (V_f xhat)
 * wbig [2C][2C] = [[w_re, w_im], [-w_im, w_re]], g [F][2], U [F][C][rank], Vm [F][rank][C]. in and out must not
 * overlap. */
int ffno_spectral_mix(const float* in, float* out, long F, long nb, long sf, long sb, long s_im, int C,
                      const float* wbig, const float* g, const float* U, const float* Vm, int rank,
                      ffno_stream_t stream);

/* ------------------------------------------------------------------------------------------------------------------
 * Input VJP (the hand-written replacement of torch.autograd.backward through FFNO3D.forward under per-block
 * checkpointing, ffno_fsdp_runtime.py:306-348 and models/ffno_model.py:751-780). u is the gradient arriving at a
 * GroupNorm's consumer: mode 0 means dL/dy = r*u (y = GN(pre)), mode 1 means dL/dy = r*u*gelu'(y) (GELU after GN),
 * mode 2 the same with the tensor-core kernels' GELU (the normal CDF of Abramowitz & Stegun 7.1.26), for the
 * GroupNorms whose GELU the split-BF16 forward applied with it.
 * ------------------------------------------------------------------------------------------------------------------ */

/* Per-group sums S1 = sum ghat, S2 = sum ghat*xhat of the GroupNorm backward, ghat = dL/dy * gamma, as partials
 * [nparts][groups][2] doubles (one row per CTA; any nparts >= 1). */
int ffno_gn_bwd_stats(int mode, const float* u, float r, const float* pre, const float* gamma, const float* beta,
                      const double* gstats, long V, int C, int groups, double* partials, int nparts,
                      ffno_stream_t stream);
/* partials -> sums [groups][2] doubles (fixed order). */
int ffno_gn_bwd_final(const double* partials, int nparts, int groups, double* sums, ffno_stream_t stream);
/* pre_bar = rstd (ghat - (w/T)(S1 + xhat S2)); w_bar[v] += the depth-weight gradient of this GroupNorm's statistics.
 * u, pre and pre_bar 32-byte aligned for C <= 64 (16-byte for C = 96), FFNO_EINVAL otherwise. */
int ffno_gn_bwd_apply(int mode, const float* u, float r, const float* pre, const float* gamma, const float* beta,
                      const double* gstats, const double* sums, const float* dw, long V, int C, int groups, float eps,
                      float* pre_bar, float* w_bar, ffno_stream_t stream);

/* Backward of pre = gelu(a @ w1) @ w2 (the C -> 2C -> C MLPs): a_bar = base + ((pre_bar @ w2t) * gelu'(a @ w1)) @ w1t,
 * recomputing a @ w1; w2t [C][2C], w1t [2C][C] are the transposed weights; base may be NULL. */
int ffno_mlp2_bwd(const float* a, const float* pre_bar, const float* base, long V, int C, const float* w1,
                  const float* w2t, const float* w1t, float* a_bar, ffno_stream_t stream);

/* Backward of ffno_fuse_fwd given fused_pre_bar: x_bar = base + d/dx, spec_bar and vert_bar = gradients w.r.t.
 * spec = gelu(GN_spec(spec_pre)) and vert (before their GroupNorm backward). Transposed weights: wf2t [C][2C],
 * wf1t [2C][2C], wg2t [2C][C], wg1t [C][3C]. */
int ffno_fuse_bwd(const float* x, const float* spec_pre, const float* spec_coefs, const float* vert_pre,
                  const float* vert_coefs, const float* fused_pre_bar, const float* base, long V, int C,
                  const float* wg1, const float* wg2, const float* bg2, const float* wf1, const float* wf2t,
                  const float* wf1t, const float* wg2t, const float* wg1t, float* x_bar, float* spec_bar,
                  float* vert_bar, ffno_stream_t stream);

/* Backward of both input gates (ffno_gate_fwd): x_bar = base + gate_s'(xs_bar) + gate_v'(xv_bar);
 * z_bar[v] += sum_c xv_bar[v][c] * zp[c] (z_proj). */
int ffno_gate_bwd(const float* x, const float* xs_bar, const float* xv_bar, const float* base, long V, int C,
                  const float* s_w1, const float* s_w2, const float* s_w2t, const float* s_w1t, const float* v_w1,
                  const float* v_w2, const float* v_w2t, const float* v_w1t, const float* zp, float* x_bar,
                  float* z_bar, ffno_stream_t stream);

/* Backward of the lift convolution: x_in_bar [cin][V] += pre_bar @ w_lift^T. */
int ffno_lift_bwd(const float* pre_bar, int cin, long V, int C, const float* w_lift, float* x_in_bar,
                  ffno_stream_t stream);

/* Backward of ffno_head_fwd given y_bar [levels][V]: x_bar [V][C] (gradient of the last block's output) and the
 * head's direct input gradient x_in_bar [cin][V] (written, not accumulated: T, ne and rho channels). p2t [nhp][2C]
 * and p1t [2C][C] are the transposed, zero-padded projection weights. */
int ffno_head_bwd(const float* x, const float* x_in, const float* y_bar, long V, int C, const float* p1,
                  const float* p2, const float* b2, const float* p2t, const float* p1t, int nhp,
                  const ffno_head_params* params, float* x_bar, float* x_in_bar, ffno_stream_t stream);

/* VJP of ffno_proj_fwd: x_bar [V][C] (written) from head_bar [nh][V]; p2t [nhp][2C] and p1t [2C][C] as for
 * ffno_head_bwd. */
int ffno_proj_bwd(const float* x, const float* head_bar, long V, int C, const float* p1, const float* p2,
                  const float* b2, const float* p2t, const float* p1t, int nh, int nhp, float* x_bar,
                  ffno_stream_t stream);

/* VJP of ffno_head_output given y_bar [levels][V]: head_bar [nh][V] and x_in_bar [cin][V], both written (x_in_bar
 * is non-zero only on the T, ne and rho channels). */
int ffno_head_output_bwd(const float* head, const float* x_in, const float* y_bar, long V, int nh,
                         const ffno_head_params* params, float* head_bar, float* x_in_bar, ffno_stream_t stream);

/* Backward of ffno_depth_weights: z_bar [D][HW] += d w / d z applied to w_bar. */
int ffno_depth_weights_bwd(const float* z, const float* w_bar, int D, long HW, float* z_bar, ffno_stream_t stream);

/* out [Ma][Mb] (double; = or +=) = A [Ma][N] (row stride lda) @ B [Mb][N]^T (row stride ldb), split over N into
 * nsplit partial sums held in part [nsplit][Ma][Mb] floats and reduced in a fixed order: the gradients of the height
 * operator's transform tables. ffno_outer_parts gives the nsplit to use. A and B 16-byte aligned, lda and ldb
 * multiples of 4 (the rows are read as float4). */
int ffno_outer_parts(int Ma, int Mb, long N);
int ffno_outer(const float* A, long lda, int Ma, const float* B, long ldb, int Mb, long N, float* part, int nsplit,
               double* out, int accumulate, ffno_stream_t stream);

/* ffno_outer without a caller-provided scratch buffer. No counterpart in the reference: it exists for hosts that bind
 * this C ABI but cannot allocate device memory for the library on each call (their device memory belongs to their own
 * runtime's allocator, or they must not allocate after start-up). The partial sums live in a fixed 16 MiB array inside
 * the library (held on every GPU that loads it until the process exits), so Ma * Mb may be at most 4 Mi (4194304);
 * larger requests return FFNO_ETOOBIG without touching the device. Allocates nothing. The first call on each device
 * looks up the array's device address (with that device current); make that first call before any stream capture.
 * Every call shares the one array, so calls that overlap on the GPU (other streams, other threads) race; nothing in it
 * needs to start at zero. The result equals ffno_outer's with nsplit = ffno_outer_parts(Ma, Mb, N) bit for bit while
 * Ma * Mb * ffno_outer_parts(Ma, Mb, N) <= 4 Mi; above that the array holds fewer splits, so the partial sums are
 * added in another order (the same value to rounding, not the same bits). The looked-up address belongs to the
 * device's current context: after cudaDeviceReset on a device, do not call this entry point on it again in the same
 * process. */
int ffno_outer_noalloc(const float* A, long lda, int Ma, const float* B, long ldb, int Mb, long N, double* out,
                       int accumulate, ffno_stream_t stream);

/* ------------------------------------------------------------------------------------------------------------------
 * Service conversions (ffno_fsdp_runtime.py). flags is one device int, OR-ed: 1 non-finite input, 2 T <= 0,
 * 4 non-positive or non-finite population, 8 non-finite gradient.
 * ------------------------------------------------------------------------------------------------------------------ */

/* _model_inputs + normalisation (:48-58, :274-276): SI features [6][V] (T, vx, vy, vz, log10 ne, log10 rho) and z [V]
 * in metres -> normalised inputs x [6][V] and z_mm [V] in Mm. */
/* Population-mesh maps, FP64 (FFNOInversion.jl/src/PopulationMesh.jl:182-227 features, :335-360 back-map, :362-408
 * and :522-573 transposes, :427-518 tangents). atm [6][ncol][nz] = T, vx, vy, vz, log10 ne, log10 rho; z [ncol][nz]
 * and mesh [nm] decreasing (top first); f / fm_bar / fm_dot [ncol][nm][6]; kind [ncol][nm] (0 inside, 1 above the top,
 * values held, 2 below the bottom, 3 corona: features left to the caller's hydrostatic extension); pm [L][ncol][nm];
 * pop [L][ncol][nz]; feature_bar / feature_dot [ncol][nz][6]; z_bar [ncol][nz]. corona != 0: points above a column top
 * are corona points. */
int ffno_mesh_features(const double* atm, const double* z, long ncol, int nz, const double* mesh, int nm, int corona,
                       double* f, int8_t* kind, ffno_stream_t stream);
int ffno_mesh_features_vjp(const double* atm, const double* z, long ncol, int nz, const double* mesh, int nm,
                           int corona, const double* f, const double* fm_bar, double* feature_bar, double* z_bar,
                           ffno_stream_t stream);
int ffno_mesh_features_jvp(const double* atm, const double* z, long ncol, int nz, const double* mesh, int nm,
                           int corona, const double* f, const double* feature_dot, double* fm_dot,
                           ffno_stream_t stream);
int ffno_mesh_backmap(const double* pm, const double* mesh, int nm, const double* z, long ncol, int nz, int L,
                      double* pop, ffno_stream_t stream);
int ffno_mesh_backmap_vjp(const double* pm, const double* mesh, int nm, const double* z, long ncol, int nz, int L,
                          const double* pop_bar, double* pm_bar, double* z_bar, ffno_stream_t stream);
int ffno_mesh_backmap_jvp(const double* pm, const double* pm_dot, const double* mesh, int nm, const double* z,
                          long ncol, int nz, int L, double* pop_dot, ffno_stream_t stream);

/* The spacing each probe interval of an adaptive population mesh needs (FFNOInversion.jl/src/PopulationMesh.jl:
 * 213-262): f [ncol][n][6] the mesh features of every column on n probe heights dz apart (ffno_mesh_features);
 * need [n - 1] holds positive spacings (the maximum spacing) on entry and, on return, for each interval the minimum
 * over the columns of dz / r, r the largest of |ln(T ratio)| / lnT_step, |d log10 ne| / log_ne_step,
 * |d log10 rho| / log_rho_step and |d v| / velocity_step over the interval (columns with r = 0 leave it). */
int ffno_mesh_refine(const double* f, long ncol, int n, double dz, double lnT_step, double log_ne_step,
                     double log_rho_step, double velocity_step, double* need, ffno_stream_t stream);

/* Periodic bilinear shear of an inclined view between Cartesian mesh columns and footprint rays
 * (FFNOInversion.jl/src/ViewAngle.jl:93-162, used by PopulationMesh.jl:296-317): A and out [nz][nx][ny] FP64 (level k
 * a contiguous plane), per level the integer cell offsets i0, j0 [nz] and fractions wx, wy [nz] in [0, 1). transpose = 0:
 * out[k][i][j] = bilinear read of A at ((i + i0 + wx) mod nx, (j + j0 + wy) mod ny); transpose = 1: its transpose
 * (adjoint), written, not accumulated. A and out must not overlap. */
int ffno_shear_levels(const double* A, int nz, long nx, long ny, const int* i0, const int* j0, const double* wx,
                      const double* wy, int transpose, double* out, ffno_stream_t stream);

/* Reverses the four axes of an array: in C-order [s0][s1][s2][s3] -> out C-order [s3][s2][s1][s0], i.e. the same
 * array in Fortran order. The protocol's arrays (FFNOInversion.jl/src/FSDPService.jl: features (6, nz, nx, ny), z,
 * populations (nz, nx, ny, L), in Fortran order; ffno_fsdp_service.py:219-322) go between their wire layout and the
 * model's with it on the device. in and out must not overlap; s1 and ceil(s0 / 32) at most 65535. */
int ffno_reverse_axes4(const float* in, long s0, long s1, long s2, long s3, float* out, ffno_stream_t stream);

/* Host-RAM streaming (ffno_batched_backend.py:147-289): strided block copy between pinned host memory and the device,
 * rows of `width` bytes `spitch` / `dpitch` apart (cudaMemcpy2DAsync, direction from the addresses). */
int ffno_copy2d(void* dst, long dpitch, const void* src, long spitch, long width, long rows, ffno_stream_t stream);

int ffno_si_inputs(const float* features, const float* z_m, long V, const float* mean_x, const float* std_x,
                   float* x, float* z_mm, int* flags, ffno_stream_t stream);
/* linear_populations + _canonical_populations (:76-78, :277-292): normalised log10 n y [L][V] -> pop [V][L] m^-3. */
int ffno_si_populations(const float* y, long V, int L, const float* mean_y, const float* std_y, float* pop,
                        int* flags, ffno_stream_t stream);
/* VJP of ffno_si_populations: pop_bar [V][L] -> y_bar [L][V]. */
int ffno_si_population_cotangent(const float* y, const float* pop_bar, long V, int L, const float* mean_y,
                                 const float* std_y, float* y_bar, int* flags, ffno_stream_t stream);
/* VJP of ffno_si_inputs: x_bar [6][V], z_bar_mm [V] -> features_bar [6][V] (per K, per m/s, per dex), z_bar_m [V]. */
int ffno_si_input_grads(const float* features, const float* x_bar, const float* z_bar_mm, long V, const float* std_x,
                        float* features_bar, float* z_bar_m, int* flags, ffno_stream_t stream);

/* ------------------------------------------------------------------------------------------------------------------
 * Tensor-core (tcgen05) kernels in split-BF16: each GEMM operand x is carried as hi = bf16(x), lo = bf16(x - hi) and
 * each product as hi*hi + hi*lo + lo*hi on the BF16 tensor cores with FP32 accumulation in tensor memory. FP32
 * activations and statistics in HBM, so each has the contract of the FP32 entry point (or stage) it names. Weights
 * come pre-packed in `wpack` (16-byte aligned): for each matrix, in the order listed, its hi then its lo half, each
 * [R][K] BF16 in the canonical K-major core-matrix order (8 x 8 blocks; the 8 rows of a block 16 bytes apart; the
 * K-blocks of one 8-row group 128 bytes apart; row groups K*16 bytes apart). The matrix of a GEMM out = in @ M^T is
 * M [out][in] (a Conv3d weight, or a transposed one in the backward). err: one device int, set non-zero if a bounded
 * wait ran out. Widths C = 16, 32, 64. Statistics partials: nparts = ffno_tc_parts(V).
 * ------------------------------------------------------------------------------------------------------------------ */
int ffno_tc_parts(long V);
int ffno_tc_width_supported(int C);
/* Widths of ffno_mlp2_fwd_tc / ffno_mlp2_bwd_tc and ffno_gate_fwd_tc / ffno_gate_bwd_tc: also C = 96, the production
 * model's width (the channel MLPs and input gates there run on tensor cores while the fusion, mixing and head keep
 * their FP32 entry points). */
int ffno_tc_channel_width_supported(int C);
/* L2 prefetch lookahead of the tensor-core pointwise kernels on the current device, in tiles of 128 voxels per
 * pipeline (0..4; default 0): a tuning knob, synchronous, not to be called while those kernels run. */
int ffno_tc_set_prefetch_tiles(int tiles);

/* ffno_mlp2_fwd; wpack = [w1 (2C x C), w2 (C x 2C)]. C = 96 also (in, pre, prev_pre, xout 32-byte aligned). */
int ffno_mlp2_fwd_tc(int mode, const float* in, const float* prev_pre, const float* prev_coefs, float res, float* xout,
                     long V, int C, const void* wpack, const float* dw, float* pre, double* partials, int nparts,
                     int groups, int* err, ffno_stream_t stream);
/* ffno_gate_fwd for one branch; wpack = [g1, g2] (C x C). C = 96 also (x 32-byte aligned). */
int ffno_gate_fwd_tc(const float* x, long V, int C, const void* wpack, const float* zp, const float* z, float* out,
                     int* err, ffno_stream_t stream);
/* First stage of ffno_fuse_fwd: gates [V][2C] = sigmoid(gelu([x, spec, vert] wg1^T) wg2^T + bias), and (if hg is not
 * NULL) the hidden pre-activation hg [V][C]; wpack = [wg1 (C x 3C), wg2 (2C x C)]. C = 96 also (rows 32-byte
 * aligned). */
int ffno_fuse1_tc(const float* x, const float* spec_pre, const float* spec_coefs, const float* vert_pre,
                  const float* vert_coefs, long V, int C, const void* wpack, const float* bias, float* gates,
                  float* hg, int* err, ffno_stream_t stream);
/* Second stage of ffno_fuse_fwd: pre = gelu(B wf1^T) wf2^T + (B[:, :C] + B[:, C:]) / 2, B = [spec gs, vert gv], with
 * GroupNorm partials; wpack = [wf1 (2C x 2C), wf2 (C x 2C)]. */
int ffno_fuse2_tc(const float* spec_pre, const float* spec_coefs, const float* vert_pre, const float* vert_coefs,
                  const float* gates, long V, int C, const void* wpack, const float* dw, float* pre, double* partials,
                  int nparts, int groups, int* err, ffno_stream_t stream);
/* The branch fusion at C = 96 (ffno_fuse_fwd / ffno_fuse_bwd, models/ffno_model.py:524-534), whose weights exceed
 * shared memory for the two-stage form: ffno_fuse1_tc (C = 96 also) for the gates and hg, then
 *   ffno_fuse_hidden_tc: hf [V][2C] = B wf1^T, B = [gelu(GN_s(spec_pre)) g_s, gelu(GN_v(vert_pre)) g_v]; wpack = [wf1
 *     (2C x 2C)];
 *   ffno_fuse_out_tc: pre [V][C] = gelu(hf) wf2^T + (B_s + B_v) / 2 with GroupNorm partials (nparts =
 *     ffno_tc_parts(V)); wpack = [wf2 (C x 2C)].
 * The backward given fused_pre_bar (fb), gates, hg and hf:
 *   ffno_fuse_bwd_h_tc: hf_bar [V][2C] = (fb wf2) * gelu'(hf); wpack = [wf2];
 *   ffno_fuse_bwd_q_tc: B_bar = hf_bar wf1 + [fb, fb] / 2, spec_bar = B_bar_s g_s, vert_bar = B_bar_v g_v, q [V][2C] =
 *     B_bar [s, v] g (1 - g) (q may be hf_bar); wpack = [wf1];
 *   ffno_fuse_bwd_x_tc: hg_bar = (q wg2) * gelu'(hg), A_bar = hg_bar wg1: x_bar = base + A_bar[:C], spec_bar +=
 *     A_bar[C:2C], vert_bar += A_bar[2C:]; wpack = ffno_fuse1_tc's [wg1 (C x 3C), wg2 (2C x C)].
 * C = 96 only; row pointers 32-byte aligned. The backward kernels read the transposed weights out of the packs. */
int ffno_fuse_hidden_tc(const float* spec_pre, const float* spec_coefs, const float* vert_pre, const float* vert_coefs,
                        const float* gates, long V, int C, const void* wpack, float* hf, int* err,
                        ffno_stream_t stream);
int ffno_fuse_out_tc(const float* spec_pre, const float* spec_coefs, const float* vert_pre, const float* vert_coefs,
                     const float* gates, const float* hf, long V, int C, const void* wpack, const float* dw,
                     float* pre, double* partials, int nparts, int groups, int* err, ffno_stream_t stream);
int ffno_fuse_bwd_h_tc(const float* fused_pre_bar, const float* hf, long V, int C, const void* wpack, float* hf_bar,
                       int* err, ffno_stream_t stream);
int ffno_fuse_bwd_q_tc(const float* spec_pre, const float* spec_coefs, const float* vert_pre, const float* vert_coefs,
                       const float* gates, const float* fused_pre_bar, const float* hf_bar, long V, int C,
                       const void* wpack, float* spec_bar, float* vert_bar, float* q, int* err, ffno_stream_t stream);
int ffno_fuse_bwd_x_tc(const float* q, const float* hg, const float* base, long V, int C, const void* wpack,
                       float* x_bar, float* spec_bar, float* vert_bar, int* err, ffno_stream_t stream);
/* ffno_mlp2_bwd; wpack = [w1 (2C x C), w2^T (2C x C), w1^T (C x 2C)]; at C = 96 the forward's pack [w1 (2C x C),
 * w2 (C x 2C)] (the kernel reads the transposes out of it; a, pre_bar, base, a_bar 32-byte aligned). */
int ffno_mlp2_bwd_tc(const float* a, const float* pre_bar, const float* base, long V, int C, const void* wpack,
                     float* a_bar, int* err, ffno_stream_t stream);
/* One branch of ffno_gate_bwd: x_bar = base + d/dx applied to g_bar, z_bar += g_bar . zp if zp; wpack = [g1, g2,
 * g2^T, g1^T], at C = 96 the forward's [g1, g2] (x 32-byte aligned). base may equal x_bar. */
int ffno_gate_bwd_tc(const float* x, const float* g_bar, const float* base, long V, int C, const void* wpack,
                     const float* zp, float* x_bar, float* z_bar, int* err, ffno_stream_t stream);
/* ffno_fuse_bwd in two stages after ffno_fuse1_tc has recomputed gates and hg:
 * a: hf_bar [V][2C] = (fused_pre_bar wf2) * gelu'(B wf1^T); wpack = [wf1 (2C x 2C), wf2^T (2C x C)]; spec_pre,
 *    vert_pre, gates and fused_pre_bar 32-byte aligned (FFNO_EINVAL otherwise)
 * b: the rest, writing x_bar, spec_bar, vert_bar; wpack = [wf1^T (2C x 2C), wg2^T (C x 2C), wg1^T (3C x C)]; its
 *    per-voxel arrays (spec_pre, vert_pre, gates, hg, fused_pre_bar, hf_bar, base, x_bar, spec_bar, vert_bar) must be
 *    32-byte aligned (FFNO_EINVAL otherwise). */
int ffno_fuse_bwd_a_tc(const float* spec_pre, const float* spec_coefs, const float* vert_pre, const float* vert_coefs,
                       const float* gates, const float* fused_pre_bar, long V, int C, const void* wpack,
                       float* hf_bar, int* err, ffno_stream_t stream);
int ffno_fuse_bwd_b_tc(const float* spec_pre, const float* spec_coefs, const float* vert_pre, const float* vert_coefs,
                       const float* gates, const float* hg, const float* fused_pre_bar, const float* hf_bar,
                       const float* base, long V, int C, const void* wpack, float* x_bar, float* spec_bar,
                       float* vert_bar, int* err, ffno_stream_t stream);
/* ffno_head_fwd and ffno_head_bwd (FFNO3D proj1 / proj2 and head_output, models/ffno_model.py:712-713, 729-748) with
 * the proj1 / proj2 GEMMs on tensor cores; b2 [nhp] (zero past nh); the LTE math in FP32 when params->math32, else
 * FP64. Forward wpack = [w1 (2C x C), w2 (nhp x 2C)]; backward wpack = [w1, w2, w2^T (2C x nhp), w1^T (C x 2C)],
 * with w2's rows past nh zero. x (the hidden state [V][C]) 32-byte aligned (FFNO_EINVAL otherwise). C = 96 also,
 * where the backward takes the forward's pack [w1, w2] (reading the transposes out of it) and x_bar is 32-byte
 * aligned too. */
int ffno_head_fwd_tc(const float* x, const float* x_in, long V, int C, const void* wpack, const float* b2, int nh,
                     int nhp, const ffno_head_params* params, float* out, float* head_out, int* err,
                     ffno_stream_t stream);
int ffno_head_bwd_tc(const float* x, const float* x_in, const float* y_bar, long V, int C, const void* wpack,
                     const float* b2, int nhp, const ffno_head_params* params, float* x_bar, float* x_in_bar,
                     int* err, ffno_stream_t stream);

/* ffno_xform on tensor cores (split-BF16), same descriptor; M <= 256, N and the input strides multiples of 8 floats,
 * the input pointer 32-byte aligned (rows are read 32 bytes a request).
 * tpack: T [M][K] packed per 128-row m-tile (rows past M zero) and, within it, per 32-wide k-chunk (K padded with
 * zeros to a multiple of 16; the last chunk narrower), each chunk its hi then lo half in the canonical K-major order
 * with the chunk's own width; ffno_xform_tc_pack_bytes gives the size. */
int ffno_xform_tc_pack_bytes(int M, int K);
int ffno_xform_tc(const void* tpack, const float* in, float* out, const ffno_xform_desc* desc, int accumulate, int* err,
                  ffno_stream_t stream);
/* ffno_xform on tensor cores with the whole table resident in shared memory (the split table [Mp][Kp] packed as one
 * canonical K-major operand, hi then lo; Mp a multiple of 16 <= 256, Kp a multiple of 16, 4 Mp Kp <=
 * ffno_xform_tcr_max_table_bytes()). N and the input strides multiples of 8 floats, the input pointer 32-byte aligned. */
int ffno_xform_tcr_max_table_bytes(void);
int ffno_xform_tcr(const void* tpack, int Mp, int Kp, const float* in, float* out, const ffno_xform_desc* desc,
                   int accumulate, int* err, ffno_stream_t stream);
/* ffno_spectral_mix on tensor cores (split-BF16); wpack = [wbig^T (2C x 2C)] with its output rows reordered so that
 * row p = 32 q + l is part l / 16 (0 re, 1 im) of channel 16 q + l % 16; C = 16, 32, 64; strides multiples of 4
 * floats. At C = 96: wpack = [M (2C x 2C)], out = g (x M) + the low-rank term, M = wbig (or wbig^T for the adjoint),
 * rank <= 8, strides multiples of 8 floats, in and out 32-byte aligned. */
int ffno_spectral_mix_tc(const float* in, float* out, long F, long nb, long sf, long sb, long s_im, int C,
                         const void* wpack, const float* g, const float* U, const float* Vm, int rank, int* err,
                         ffno_stream_t stream);
/* ffno_outer with the products on tensor cores (split-BF16, FP32 accumulation per split; the splits reduced in double
 * in a fixed order). Same part / nsplit contract (ffno_outer_parts); additionally N a multiple of 4 and lda, ldb >= N;
 * the shorter of Ma, Mb at most 256. */
int ffno_outer_tc(const float* A, long lda, int Ma, const float* B, long ldb, int Mb, long N, float* part, int nsplit,
                  double* out, int accumulate, int* err, ffno_stream_t stream);
/* ffno_outer_tc writing out rows of stride ldo >= Mb (a block of columns of a wider product): the gradient of a
 * production height table (2 M' up to ~1300 rows) taken in slices of the longer operand that fit the accumulator. */
int ffno_outer_tc_ld(const float* A, long lda, int Ma, const float* B, long ldb, int Mb, long N, float* part,
                     int nsplit, double* out, long ldo, int accumulate, int* err, ffno_stream_t stream);

/* ---- per-column height tables (HeightSpectralConv's non-shared path, models/ffno_model.py:276-280, 306-308), FP64
 * arithmetic. Column c has heights z_raw[c][0..D) (unshifted); k[0..live) the live wavenumbers; f[c][m] = factor_m
 * taper_m / length with the column's own taper. Writes the FP32 tables tzf [ncol][2 live][D] (Filon weights, real rows
 * then imaginary rows), tzi [ncol][D][2 live] (cos, -sin of z_j k_m times f) and their transposes tzf_t
 * [ncol][D][2 live], tzi_t [ncol][2 live][D], z_j = z_raw[c][j] - min_j z_raw[c][j]. */
#define FFNO_PERCOL_MAX_D 4096
#define FFNO_PERCOL_MAX_LIVE 2048
int ffno_percol_tables(const double* z_raw, int D, long ncol, const double* k, int live, const double* f, float* tzf,
                       float* tzi, float* tzf_t, float* tzi_t, ffno_stream_t stream);
/* Its gradient: z_bar[j * ncol + c] += d/dz_raw[c][j] of sum(tzf_bar * tzf) + sum(tzi_bar * tzi) (FP64 bars in the
 * layouts of tzf and tzi). df[c][m] = d f[c][m] / d dz_c, dz_c the median spacing of column c, which is spacing
 * med[c] (|z_raw[c][med + 1] - z_raw[c][med]|, the index torch.median returns); the minimum's gradient is shared
 * evenly by tied minima. */
int ffno_percol_tables_vjp(const double* z_raw, int D, long ncol, const double* k, int live, const double* f,
                           const double* df, const int* med, const double* tzf_bar, const double* tzi_bar,
                           float* z_bar, ffno_stream_t stream);
/* The same gradient for one column (a shared height grid: models/ffno_model.py:266-275, 302-305), spread over its
 * (mode, node) pairs instead of one CTA: z_bar[j * z_stride] += d/dz_raw[j]; med is the median spacing's index;
 * scratch holds 3 * live * D doubles. Sums run in a fixed order. */
int ffno_column_tables_vjp(const double* z_raw, int D, const double* k, int live, const double* f, const double* df,
                           int med, const double* tzf_bar, const double* tzi_bar, double* scratch, float* z_bar,
                           long z_stride, ffno_stream_t stream);

/* ---- forward-mode derivative (JVP): jvp_local (ffno_fsdp_runtime.py:350-372), the tangent of FFNO3D.forward along
 * an input tangent with the heights fixed. The linear stages reuse the forward entry points on the tangent (the lift
 * convolution ffno_lift_fwd, the DFTs ffno_xform / ffno_xform_pt, the mixing ffno_spectral_mix); these linearise the
 * nonlinear ones next to their primal inputs. FP32. */
/* GroupNorm tangent (DepthWeightedGroupNorm :77-95): per-CTA partials [nparts][groups][2] of S1 = sum w pre_dot and
 * S2 = sum w xhat pre_dot (reduce with ffno_gn_bwd_final), then out = base + res * gamma r (pre_dot - S1/T - xhat
 * S2/T) [* gelu'(y) with act = 1]. gstats as written by ffno_gn_finalize for the primal. base may be NULL. */
int ffno_gn_jvp_stats(const float* pre, const float* pre_dot, const double* gstats, const float* dw, long V, int C,
                      int groups, double* partials, int nparts, ffno_stream_t stream);
int ffno_gn_jvp_apply(const float* pre, const float* pre_dot, const float* gamma, const float* beta,
                      const double* gstats, const double* sums, int act, const float* base, float res, long V, int C,
                      int groups, float* out, ffno_stream_t stream);
/* Tangent of ffno_gate_fwd (the z_proj term is constant): same weights [K][N]. */
int ffno_gate_jvp(const float* x, const float* x_dot, long V, int C, const float* w1, const float* w2, float* out_dot,
                  ffno_stream_t stream);
/* Tangent of the MLP C -> 2C -> C of ffno_mlp2_fwd at input a (the residual prologue is applied by the caller). */
int ffno_mlp2_jvp(const float* a, const float* a_dot, long V, int C, const float* w1, const float* w2, float* out_dot,
                  ffno_stream_t stream);
/* Tangent of ffno_fuse_fwd's fused pre-activation (_fuse_branches :524-534) given the tangents spec_dot / vert_dot of
 * the branch outputs gelu(GN(spec_pre)), gelu(GN(vert_pre)). */
int ffno_fuse_jvp(const float* x, const float* x_dot, const float* spec_pre, const float* spec_coefs,
                  const float* vert_pre, const float* vert_coefs, const float* spec_dot, const float* vert_dot, long V,
                  int C, const float* wg1, const float* wg2, const float* bg2, const float* wf1, const float* wf2,
                  float* fused_dot, ffno_stream_t stream);
/* Tangent of ffno_head_fwd along the last block's tangent x_dot [V][C] and the input tangent x_in_dot [cin][V]:
 * out_dot [levels][V] (normalised log10 n). */
int ffno_head_jvp(const float* x, const float* x_dot, const float* x_in, const float* x_in_dot, long V, int C,
                  const float* p1, const float* p2, const float* b2, int nhp, const ffno_head_params* params,
                  float* out_dot, ffno_stream_t stream);
/* Service units: SI feature tangent (6, nz, nx, ny) -> normalised model-input tangent; model-output tangent ->
 * population tangent (nz, nx, ny, L) in m^-3 (0 where the +-37 clamp is active). flags as ffno_si_*. */
int ffno_si_input_tangent(const float* features, const float* tangent, long V, const float* std_x, float* x_dot,
                          int* flags, ffno_stream_t stream);
int ffno_si_population_tangent(const float* y, const float* y_dot, long V, int L, const float* mean_y,
                               const float* std_y, float* out, int* flags, ffno_stream_t stream);

/* Self-test of the tensor-core primitives (no reference counterpart: it pins this library's tcgen05 descriptor and
 * tensor-memory conventions): D [128][N] = bf16(A [128][K]) @ bf16(B [N][K])^T in FP32, one CTA, with B staged
 * K-major (b_mn = 0) or MN-major (b_mn = 1); K, N multiples of 16 up to 256. *status (device int) is set to 1 if the
 * MMA completion wait ran out. */
int ffno_tc_selftest(const float* A, const float* B, int K, int N, int b_mn, float* D, int* status,
                     ffno_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* FFNOML_GB300_H */
