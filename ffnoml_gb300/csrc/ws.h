// Warp-specialised tensor-core kernels (pointwise_ws.cu), called by the C entry points of pointwise_tc.cu for the
// widths they support.
#pragma once
#include <cuda_runtime.h>

namespace ffno {
namespace ws {

bool mlp2_fwd_supported(int C);
int mlp2_fwd(int mode, const float* in, const float* prev_pre, const float* prev_coefs, float res, float* xout, long V,
             int C, const void* wpack, const float* dw, float* pre, double* partials, int nparts, int* err,
             cudaStream_t stream);
bool fuse1_supported(int C);
int fuse1(const float* x, const float* spec_pre, const float* spec_coefs, const float* vert_pre,
          const float* vert_coefs, long V, int C, const void* wpack, const float* bias, float* gates, float* hg,
          int* err, cudaStream_t stream);
bool fuse2_supported(int C);
int fuse2(const float* spec_pre, const float* spec_coefs, const float* vert_pre, const float* vert_coefs,
          const float* gates, long V, int C, const void* wpack, const float* dw, float* pre, double* partials,
          int nparts, int* err, cudaStream_t stream);
bool gate_fwd_supported(int C);
int gate_fwd(const float* x, long V, int C, const void* wpack, const float* zp, const float* z, float* out, int* err,
             cudaStream_t stream);
bool gate_bwd_supported(int C);
int gate_bwd(const float* x, const float* g_bar, const float* base, long V, int C, const void* wpack, const float* zp,
             float* x_bar, float* z_bar, int* err, cudaStream_t stream);
bool mlp2_bwd_supported(int C);
int mlp2_bwd(const float* a, const float* pre_bar, const float* base, long V, int C, const void* wpack, float* a_bar,
             int* err, cudaStream_t stream);

}  // namespace ws
}  // namespace ffno
