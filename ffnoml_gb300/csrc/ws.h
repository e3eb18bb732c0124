// Warp-specialised tensor-core kernels (pointwise_ws.cu), called by the C entry points of pointwise_tc.cu for the
// widths they support.
#pragma once
#include <cuda_runtime.h>

namespace ffno {
namespace ws {

bool mlp2_bwd_supported(int C);
int mlp2_bwd(const float* a, const float* pre_bar, const float* base, long V, int C, const void* wpack, float* a_bar,
             int* err, cudaStream_t stream);

}  // namespace ws
}  // namespace ffno
