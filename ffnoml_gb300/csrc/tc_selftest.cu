// Self-test of the tcgen05 primitives: one CTA computes D [128 x N] = A [128 x K] * B [N x K]^T with BF16 operands
// staged in canonical K-major shared-memory tiles and an FP32 accumulator in tensor memory. Used by the GPU tests to
// pin the descriptor and TMEM conventions of the BF16 kernels.
#include "common.cuh"
#include "tc.cuh"

using namespace ffno;

namespace {

__global__ void __launch_bounds__(128) k_tc_selftest(const float* __restrict__ A, const float* __restrict__ B, int K,
                                                     int N, int b_mn, float* __restrict__ D,
                                                     int* __restrict__ status) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tslot;
  uint8_t* sa = smem;
  uint8_t* sb = smem + 128 * K * 2;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int e = tid; e < 128 * K; e += 128) {
    const int r = e / K, k = e % K;
    *reinterpret_cast<__nv_bfloat16*>(sa + tc::kmajor_offset(r, k, K)) = __float2bfloat16_rn(A[e]);
  }
  for (int e = tid; e < N * K; e += 128) {
    const int r = e / K, k = e % K;
    const uint32_t off = b_mn ? tc::mnmajor_offset(r, k, N) : tc::kmajor_offset(r, k, K);
    *reinterpret_cast<__nv_bfloat16*>(sb + off) = __float2bfloat16_rn(B[e]);
  }
  if (warp == 0) tc::tmem_alloc(&tslot, 512);
  if (tid == 0) {
    tc::mbar_init(&bar, 1);
    tc::mbar_init_fence();
  }
  tc::fence_async_smem();
  tc::tc_before_sync();
  __syncthreads();
  tc::tc_after_sync();
  const uint32_t taddr = tslot;
  if (tid == 0) {
    if (b_mn)
      tc::gemm_128xN_bmn(taddr, tc::smem_u32(sa), tc::smem_u32(sb), K, N, false);
    else
      tc::gemm_128xN(taddr, tc::smem_u32(sa), tc::smem_u32(sb), K, N, false);
    tc::mma_commit(&bar);
  }
  const bool ok = tc::mbar_wait(&bar, 0);
  if (!ok && tid == 0) atomicExch(status, 1);
  tc::tc_after_sync();
  if (ok) {
    for (int c0 = 0; c0 < N; c0 += 16) {
      float v[16];
      tc::tmem_ld16(taddr + ((uint32_t)(32 * warp) << 16) + (uint32_t)c0, v);
      const int row = 32 * warp + lane;
#pragma unroll
      for (int i = 0; i < 16; ++i) D[row * N + c0 + i] = v[i];
    }
  }
  tc::tc_before_sync();
  __syncthreads();
  if (warp == 0) tc::tmem_free(taddr, 512);
}

}  // namespace

extern "C" int ffno_tc_selftest(const float* A, const float* B, int K, int N, int b_mn, float* D, int* status,
                                ffno_stream_t stream) {
  if (!A || !B || !D || !status || K < 16 || K % 16 || K > 256 || N < 16 || N % 16 || N > 256) return FFNO_EINVAL;
  const size_t smem = (size_t)(128 + N) * K * 2 + 1024;
  if (!ffno::smem_cap_ok(k_tc_selftest, smem))
    return FFNO_ELAUNCH;
  k_tc_selftest<<<1, 128, smem, (cudaStream_t)stream>>>(A, B, K, N, b_mn, D, status);
  FFNO_CHECK_LAUNCH();
  return FFNO_OK;
}
