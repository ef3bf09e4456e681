// surrogate.cu -- the learned field-subcycle surrogate: BF16 3D convolutions
// on the 5th-generation tensor cores (tcgen05.mma, FP32 accumulation in
// tensor memory).
//
// This unit starts with the GEMM core that the convolutions are built on and
// an entry that runs it on caller data, so its operand layouts can be checked
// against a CPU product.
#include <cstdint>
#include <string>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/swap_gpu.h"
#include "tc05.cuh"

namespace {

constexpr uint32_t WAIT_LIMIT = 1u << 20;  // polls of an mbarrier before giving up

// D (128 x 32, FP32) = A (128 x K, bf16) * B (32 x K, bf16)^T, one CTA of
// 128 threads, K a multiple of 16 up to 256.
__global__ void __launch_bounds__(128) k_tc_gemm_check(const __nv_bfloat16* __restrict__ A,
                                                       const __nv_bfloat16* __restrict__ B, float* __restrict__ D,
                                                       int K, int* err) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t mbar;
  __shared__ uint32_t tslot;
  uint8_t* sA = smem;
  uint8_t* sB = smem + 128 * K * 2;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  for (int i = tid; i < 128 * K; i += blockDim.x)
    *reinterpret_cast<__nv_bfloat16*>(sA + tc05::core_offset(i / K, i % K, 128)) = A[i];
  for (int i = tid; i < 32 * K; i += blockDim.x)
    *reinterpret_cast<__nv_bfloat16*>(sB + tc05::core_offset(i / K, i % K, 32)) = B[i];
  if (warp == 0) tc05::tmem_alloc(&tslot, 32);
  if (tid == 0) {
    tc05::mbar_init(&mbar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc05::fence_async_smem();
  tc05::fence_before_sync();
  __syncthreads();
  tc05::fence_after_sync();
  const uint32_t tmem = tslot;
  if (tid == 0) {
    constexpr uint32_t idesc = tc05::idesc_bf16_f32(128, 32);
    const uint32_t a0 = tc05::smem_u32(sA), b0 = tc05::smem_u32(sB);
    for (int s = 0; s < K / 16; ++s) {
      const uint64_t ad = tc05::desc_noswizzle(a0 + s * 2 * (16 * 128), 16 * 128, 128);
      const uint64_t bd = tc05::desc_noswizzle(b0 + s * 2 * (4 * 128), 4 * 128, 128);
      tc05::mma_bf16(tmem, ad, bd, idesc, s > 0);
    }
    tc05::mma_commit(&mbar);
  }
  __syncwarp();
  if (!tc05::mbar_wait(&mbar, 0, WAIT_LIMIT)) atomicCAS(err, 0, SWAP_EWAIT);
  tc05::fence_after_sync();
  float v[32];
  tc05::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16), v);
#pragma unroll
  for (int j = 0; j < 32; ++j) D[(warp * 32 + lane) * 32 + j] = v[j];
  tc05::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc05::tmem_free(tmem, 32);
}

}  // namespace

// Validation entry: D = A * B^T on the tensor cores for device arrays A
// (128 x K bf16, row-major), B (32 x K bf16, row-major), D (128 x 32 FP32).
extern "C" int swap_tc_gemm_check(const void* A, const void* B, float* D, int32_t K) {
  if (!A || !B || !D || K < 16 || K > 256 || K % 16) return SWAP_EINVAL;
  int* err = nullptr;
  if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) return SWAP_ECUDA;
  cudaMemset(err, 0, sizeof(int));
  const int smem = 128 * 1024;  // room for any reading of the operand layout
  cudaFuncSetAttribute(k_tc_gemm_check, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  k_tc_gemm_check<<<1, 128, smem>>>(static_cast<const __nv_bfloat16*>(A), static_cast<const __nv_bfloat16*>(B), D,
                                    K, err);
  cudaError_t e = cudaDeviceSynchronize();
  int h = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(err);
  if (e != cudaSuccess) return SWAP_ECUDA;
  return h ? SWAP_EWAIT : SWAP_OK;
}
