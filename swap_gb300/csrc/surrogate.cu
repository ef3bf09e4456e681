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

// ---------------------------------------------------------------------------
// 3x3x3 periodic convolution as an implicit GEMM on the tensor cores
// ---------------------------------------------------------------------------
//
// Activations are channel-last BF16, X[v][CIN] with v = x + nx*(y + ny*z).
// Weights are W[tap][cout][cin] BF16 with tap = (dz+1)*9 + (dy+1)*3 + (dx+1);
// one layer's weights stay in shared memory as 27 B operands.  A CTA owns
// tiles of 128 consecutive voxels: for every tap its 128 threads gather the
// neighbours' channel vectors into an A operand (double-buffered) while the
// tensor core multiplies the previous tap, accumulating D = 128 x COUT in
// tensor memory.  The epilogue adds the bias and writes BF16 (with GELU) or
// FP32.

struct ConvArgs {
  int nx, ny, nz;
  long long V;                         // voxels, a multiple of 128
  const __nv_bfloat16* X;              // [V][CIN]
  const __nv_bfloat16* W;              // [27][COUT][CIN]
  const float* bias;                   // [COUT] (may be null)
  __nv_bfloat16* Y;                    // [V][COUT] activations out (may be null)
  __nv_bfloat16* Z;                    // [V][COUT] pre-activations out (may be null)
  float* Yf;                           // [V][ldf] FP32 out (may be null)
  int ldf, nstore;                     // FP32 row length and channels stored
  int gelu;                            // apply GELU for Y
  int* err;
};

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }

template <int CIN, int COUT>
__global__ void __launch_bounds__(128) k_conv3(ConvArgs a) {
  static_assert(CIN % 16 == 0 && (COUT == 16 || COUT == 32), "operand shapes");
  constexpr int WBYTES = 27 * COUT * CIN * 2, ABYTES = 128 * CIN * 2;
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* sW = smem;
  uint8_t* sA0 = smem + WBYTES;
  __shared__ uint64_t mbar[2];
  __shared__ uint32_t tslot;
  __shared__ float sbias[COUT];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // weights into the K-major core layout, one B operand (COUT x CIN) per tap
  for (int i = tid; i < 27 * COUT * CIN; i += 128) {
    const int t = i / (COUT * CIN), r = i % (COUT * CIN), n = r / CIN, k = r % CIN;
    *reinterpret_cast<__nv_bfloat16*>(sW + t * (COUT * CIN * 2) + tc05::core_offset(n, k, COUT)) = a.W[i];
  }
  if (tid < COUT) sbias[tid] = a.bias ? a.bias[tid] : 0.0f;
  if (warp == 0) tc05::tmem_alloc(&tslot, 32);
  if (tid == 0) {
    tc05::mbar_init(&mbar[0], 1);
    tc05::mbar_init(&mbar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc05::fence_async_smem();
  tc05::fence_before_sync();
  __syncthreads();
  tc05::fence_after_sync();
  const uint32_t tmem = tslot;
  constexpr uint32_t idesc = tc05::idesc_bf16_f32(128, COUT);
  const uint32_t w0 = tc05::smem_u32(sW), abase = tc05::smem_u32(sA0);
  uint32_t issued[2] = {0, 0}, waited[2] = {0, 0};
  bool ok = true;
  const long long ntiles = a.V / 128;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long v = tile * 128 + tid;
    const int x = (int)(v % a.nx), y = (int)((v / a.nx) % a.ny), z = (int)(v / ((long long)a.nx * a.ny));
    for (int t = 0; t < 27; ++t) {
      const int b = t & 1;
      if (issued[b] > waited[b]) {  // the MMAs that read this buffer are done
        ok &= tc05::mbar_wait(&mbar[b], waited[b] & 1, WAIT_LIMIT);
        ++waited[b];
      }
      const int dx = t % 3 - 1, dy = (t / 3) % 3 - 1, dz = t / 9 - 1;
      int xn = x + dx, yn = y + dy, zn = z + dz;
      xn = xn < 0 ? xn + a.nx : (xn >= a.nx ? xn - a.nx : xn);
      yn = yn < 0 ? yn + a.ny : (yn >= a.ny ? yn - a.ny : yn);
      zn = zn < 0 ? zn + a.nz : (zn >= a.nz ? zn - a.nz : zn);
      const long long u = xn + (long long)a.nx * (yn + (long long)a.ny * zn);
      const uint4* src = reinterpret_cast<const uint4*>(a.X + u * CIN);
      uint8_t* dst = sA0 + b * ABYTES;
#pragma unroll
      for (int q = 0; q < CIN / 8; ++q) *reinterpret_cast<uint4*>(dst + tc05::core_offset(tid, 8 * q, 128)) = src[q];
      tc05::fence_async_smem();
      tc05::fence_before_sync();
      __syncthreads();
      tc05::fence_after_sync();
      if (tid == 0) {
#pragma unroll
        for (int kk = 0; kk < CIN / 16; ++kk) {
          const uint64_t ad = tc05::desc_noswizzle(abase + b * ABYTES + kk * 2 * (16 * 128), 16 * 128, 128);
          const uint64_t bd =
              tc05::desc_noswizzle(w0 + t * (COUT * CIN * 2) + kk * 2 * ((COUT / 8) * 128), (COUT / 8) * 128, 128);
          tc05::mma_bf16(tmem, ad, bd, idesc, t > 0 || kk > 0);
        }
        tc05::mma_commit(&mbar[b]);
      }
      ++issued[b];
    }
    for (int b = 0; b < 2; ++b)
      if (issued[b] > waited[b]) {
        ok &= tc05::mbar_wait(&mbar[b], waited[b] & 1, WAIT_LIMIT);
        ++waited[b];
      }
    tc05::fence_after_sync();
    float acc[COUT];
    if (COUT == 32) tc05::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16), acc);
    else tc05::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16), acc);
    const long long vo = tile * 128 + warp * 32 + lane;
#pragma unroll
    for (int c = 0; c < COUT; ++c) acc[c] += sbias[c];
    if (a.Z) {
#pragma unroll
      for (int c = 0; c < COUT; c += 8) {
        __nv_bfloat16 h[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) h[e] = __float2bfloat16(acc[c + e]);
        *reinterpret_cast<uint4*>(a.Z + vo * COUT + c) = *reinterpret_cast<const uint4*>(h);
      }
    }
    if (a.Y) {
#pragma unroll
      for (int c = 0; c < COUT; c += 8) {
        __nv_bfloat16 h[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) h[e] = __float2bfloat16(a.gelu ? gelu(acc[c + e]) : acc[c + e]);
        *reinterpret_cast<uint4*>(a.Y + vo * COUT + c) = *reinterpret_cast<const uint4*>(h);
      }
    }
    if (a.Yf) {
#pragma unroll
      for (int c = 0; c < COUT; ++c)
        if (c < a.nstore) a.Yf[vo * a.ldf + c] = acc[c];
    }
    tc05::fence_before_sync();
    __syncthreads();  // accumulator reads done before the next tile's MMAs
    tc05::fence_after_sync();
  }
  if (!ok) atomicCAS(a.err, 0, SWAP_EWAIT);
  tc05::fence_before_sync();
  __syncthreads();
  if (warp == 0) tc05::tmem_free(tmem, 32);
}

template <int CIN, int COUT>
cudaError_t launch_conv3(const ConvArgs& a, int nsm, cudaStream_t st) {
  const int smem = 27 * COUT * CIN * 2 + 2 * 128 * CIN * 2;
  cudaError_t e = cudaFuncSetAttribute(k_conv3<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  const long long ntiles = a.V / 128;
  const int grid = (int)(ntiles < 2LL * nsm ? ntiles : 2LL * nsm);
  k_conv3<CIN, COUT><<<grid, 128, smem, st>>>(a);
  return cudaGetLastError();
}

cudaError_t conv3(int cin, int cout, const ConvArgs& a, cudaStream_t st) {
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (cin == 16 && cout == 32) return launch_conv3<16, 32>(a, nsm, st);
  if (cin == 32 && cout == 32) return launch_conv3<32, 32>(a, nsm, st);
  if (cin == 32 && cout == 16) return launch_conv3<32, 16>(a, nsm, st);
  if (cin == 16 && cout == 16) return launch_conv3<16, 16>(a, nsm, st);
  return cudaErrorInvalidValue;
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

// Validation entry: one periodic 3x3x3 convolution layer on the tensor
// cores.  Device arrays X [V][cin] bf16, W [27][cout][cin] bf16, bias
// [cout] FP32 (may be null); writes Y [V][cout] bf16 (GELU when gelu != 0)
// when Y is given and Yf [V][cout] FP32 (pre-activation) when Yf is given.
extern "C" int swap_conv3_check(int32_t nx, int32_t ny, int32_t nz, int32_t cin, int32_t cout, const void* X,
                                const void* W, const float* bias, void* Y, float* Yf, int32_t gelu_on) {
  const long long V = (long long)nx * ny * nz;
  if (nx < 1 || ny < 1 || nz < 1 || V % 128 || !X || !W || (!Y && !Yf)) return SWAP_EINVAL;
  int* err = nullptr;
  if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) return SWAP_ECUDA;
  cudaMemset(err, 0, sizeof(int));
  ConvArgs a{};
  a.nx = nx; a.ny = ny; a.nz = nz; a.V = V;
  a.X = static_cast<const __nv_bfloat16*>(X);
  a.W = static_cast<const __nv_bfloat16*>(W);
  a.bias = bias;
  a.Y = static_cast<__nv_bfloat16*>(Y);
  a.Yf = Yf;
  a.ldf = cout;
  a.nstore = cout;
  a.gelu = gelu_on;
  a.err = err;
  cudaError_t e = conv3(cin, cout, a, nullptr);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  int h = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&h, err, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(err);
  if (e == cudaErrorInvalidValue) return SWAP_EINVAL;
  if (e != cudaSuccess) return SWAP_ECUDA;
  return h ? SWAP_EWAIT : SWAP_OK;
}
