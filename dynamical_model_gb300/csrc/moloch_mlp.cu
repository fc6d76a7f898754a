// Tensor-core (tcgen05) GEMM and the kernels of the learned acoustic-cycle
// surrogate: a per-column MLP trained and run on BF16 operands with FP32
// accumulation in TMEM.
//
// k_gemm_tc computes C = act(A * B^T + bias) for A [M][K] and B [N][K] in
// BF16, row-major with K contiguous (both operands K-major), C in FP32
// and/or BF16.  One CTA owns 128 rows x up to 256 columns; the K loop
// stages 64-wide chunks of A and B in shared memory in the no-swizzle
// K-major core-matrix layout (moloch_tc.cuh), one thread issues four
// 128 x N x 16 MMAs per chunk and commits them to an mbarrier that the
// whole CTA waits on (bounded).  The accumulator lives in TMEM and is read
// back with tcgen05.ld by the four warps, one 32-lane quarter each.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdio>

#include "../../include/moloch_gb300.h"
#include "moloch_tc.cuh"

extern "C" void moloch_internal_set_error(const char* msg);

namespace moloch {
namespace mlp {

constexpr int kChunkK = 64;              // K elements staged per chunk
constexpr int kTileM = 128;              // UMMA M
constexpr int kTileN = 256;              // max N per CTA
constexpr int kASlot = 32 * 1024;        // A chunk (16 KB) with room to spare
constexpr int kBSlot = 64 * 1024;        // B chunk (32 KB) with room to spare
constexpr int kSmem = kASlot + kBSlot;

enum Act { ACT_NONE = 0, ACT_SILU = 1 };

static __device__ int g_tc_error;  // set when a bounded wait gives up

__device__ __forceinline__ float silu(float x) { return x / (1.0f + __expf(-x)); }

__global__ void __launch_bounds__(128, 1)
    k_gemm_tc(const __nv_bfloat16* __restrict__ A, int lda, const __nv_bfloat16* __restrict__ B, int ldb,
              float* __restrict__ C, int ldc, __nv_bfloat16* __restrict__ Cb, int ldcb,
              const float* __restrict__ bias, int M, int N, int K, int act) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tmem_base;
  uint8_t* sA = smem;
  uint8_t* sB = smem + kASlot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int m0 = blockIdx.x * kTileM, n0 = blockIdx.y * kTileN;
  const int nt = min(kTileN, N - n0);  // multiple of 16
  if (warp == 0) tc::tmem_alloc(&tmem_base, 256);
  if (tid == 0) tc::mbar_init(&bar, 1);
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tbase = tmem_base;
  const uint32_t idesc = tc::idesc_bf16(nt);
  const uint32_t aaddr = tc::smem_u32(sA), baddr = tc::smem_u32(sB);
  constexpr uint32_t kLBO = 128, kSBO = (kChunkK / 8) * 128;
  uint32_t parity = 0;
  bool ok = true;
  for (int k0 = 0; k0 < K; k0 += kChunkK) {
    // stage the chunk: one 16-byte vector = one core-matrix row (8 BF16)
    for (int q = tid; q < kTileM * (kChunkK / 8); q += 128) {
      const int r = q / (kChunkK / 8), kc = q % (kChunkK / 8);
      uint4 val = make_uint4(0, 0, 0, 0);
      if (m0 + r < M) val = *reinterpret_cast<const uint4*>(A + (size_t)(m0 + r) * lda + k0 + kc * 8);
      *reinterpret_cast<uint4*>(sA + ((r >> 3) * (kChunkK / 8) + kc) * 128 + (r & 7) * 16) = val;
    }
    for (int q = tid; q < nt * (kChunkK / 8); q += 128) {
      const int r = q / (kChunkK / 8), kc = q % (kChunkK / 8);
      const uint4 val = *reinterpret_cast<const uint4*>(B + (size_t)(n0 + r) * ldb + k0 + kc * 8);
      *reinterpret_cast<uint4*>(sB + ((r >> 3) * (kChunkK / 8) + kc) * 128 + (r & 7) * 16) = val;
    }
    tc::fence_proxy_async();  // generic-proxy stores -> visible to the tensor core
    __syncthreads();
    if (tid == 0) {
      tc::tc_fence_after();
#pragma unroll
      for (int kk = 0; kk < kChunkK / 16; ++kk) {  // K = 16 per MMA = two core matrices
        const uint64_t ad = tc::smem_desc(aaddr + kk * 256, kLBO, kSBO);
        const uint64_t bd = tc::smem_desc(baddr + kk * 256, kLBO, kSBO);
        tc::mma_bf16(tbase, ad, bd, idesc, (k0 > 0 || kk > 0) ? 1 : 0);
      }
      tc::mma_commit(&bar);
    }
    if (!tc::mbar_wait(&bar, parity)) {
      ok = false;
      atomicExch(&g_tc_error, 1);
      break;
    }
    parity ^= 1;
    tc::tc_fence_after();
    __syncthreads();  // everyone saw the MMAs finish: the chunk buffers are free
  }
  if (ok) {
    const uint32_t lrow = (uint32_t)(warp * 32) << 16;
    const int row = m0 + warp * 32 + lane;
    for (int c = 0; c < nt; c += 16) {
      float v[16];
      tc::tmem_ld16(tbase + lrow + c, v);
      if (row < M) {
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int col = n0 + c + q;
          float x = v[q] + (bias ? bias[col] : 0.f);
          if (C) C[(size_t)row * ldc + col] = x;
          if (Cb) Cb[(size_t)row * ldcb + col] = __float2bfloat16_rn(act == ACT_SILU ? silu(x) : x);
        }
      }
    }
  } else {
    // a wait gave up: let any MMA still in flight finish (bounded) before
    // the accumulator columns are released
    tc::mbar_wait(&bar, parity);
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tbase, 256);
}

}  // namespace mlp
}  // namespace moloch

using namespace moloch::mlp;

// GEMM on device buffers for the surrogate and its tests.
extern "C" int moloch_tc_gemm(const void* A, int lda, const void* B, int ldb, float* C, int ldc, void* Cb, int ldcb,
                              const float* bias, int M, int N, int K, int act, void* stream) {
  if (!A || !B || (!C && !Cb) || M <= 0 || N <= 0 || K <= 0) {
    moloch_internal_set_error("tc_gemm: bad arguments");
    return MOLOCH_ERR_ARG;
  }
  if (N % 16 || K % kChunkK || lda % 8 || ldb % 8 || lda < K || ldb < K || (C && ldc < N) || (Cb && ldcb < N)) {
    moloch_internal_set_error("tc_gemm: need N % 16 == 0, K % 64 == 0, 16-byte aligned rows");
    return MOLOCH_ERR_ARG;
  }
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
    attr = true;
  }
  dim3 grid((M + kTileM - 1) / kTileM, (N + kTileN - 1) / kTileN);
  k_gemm_tc<<<grid, 128, kSmem, (cudaStream_t)stream>>>((const __nv_bfloat16*)A, lda, (const __nv_bfloat16*)B, ldb, C, ldc,
                                                         (__nv_bfloat16*)Cb, ldcb, bias, M, N, K, act);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    moloch_internal_set_error(cudaGetErrorString(e));
    return MOLOCH_ERR_CUDA;
  }
  return MOLOCH_OK;
}

// Reads and clears the flag a bounded tensor-core wait sets when it gives
// up (synchronises the device).
extern "C" int moloch_tc_status(void) {
  int v = 0;
  if (cudaDeviceSynchronize() != cudaSuccess) return MOLOCH_ERR_CUDA;
  cudaMemcpyFromSymbol(&v, g_tc_error, sizeof(int));
  const int z = 0;
  cudaMemcpyToSymbol(g_tc_error, &z, sizeof(int));
  return v ? MOLOCH_ERR_TIMEOUT : MOLOCH_OK;
}
