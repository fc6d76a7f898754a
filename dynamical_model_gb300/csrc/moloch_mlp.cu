// Tensor-core (tcgen05) GEMM and the kernels of the learned acoustic-cycle
// surrogate: a per-column MLP trained and run on BF16 operands with FP32
// accumulation in TMEM.
//
// k_gemm_tc computes C = act(A * B^T + bias) for A [M][K] and B [N][K] in
// BF16, row-major with K contiguous (both operands K-major), C in FP32
// and/or BF16, in output tiles of 128 rows x up to 256 columns handed out
// round-robin to persistent CTAs (one per SM).  Every wait is bounded; a
// wait that gives up sets g_tc_error, and the CTA still drains its copies
// and MMAs in flight (bounded) before it frees TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <mutex>

#include "../../include/moloch_gb300.h"
#include "moloch_tc.cuh"
#include "moloch_view.h"

extern "C" void moloch_internal_set_error(const char* msg);

namespace moloch {
namespace mlp {

constexpr int kChunkK = 64;               // K elements per stage (128 B rows: one swizzle atom)
constexpr int kTileM = 128;               // UMMA M
constexpr int kTileN = 256;               // max N per CTA
constexpr int kStages = 4;
constexpr int kAStage = kTileM * kChunkK * 2;   // 16 KB
constexpr int kBStage = kTileN * kChunkK * 2;   // 32 KB
constexpr int kSmem = kStages * (kAStage + kBStage) + 1024;  // + alignment slack
constexpr int kThreads = 320;  // loader warp, MMA warp, eight epilogue warps
constexpr int kEpiThreads = 256;

enum Act { ACT_NONE = 0, ACT_SILU = 1 };

static __device__ int g_tc_error;  // set when a bounded wait gives up
// limit of every mbarrier wait of k_gemm_tc, SM clock cycles
static __device__ long long g_tc_spin = kDefaultSpinCycles;
// test hook: the loader of CTA g_tc_skip_cta leaves its K-chunk number
// g_tc_skip_it (counted over the CTA's tiles) unarmed and unissued, so the
// MMA wait for it finds nothing in flight and runs out (-1: off)
static __device__ int g_tc_skip_cta = -1;
static __device__ int g_tc_skip_it = -1;

// x * sigmoid(x) with the fast reciprocal divide (relative error ~1e-7,
// far below the BF16 rounding of the stored activation); exp(-x) = inf
// for very negative x gives 0
__device__ __forceinline__ float silu(float x) { return __fdividef(x, 1.0f + __expf(-x)); }

// Persistent CTA (one per SM), ten warps: warp 0 issues the TMA loads of
// 64-wide K chunks of A and B (128-byte swizzle) into a kStages-deep ring of
// shared-memory stages, warp 1 issues the 128 x N x 16 MMAs of each chunk
// and commits them to the stage's "empty" barrier, and warps 2-9 drain the
// accumulator of the previous tile from TMEM (tcgen05.ld; two warps per
// 32-lane quarter, taking alternate 32-column groups) while the next tile
// accumulates: two accumulators of 256 columns each are double-buffered in
// the 512 TMEM columns.  The epilogue is latency-bound per warp (bias,
// SiLU, BF16 packing, row stores), so it gets two warps per quarter.
__global__ void __launch_bounds__(kThreads, 1)
    k_gemm_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB, int boxB,
              float* __restrict__ C, int ldc, __nv_bfloat16* __restrict__ Cb, int ldcb,
              const float* __restrict__ bias, int M, int N, int K, int act, const int* __restrict__ run,
              float* __restrict__ Ct, int ldct) {
  if (run && !*run) return;  // device-side skip (a captured step whose surrogate is off)
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full[kStages], empty[kStages], acc_full[2], acc_empty[2], done;
  __shared__ uint32_t tmem_base;
  __shared__ int s_fail, s_issued, s_consumed;
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nm = (M + kTileM - 1) / kTileM, nn = (N + kTileN - 1) / kTileN, ntiles = nm * nn;
  const int nk = K / kChunkK;
  const long long lim = g_tc_spin;
  const int skip_it = (int)blockIdx.x == g_tc_skip_cta ? g_tc_skip_it : -1;
  if (warp == 0) tc::tmem_alloc(&tmem_base, 512);
  if (tid == 32) {
    for (int s = 0; s < kStages; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(&acc_full[b], 1);
      tc::mbar_init(&acc_empty[b], kEpiThreads);
    }
    tc::mbar_init(&done, 1);
    s_fail = 0;
    s_issued = 0;
    s_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tbase = tmem_base;
  const uint32_t stage_bytes = (uint32_t)(kTileM + boxB) * kChunkK * 2;
  if (tid == 0) {
    // ---- loader
    int it = 0;
    for (int t = blockIdx.x; t < ntiles && !*(volatile int*)&s_fail; t += gridDim.x) {
      const int m0 = (t % nm) * kTileM, n0 = (t / nm) * kTileN;
      for (int kc = 0; kc < nk; ++kc, ++it) {
        const int s = it % kStages;
        if (it >= kStages && !tc::mbar_wait_cycles(&empty[s], ((it / kStages) - 1) & 1, lim)) {
          s_fail = 1;
          break;
        }
        if (it == skip_it) continue;  // test hook: this stage stays unarmed
        uint8_t* sa = smem + s * (kAStage + kBStage);
        tc::mbar_arrive_expect_tx(&full[s], stage_bytes);
        tc::tma_load_2d(sa, &tmA, kc * kChunkK, m0, &full[s]);
        tc::tma_load_2d(sa + kAStage, &tmB, kc * kChunkK, n0, &full[s]);
        s_issued = it + 1;
      }
    }
  } else if (tid == 32) {
    // ---- MMA issuer
    int it = 0, lt = 0;
    for (int t = blockIdx.x; t < ntiles && !*(volatile int*)&s_fail; t += gridDim.x, ++lt) {
      const int n0 = (t / nm) * kTileN;
      const int nt = min(kTileN, N - n0);
      const uint32_t idesc = tc::idesc_bf16(nt);
      const int b = lt & 1;
      if (lt >= 2 && !tc::mbar_wait_cycles(&acc_empty[b], ((lt >> 1) - 1) & 1, lim)) {
        s_fail = 1;
        break;
      }
      tc::tc_fence_after();
      const uint32_t dacc = tbase + (uint32_t)(b * kTileN);
      for (int kc = 0; kc < nk; ++kc, ++it) {
        const int s = it % kStages;
        if (!tc::mbar_wait_cycles(&full[s], (it / kStages) & 1, lim)) {
          s_fail = 1;
          break;
        }
        tc::tc_fence_after();
        const uint32_t aaddr = tc::smem_u32(smem + s * (kAStage + kBStage));
        const uint32_t baddr = aaddr + kAStage;
#pragma unroll
        for (int kk = 0; kk < kChunkK / 16; ++kk)
          tc::mma_bf16(dacc, tc::smem_desc_sw128(aaddr + kk * 32), tc::smem_desc_sw128(baddr + kk * 32), idesc,
                       (kc > 0 || kk > 0) ? 1 : 0);
        tc::mma_commit(&empty[s]);
        s_consumed = it + 1;
      }
      if (*(volatile int*)&s_fail) break;
      tc::mma_commit(&acc_full[b]);
    }
    tc::mma_commit(&done);  // arrives once every MMA issued above has completed
  } else if (warp >= 2) {
    // ---- epilogue: warp w reads TMEM lanes 32*(w%4) .. +31 and the
    // 32-column groups h, h+2, h+4, ... of the tile (h = (w-2)/4)
    const int q = warp & 3, h = (warp - 2) >> 2;
    const uint32_t lrow = (uint32_t)(q * 32) << 16;
    const bool bias4 = bias && ((reinterpret_cast<uintptr_t>(bias) & 15) == 0);
    int lt = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++lt) {
      const int b = lt & 1;
      if (!tc::mbar_wait_cycles(&acc_full[b], (lt >> 1) & 1, lim)) {
        s_fail = 1;
        break;
      }
      tc::tc_fence_after();
      const int m0 = (t % nm) * kTileM, n0 = (t / nm) * kTileN;
      const int nt = min(kTileN, N - n0);
      const int row = m0 + q * 32 + lane;
      for (int c = 32 * h; c < nt; c += 64) {
        float v[32];
        const int w = min(32, nt - c);  // 32, or 16 at the end of a 16-wide tile
        if (w == 32)
          tc::tmem_ld32(tbase + lrow + (uint32_t)(b * kTileN + c), v);
        else
          tc::tmem_ld16(tbase + lrow + (uint32_t)(b * kTileN + c), v);
        if (row < M) {
          if (bias4) {
#pragma unroll
            for (int e = 0; e < 8; ++e) {
              if (4 * e < w) {
                const float4 bb = *reinterpret_cast<const float4*>(bias + n0 + c + 4 * e);
                v[4 * e] += bb.x; v[4 * e + 1] += bb.y; v[4 * e + 2] += bb.z; v[4 * e + 3] += bb.w;
              }
            }
          } else if (bias) {
#pragma unroll
            for (int e = 0; e < 32; ++e)
              if (e < w) v[e] += bias[n0 + c + e];
          }
#pragma unroll
          for (int g = 0; g < 2; ++g) {  // two 16-column halves
            if (16 * g >= w) break;
            const float* vg = v + 16 * g;
            const int cg = c + 16 * g;
            if (C) {
              float4* cp = reinterpret_cast<float4*>(C + (size_t)row * ldc + n0 + cg);
#pragma unroll
              for (int e = 0; e < 4; ++e) cp[e] = make_float4(vg[4 * e], vg[4 * e + 1], vg[4 * e + 2], vg[4 * e + 3]);
            }
            if (Ct) {  // transposed: the 32 lanes of a warp write 32 consecutive rows of C
#pragma unroll
              for (int e = 0; e < 16; ++e) Ct[(size_t)(n0 + cg + e) * ldct + row] = vg[e];
            }
            if (Cb) {
              uint32_t pk[8];
#pragma unroll
              for (int e = 0; e < 8; ++e) {
                float x0 = vg[2 * e], x1 = vg[2 * e + 1];
                if (act == ACT_SILU) {
                  x0 = silu(x0);
                  x1 = silu(x1);
                }
                const __nv_bfloat162 b2 = __floats2bfloat162_rn(x0, x1);
                pk[e] = *reinterpret_cast<const uint32_t*>(&b2);
              }
              uint4* bp = reinterpret_cast<uint4*>(Cb + (size_t)row * ldcb + n0 + cg);
              bp[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
              bp[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
            }
          }
        }
      }
      tc::tc_fence_before();
      tc::mbar_arrive(&acc_empty[b]);
    }
  }
  __syncthreads();
  if (tid == 0) {
    // every MMA has completed before TMEM is released; loads still in
    // flight after a failed wait are drained (all waits bounded)
    if (!tc::mbar_wait_cycles(&done, 0, lim)) s_fail = 1;
    if (s_fail) {
      atomicExch(&g_tc_error, 1);
      for (int it = s_consumed; it < s_issued; ++it) tc::mbar_wait_cycles(&full[it % kStages], (it / kStages) & 1, lim);
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (warp == 0) tc::tmem_dealloc(tbase, 512);
}

// ---- host side -------------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  });
  return fn;
}

// BF16 row-major [rows][cols] (ld elements) as a TMA map with box
// [box_rows][64], 128-byte swizzle, zero fill outside
static bool make_map(CUtensorMap* m, const void* base, int rows, int cols, int ld, int box_rows) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kChunkK, (cuuint32_t)box_rows};
  const cuuint32_t es[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

static int num_sms() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

static void gemm_attr() {
  static std::once_flag once;
  std::call_once(once, [] { cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem); });
}

// checks shapes, builds the two maps and launches; MOLOCH_OK or an error code
static int launch_gemm(const void* A, int lda, const void* B, int ldb, float* C, int ldc, void* Cb, int ldcb,
                       const float* bias, int M, int N, int K, int act, cudaStream_t st,
                       const int* run = nullptr, float* Ct = nullptr, int ldct = 0) {
  if (!A || !B || (!C && !Cb && !Ct) || M <= 0 || N <= 0 || K <= 0 || (Ct && ldct < M)) {
    moloch_internal_set_error("tc_gemm: bad arguments");
    return MOLOCH_ERR_ARG;
  }
  if (N % 16 || K % kChunkK || lda % 8 || ldb % 8 || lda < K || ldb < K || (C && (ldc < N || ldc % 4)) ||
      (Cb && (ldcb < N || ldcb % 8)) || ((uintptr_t)A | (uintptr_t)B) % 16 || ((uintptr_t)C % 16) ||
      ((uintptr_t)Cb % 16)) {
    moloch_internal_set_error("tc_gemm: need N % 16 == 0, K % 64 == 0, 16-byte aligned rows");
    return MOLOCH_ERR_ARG;
  }
  gemm_attr();
  const int boxB = N < kTileN ? N : kTileN;
  CUtensorMap ta, tb;
  if (!make_map(&ta, A, M, K, lda, kTileM) || !make_map(&tb, B, N, K, ldb, boxB)) {
    moloch_internal_set_error("tc_gemm: cuTensorMapEncodeTiled failed");
    return MOLOCH_ERR_CUDA;
  }
  const int ntiles = ((M + kTileM - 1) / kTileM) * ((N + kTileN - 1) / kTileN);
  k_gemm_tc<<<std::min(ntiles, num_sms()), kThreads, kSmem, st>>>(ta, tb, boxB, C, ldc, (__nv_bfloat16*)Cb, ldcb,
                                                                   bias, M, N, K, act, run, Ct, ldct);
  return MOLOCH_OK;
}

}  // namespace mlp
}  // namespace moloch

using namespace moloch::mlp;

// GEMM on device buffers for the surrogate and its tests.
extern "C" int moloch_tc_gemm(const void* A, int lda, const void* B, int ldb, float* C, int ldc, void* Cb, int ldcb,
                              const float* bias, int M, int N, int K, int act, void* stream) {
  int rc = launch_gemm(A, lda, B, ldb, C, ldc, Cb, ldcb, bias, M, N, K, act, (cudaStream_t)stream);
  if (rc) return rc;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    moloch_internal_set_error(cudaGetErrorString(e));
    return MOLOCH_ERR_CUDA;
  }
  return MOLOCH_OK;
}

// Limit of the GEMM's mbarrier waits (SM cycles, <= 0: the default) and the
// test hook that leaves one K chunk of one CTA unissued (-1: off).
extern "C" int moloch_tc_set_wait_limit(long long cycles, int skip_cta, int skip_chunk) {
  const long long c = cycles > 0 ? cycles : moloch::kDefaultSpinCycles;
  if (cudaMemcpyToSymbol(g_tc_spin, &c, sizeof(c)) != cudaSuccess ||
      cudaMemcpyToSymbol(g_tc_skip_cta, &skip_cta, sizeof(int)) != cudaSuccess ||
      cudaMemcpyToSymbol(g_tc_skip_it, &skip_chunk, sizeof(int)) != cudaSuccess) {
    moloch_internal_set_error("tc_set_wait_limit: cudaMemcpyToSymbol failed");
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

// =========================================================================
// Surrogate of one acoustic cycle (sound(), nompi/mod_moloch.F90:483-851)
// =========================================================================
#include "moloch_sur.h"

namespace moloch {
namespace mlp {

// value of field f (u, v, w levels 2..kz+1, pai, tetav) at (j, i, level k)
__device__ __forceinline__ float sur_field(const View<float>& d, int f, int j, int i, int k) {
  const size_t q = (size_t)j + (size_t)d.nj * i + (size_t)k * d.pl;
  switch (f) {
    case 0: return d.ubuf[d.cur][q];
    case 1: return d.vbuf[d.cur][q];
    case 2: return d.w[q + d.pl];
    case 3: return d.pai[q];
    default: return d.tetav[q];
  }
}

// Features of ncols columns (cols == nullptr: all columns in order).  Feature
// index (f * kz + k) * 9 + nb: field f (u, v, w levels 2..kz+1, pai,
// tetav), level k, neighbour nb = (di + 1) * 3 + (dj + 1) fastest.  Work
// items of 128 columns x one 64-feature chunk (ldo / 64 chunks per column),
// one thread per column, blocks looping over the items.  A chunk starting
// at feature f0 covers at most 8 field planes, and where each of its 64
// features sits (plane, neighbour) depends only on f0 % 9: one fully
// unrolled body per value of f0 % 9 keeps the plane pointers, the nine
// neighbour offsets and the 64 values in registers, all 64 loads issued
// before any is used (the planes come from HBM; the 9 neighbours of
// consecutive columns hit L1).  The 128 rows of the item are staged in
// shared memory and leave as whole 128-byte (BF16) or 256-byte (FP32) row
// segments, 8 or 16 threads per row.  NORM: normalise with the dataset
// statistics and write BF16; else write raw FP32.
// row strides of the staging tile, in 32-bit words: 144 B (BF16 rows of
// 64 features + 16 B) and 272 B (FP32 rows + 16 B), so that the eight
// 16-byte stores of a quarter warp land in distinct banks
constexpr int kStageBf = 36, kStageF32 = 68;

template <bool NORM, int OFF>
__device__ __forceinline__ void feature_item(const float* const (&pp)[8], const float (&sub)[8],
                                             const float (&mul)[8], const int (&nbo)[9], bool valid, int np_rel,
                                             uint32_t* stage_row) {
  float val[64];
#pragma unroll
  for (int r = 0; r < 64; ++r) {
    const int pr = (OFF + r) / 9, nb = (OFF + r) % 9;
    val[r] = (valid && pr < np_rel) ? __ldg(pp[pr] + nbo[nb]) : 0.f;
  }
  if (!valid) return;
  if (NORM) {
    uint32_t pk[32];
#pragma unroll
    for (int e = 0; e < 32; ++e) {
      const int r0 = 2 * e, r1 = 2 * e + 1;
      const int p0 = (OFF + r0) / 9, p1 = (OFF + r1) / 9;
      const float x0 = p0 < np_rel ? (val[r0] - sub[p0]) * mul[p0] : 0.f;
      const float x1 = p1 < np_rel ? (val[r1] - sub[p1]) * mul[p1] : 0.f;
      const __nv_bfloat162 b2 = __floats2bfloat162_rn(x0, x1);
      pk[e] = *reinterpret_cast<const uint32_t*>(&b2);
    }
    uint4* dst = reinterpret_cast<uint4*>(stage_row);
#pragma unroll
    for (int e = 0; e < 8; ++e) dst[e] = make_uint4(pk[4 * e], pk[4 * e + 1], pk[4 * e + 2], pk[4 * e + 3]);
  } else {
    float4* dst = reinterpret_cast<float4*>(stage_row);
#pragma unroll
    for (int e = 0; e < 16; ++e) dst[e] = make_float4(val[4 * e], val[4 * e + 1], val[4 * e + 2], val[4 * e + 3]);
  }
}

template <bool NORM>
__global__ void __launch_bounds__(128) k_sur_features(View<float> d, const int* __restrict__ cols, int ncols,
                                                      const float* __restrict__ xmean, const float* __restrict__ xstd,
                                                      void* out, int ldo, const int* __restrict__ run) {
  if (run && !*run) return;
  __shared__ __align__(16) uint32_t stage[128 * kStageF32];  // the item's 128 output rows
  const int t = threadIdx.x;
  const int kz = d.kz, np = 5 * kz;  // field planes
  const int srow = NORM ? kStageBf : kStageF32;
  const int ntile = (ncols + 127) / 128, items = ntile * (ldo / 64);
  // work items (column tile, 64-feature chunk), the column tile fastest
  for (int item = blockIdx.x; item < items; item += gridDim.x) {
    const int c0 = (item % ntile) * 128;
    const int cidx = c0 + t;
    const int f0 = (item / ntile) * 64;
    const bool valid = cidx < ncols;
    int nbo[9];
    {
      int j = 0, i = 0;
      if (valid) {
        const int col = cols ? cols[cidx] : cidx;
        j = col % d.nj;
        i = col / d.nj;
      }
      const int jm = j == 0 ? d.nj - 1 : j - 1, jp = j == d.nj - 1 ? 0 : j + 1;
      const int im = i == 0 ? d.ni - 1 : i - 1, ip = i == d.ni - 1 ? 0 : i + 1;
      const int jj[3] = {jm, j, jp}, ii[3] = {im, i, ip};
#pragma unroll
      for (int nb = 0; nb < 9; ++nb) nbo[nb] = jj[nb % 3] + d.nj * ii[nb / 3];
    }
    const int p0 = f0 / 9, off = f0 - 9 * p0;
    const int np_rel = np - p0;  // planes of this chunk that exist (the rest is padding)
    const float* pp[8];
    float sub[8], mul[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const int plane = p0 + q < np ? p0 + q : np - 1;
      const int fld = plane / kz, k = plane - fld * kz;
      const float* b = fld == 0 ? d.ubuf[d.cur] : fld == 1 ? d.vbuf[d.cur] : fld == 2 ? d.w + d.pl
                     : fld == 3 ? d.pai : d.tetav;
      pp[q] = b + (size_t)k * d.pl;
      if (NORM) {
        sub[q] = xmean[plane];
        mul[q] = 1.0f / xstd[plane];
      } else {
        sub[q] = 0.f;
        mul[q] = 1.f;
      }
    }
    uint32_t* const row = stage + t * srow;
    switch (off) {
      case 0: feature_item<NORM, 0>(pp, sub, mul, nbo, valid, np_rel, row); break;
      case 1: feature_item<NORM, 1>(pp, sub, mul, nbo, valid, np_rel, row); break;
      case 2: feature_item<NORM, 2>(pp, sub, mul, nbo, valid, np_rel, row); break;
      case 3: feature_item<NORM, 3>(pp, sub, mul, nbo, valid, np_rel, row); break;
      case 4: feature_item<NORM, 4>(pp, sub, mul, nbo, valid, np_rel, row); break;
      case 5: feature_item<NORM, 5>(pp, sub, mul, nbo, valid, np_rel, row); break;
      case 6: feature_item<NORM, 6>(pp, sub, mul, nbo, valid, np_rel, row); break;
      case 7: feature_item<NORM, 7>(pp, sub, mul, nbo, valid, np_rel, row); break;
      default: feature_item<NORM, 8>(pp, sub, mul, nbo, valid, np_rel, row); break;
    }
    __syncthreads();
    // the staged rows leave as whole 128-byte (BF16) / 256-byte (FP32)
    // segments, 16 bytes per thread, 8 or 16 threads per row
    if (NORM) {
      for (int q = t; q < 128 * 8; q += 128) {
        const int rr = q >> 3, part = q & 7;
        if (c0 + rr < ncols)
          *reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(out) + (size_t)(c0 + rr) * ldo + f0 + part * 8) =
              *reinterpret_cast<const uint4*>(stage + rr * kStageBf + part * 4);
      }
    } else {
      for (int q = t; q < 128 * 16; q += 128) {
        const int rr = q >> 4, part = q & 15;
        if (c0 + rr < ncols)
          *reinterpret_cast<uint4*>(reinterpret_cast<float*>(out) + (size_t)(c0 + rr) * ldo + f0 + part * 4) =
              *reinterpret_cast<const uint4*>(stage + rr * kStageF32 + part * 4);
      }
    }
    __syncthreads();
  }
}

// centre-column values of the five fields (5 * kz per column)
__global__ void k_sur_snapshot(View<float> d, const int* __restrict__ cols, int ncols, float* __restrict__ snap) {
  const int c = blockIdx.x, t = threadIdx.x, kz = d.kz;
  if (c >= ncols) return;
  const int col = cols[c];
  const int j = col % d.nj, i = col / d.nj;
  for (int q = t; q < 5 * kz; q += blockDim.x) snap[(size_t)c * 5 * kz + q] = sur_field(d, q / kz, j, i, q % kz);
}

// raw increments (post - pre) into T [ncols][ldt]
__global__ void k_sur_increment(View<float> d, const int* __restrict__ cols, int ncols, const float* __restrict__ snap,
                                float* __restrict__ T, int ldt) {
  const int c = blockIdx.x, t = threadIdx.x, kz = d.kz;
  if (c >= ncols) return;
  const int col = cols[c];
  const int j = col % d.nj, i = col / d.nj;
  for (int q = t; q < ldt; q += blockDim.x)
    T[(size_t)c * ldt + q] = q < 5 * kz ? sur_field(d, q / kz, j, i, q % kz) - snap[(size_t)c * 5 * kz + q] : 0.f;
}

// in-place normalisation of a row-major [n][ld] FP32 array (the first m
// columns; column c uses statistic c / group), with optional BF16 copy
__global__ void k_sur_normalize(float* __restrict__ a, int n, int ld, int m, const float* __restrict__ mean,
                                const float* __restrict__ stdv, __nv_bfloat16* __restrict__ ab, int group) {
  const size_t tot = (size_t)n * ld;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < tot; q += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(q % ld);
    float v = a[q];
    if (c < m) {
      const int s = c / group;
      v = stdv[s] > 0.f ? (v - mean[s]) / stdv[s] : 0.f;  // zero spread: the output is its mean
    } else {
      v = 0.f;
    }
    a[q] = v;
    if (ab) ab[q] = __float2bfloat16_rn(v);
  }
}

// out[c][r] = in[r][c] for BF16 [rows][cols] (ld_in) -> [cols][rows] (ld_out)
template <class TI>
__global__ void k_transpose_bf16(const TI* __restrict__ in, int rows, int cols, int ld_in,
                                 __nv_bfloat16* __restrict__ out, int ld_out) {
  __shared__ float t[32][33];
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int r = r0 + y, c = c0 + threadIdx.x;
    t[y][threadIdx.x] = (r < rows && c < cols) ? (float)in[(size_t)r * ld_in + c] : 0.f;
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += blockDim.y) {
    const int c = c0 + y, r = r0 + threadIdx.x;
    if (c < cols && r < rows) out[(size_t)c * ld_out + r] = __float2bfloat16_rn(t[threadIdx.x][y]);
  }
}

// MSE gradient: dY = 2 (Y - T) / (n * m) over the first m columns (zero in
// the padding), BF16; the block's sum of squared errors into lpart[block]
// (summed in a fixed order by k_sum_parts, so the reported loss does not
// depend on the order blocks finish in).  256 threads per block.
__global__ void __launch_bounds__(256) k_sur_loss_grad(const float* __restrict__ Y, const float* __restrict__ T, int n,
                                                       int ld, int m, __nv_bfloat16* __restrict__ dY,
                                                       float* __restrict__ lpart) {
  __shared__ float wsum[8];
  float acc = 0.f;
  const float sc = 2.0f / ((float)n * (float)m);
  const size_t tot = (size_t)n * ld;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < tot; q += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(q % ld);
    float g = 0.f;
    if (c < m) {
      const float e = Y[q] - T[q];
      acc += e * e;
      g = sc * e;
    }
    dY[q] = __float2bfloat16_rn(g);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    float b = 0.f;
    for (int w = 0; w < 8; ++w) b += wsum[w];
    lpart[blockIdx.x] = b;
  }
}

// *out = sum of part[0 .. n), in a fixed order (one block of 256 threads)
__global__ void __launch_bounds__(256) k_sum_parts(const float* __restrict__ part, int n, float* __restrict__ out) {
  __shared__ float red[256];
  float v = 0.f;
  for (int b = threadIdx.x; b < n; b += 256) v += part[b];
  red[threadIdx.x] = v;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// dZ = dH * silu'(Z), BF16
__global__ void k_silu_backward(const float* __restrict__ dH, const float* __restrict__ Z, size_t n,
                                __nv_bfloat16* __restrict__ dZ) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const float z = Z[q], sg = 1.0f / (1.0f + __expf(-z));
    dZ[q] = __float2bfloat16_rn(dH[q] * (sg * (1.0f + z * (1.0f - sg))));
  }
}

// column sums of a BF16 [n][ld] matrix (bias gradients), first m columns
__global__ void k_colsum_bf16(const __nv_bfloat16* __restrict__ a, int n, int ld, int m, float* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m) return;
  float s = 0.f;
  for (int r = 0; r < n; ++r) s += __bfloat162float(a[(size_t)r * ld + c]);
  out[c] = s;
}

// Adam on an [rows][cols] FP32 master matrix; refreshes the BF16 copy and
// (if WT) its transpose [cols][ldt]
__global__ void k_adam(float* __restrict__ W, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       int rows, int cols, float lr, float b1, float b2, float eps, float c1, float c2,
                       __nv_bfloat16* __restrict__ Wb, __nv_bfloat16* __restrict__ WT, int ldt) {
  const size_t tot = (size_t)rows * cols;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < tot; q += (size_t)gridDim.x * blockDim.x) {
    const float gg = g[q];
    const float mm = b1 * m[q] + (1.f - b1) * gg;
    const float vv = b2 * v[q] + (1.f - b2) * gg * gg;
    m[q] = mm;
    v[q] = vv;
    const float w = W[q] - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    W[q] = w;
    if (Wb) Wb[q] = __float2bfloat16_rn(w);
    if (WT) {
      const int r = (int)(q / cols), c = (int)(q % cols);
      WT[(size_t)c * ldt + r] = __float2bfloat16_rn(w);
    }
  }
}

// ---- control of a surrogate cycle (all decisions on the device, so that a
// whole step stays one captured graph).  Control block `ctl`:
//   [0] flag       1: the surrogate's increments are committed this cycle
//                  and the plain substeps return at once (their skip flag)
//   [1] bad        set by k_sur_check
//   [2] cycle      sound() calls seen since attach
//   [3] judge      1: this cycle is a judge cycle
//   [4] enabled    verdict of the last judge cycle
//   [5] maxratio   largest |y| / envelope seen since attach (float bits)
//   [6] lasterr    error of the last judge cycle (float bits)
//   [7] run        1: the inference runs this cycle (enabled or judge)
//   [8] nextjudge  cycle of the next judge
//   [9] interval   cycles from this judge to the next one
// counts: [0] cycles, [1] cycles run by the plain loop, [2] judge cycles,
// [3] judge cycles that disabled the surrogate.
// A judge cycle runs both the inference and the plain sound loop, and the
// plain loop judges the prediction: the relative RMS error of the
// increments, worst of the five fields, must be <= tol.  After a passing
// verdict the next judge comes judge_every cycles later; after a failing
// one the surrogate is off (no inference at all) and the interval doubles,
// up to max_interval cycles.
enum {
  CTL_FLAG = 0, CTL_BAD, CTL_CYCLE, CTL_JUDGE, CTL_ENABLED, CTL_MAXRATIO, CTL_LASTERR, CTL_RUN, CTL_NEXTJUDGE,
  CTL_INTERVAL, CTL_COUNT = 32
};

__global__ void k_sur_begin(int* __restrict__ ctl, int judge_every) {
  const int cyc = ctl[CTL_CYCLE]++;
  const int judge = judge_every > 0 && cyc == ctl[CTL_NEXTJUDGE];
  ctl[CTL_JUDGE] = judge;
  ctl[CTL_RUN] = judge || ctl[CTL_ENABLED];
  ctl[CTL_BAD] = 0;
}

// every increment finite and within threshold x the envelope of the
// training targets (per output, normalised units); tracks the largest ratio
// (Y output-major: [outputs][n]; grid.y strides over outputs, grid.x over
// columns: a small fixed grid, so that a cycle without inference pays for
// few empty blocks)
__global__ void k_sur_check(const float* __restrict__ Y, int n, int ld, int m, const float* __restrict__ env,
                            float threshold, int* __restrict__ ctl, const int* __restrict__ run) {
  if (run && !*run) return;
  int b = 0;
  float rmax = 0.f;
  for (int o = blockIdx.y; o < m; o += gridDim.y) {
    const float lim = threshold * env[o];
    const float rcp_env = 1.0f / env[o];
    const float* __restrict__ yo = Y + (size_t)o * n;
    const int stride = gridDim.x * blockDim.x;
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    auto take = [&](float y) {
      if (!(y <= lim)) b = 1;  // also catches NaN
      rmax = y == y ? fmaxf(rmax, y * rcp_env) : __int_as_float(0x7f800000);
    };
    for (; c + 7 * stride < n; c += 8 * stride) {  // eight independent loads in flight
      float y[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) y[u] = fabsf(yo[c + u * stride]);
#pragma unroll
      for (int u = 0; u < 8; ++u) take(y[u]);
    }
    for (; c < n; c += stride) take(fabsf(yo[c]));
  }
  for (int q = 16; q > 0; q >>= 1) rmax = fmaxf(rmax, __shfl_xor_sync(0xffffffffu, rmax, q));
  if (__any_sync(0xffffffffu, b) && (threadIdx.x & 31) == 0) atomicOr(&ctl[CTL_BAD], 1);
  if ((threadIdx.x & 31) == 0) atomicMax(&ctl[CTL_MAXRATIO], __float_as_int(rmax));
}

__global__ void k_sur_decide(int* __restrict__ ctl, unsigned long long* __restrict__ counts) {
  const int use = ctl[CTL_RUN] && ctl[CTL_ENABLED] && !ctl[CTL_BAD] && !ctl[CTL_JUDGE];
  ctl[CTL_FLAG] = use;
  counts[0] += 1;
  if (!use) counts[1] += 1;
}

// judge cycles: copy of the pre-cycle state of the five fields
__global__ void k_sur_judge_snapshot(View<float> d, const int* __restrict__ ctl, float* __restrict__ snap) {
  if (!ctl[CTL_JUDGE]) return;
  const size_t n = (size_t)d.pl * d.kz;
  const float* src[5] = {d.ubuf[d.cur], d.vbuf[d.cur], d.w + d.pl, d.pai, d.tetav};
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < 5 * n; q += (size_t)gridDim.x * blockDim.x) {
    const int f = (int)(q / n);
    snap[q] = src[f][q - (size_t)f * n];
  }
}

// judge cycles, after the plain loop: sums of (predicted - actual)^2 and
// actual^2 of the increments, per field; block b writes its ten partial
// sums to jacc[10 b ..], which k_sur_verdict adds in a fixed order (no
// atomics: the verdict of a cycle near the tolerance must not depend on the
// order in which blocks finish)
__global__ void __launch_bounds__(256) k_sur_judge(View<float> d, const int* __restrict__ ctl,
                                                   const float* __restrict__ snap, const float* __restrict__ Y, int ld,
                                                   const float* __restrict__ ymean, const float* __restrict__ ystd,
                                                   double* __restrict__ jacc) {
  if (!ctl[CTL_JUDGE]) return;
  const size_t pl = d.pl, n = pl * d.kz;
  const float* post[5] = {d.ubuf[d.cur], d.vbuf[d.cur], d.w + d.pl, d.pai, d.tetav};
  __shared__ double red[8][10];
  double acc[10];
#pragma unroll
  for (int q = 0; q < 10; ++q) acc[q] = 0.0;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x) {
    const int k = (int)(q / pl);
    const size_t c = q - (size_t)k * pl;
#pragma unroll
    for (int f = 0; f < 5; ++f) {
      const int o = f * d.kz + k;
      const float act = post[f][q] - snap[(size_t)f * n + q];
      const float pred = Y[(size_t)o * ld + c] * ystd[o] + ymean[o];  // output-major
      const float e = pred - act;
      acc[2 * f] += (double)e * e;
      acc[2 * f + 1] += (double)act * act;
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 10; ++q) {
    double v = acc[q];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[wid][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < 10) {
    double v = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += red[w][threadIdx.x];
    jacc[(size_t)blockIdx.x * 10 + threadIdx.x] = v;
  }
}

// one block of 256 threads: the judge's per-block partial sums added in a
// fixed order (strided per thread, then a fixed tree), then the verdict
__global__ void __launch_bounds__(256) k_sur_verdict(int* __restrict__ ctl, const double* __restrict__ jpart,
                                                     int nparts, float tol, int judge_every, int max_interval,
                                                     unsigned long long* __restrict__ counts) {
  if (!ctl[CTL_JUDGE]) return;
  __shared__ double red[10][256];
  for (int q = 0; q < 10; ++q) {
    double v = 0.0;
    for (int b = threadIdx.x; b < nparts; b += blockDim.x) v += jpart[(size_t)b * 10 + q];
    red[q][threadIdx.x] = v;
  }
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h)
      for (int q = 0; q < 10; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x != 0) return;
  double jacc[10];
  for (int q = 0; q < 10; ++q) jacc[q] = red[q][0];
  double worst = 0.0;
  for (int f = 0; f < 5; ++f) {
    const double r = jacc[2 * f + 1] > 0.0 ? sqrt(jacc[2 * f] / jacc[2 * f + 1]) : (jacc[2 * f] > 0.0 ? 1e30 : 0.0);
    worst = r == r ? fmax(worst, r) : 1e30;
  }
  const int ok = worst <= (double)tol;
  ctl[CTL_ENABLED] = ok;
  ctl[CTL_LASTERR] = __float_as_int((float)worst);
  const int iv = ok ? judge_every : min(2 * ctl[CTL_INTERVAL], max_interval);
  ctl[CTL_INTERVAL] = iv;
  ctl[CTL_NEXTJUDGE] = ctl[CTL_CYCLE] - 1 + iv;  // counted from this (judge) cycle
  counts[2] += 1;
  if (!ok) counts[3] += 1;
}

// gather rows of a row-major array: out[r] = in[idx[r]]
template <class E>
__global__ void k_gather_rows(const E* __restrict__ in, const int* __restrict__ idx, int n, int ld, E* __restrict__ out) {
  const size_t tot = (size_t)n * ld;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < tot; q += (size_t)gridDim.x * blockDim.x) {
    const size_t r = q / ld, c = q % ld;
    out[q] = in[(size_t)idx[r] * ld + c];
  }
}

// Accepted cycle, part 1: generalised vertical velocity s (Equation 10,
// :557-570 and :843-849).  The reference evaluates the u, v part with the
// winds at the start of the last substep; they are taken as the pre-cycle
// winds plus (nsound - 1) / nsound of the predicted increment, and w is the
// new w.  Writes s only, so it runs before part 2 changes u, v, w.
__global__ void __launch_bounds__(256) k_sur_vvel(View<float> d, const float* __restrict__ Y, int ld,
                                                  const float* __restrict__ ymean, const float* __restrict__ ystd,
                                                  const int* __restrict__ ctl, int nsound) {
  if (!ctl[CTL_FLAG]) return;
  const int jj = blockIdx.x * 32 + threadIdx.x, ii = blockIdx.y * 8 + threadIdx.y;
  const int nj = d.nj, ni = d.ni, kz = d.kz;
  if (jj >= nj || ii >= ni) return;
  const size_t pl = d.pl, c = jj + (size_t)nj * ii;
  const int jp = jj == nj - 1 ? 0 : jj + 1, ip = ii == ni - 1 ? 0 : ii + 1;
  const size_t ce = jp + (size_t)nj * ii, cn = jj + (size_t)nj * ip;
  const float* __restrict__ u = d.ubuf[d.cur];
  const float* __restrict__ v = d.vbuf[d.cur];
  const float fr = (float)(nsound - 1) / (float)nsound;
  // Y output-major: output q of column col at Y[q * ld + col] (ld = columns)
  auto inc = [&](size_t col, int f, int k) { const int q = f * kz + k; return Y[(size_t)q * ld + col] * ystd[q] + ymean[q]; };
  auto ul = [&](size_t col, int k) { return u[col + k * pl] + fr * inc(col, 0, k); };
  auto vl = [&](size_t col, int k) { return v[col + k * pl] + fr * inc(col, 1, k); };
  const float hx0 = d.hx[c], hx1 = d.hx[ce], hy0 = d.hy[c], hy1 = d.hy[cn];
  d.s[c] = 0.f;
  d.s[c + (size_t)kz * pl] = 0.f;
  for (int k = 1; k < kz; ++k) {
    const size_t q = c + (size_t)k * pl;
    const float zuh = (ul(c, k) + ul(c, k - 1)) * hx0 + (ul(ce, k) + ul(ce, k - 1)) * hx1;
    const float zvh = (vl(c, k) + vl(c, k - 1)) * hy0 + (vl(cn, k) + vl(cn, k - 1)) * hy1;
    const float suv = -((0.25f * (zuh + zvh)) * d.gzitak[k]);
    const float wn = d.w[q] + inc(c, 2, k - 1);
    d.s[q] = (wn + suv) * d.fmzf[q];
  }
}

// Accepted cycle, part 2: state += denormalised increments, column by
// column; u, v go to the buffer the plain loop leaves them in (outpar: the
// parity of its buffer flips over the cycle).
__global__ void __launch_bounds__(256) k_sur_apply(View<float> d, const float* __restrict__ Y, int ld,
                                                   const float* __restrict__ ymean, const float* __restrict__ ystd,
                                                   const int* __restrict__ ctl, int outpar) {
  if (!ctl[CTL_FLAG]) return;
  const int jj = blockIdx.x * 32 + threadIdx.x, ii = blockIdx.y * 8 + threadIdx.y;
  const int nj = d.nj, ni = d.ni, kz = d.kz;
  if (jj >= nj || ii >= ni) return;
  const size_t pl = d.pl, c = jj + (size_t)nj * ii;
  const float* __restrict__ yr = Y + c;  // output-major: output q at yr[q * ld]
  const float* u = d.ubuf[d.cur];
  const float* v = d.vbuf[d.cur];
  float* uo = d.ubuf[d.cur ^ outpar];
  float* vo = d.vbuf[d.cur ^ outpar];
  auto inc = [&](int f, int k) { const int q = f * kz + k; return yr[(size_t)q * ld] * ystd[q] + ymean[q]; };
  for (int k = 0; k < kz; ++k) {
    const size_t q = c + (size_t)k * pl;
    uo[q] = u[q] + inc(0, k);
    vo[q] = v[q] + inc(1, k);
    d.w[q + pl] = d.w[q + pl] + inc(2, k);
    d.pai[q] = d.pai[q] + inc(3, k);
    d.tetav[q] = d.tetav[q] + inc(4, k);
  }
}

}  // namespace mlp
}  // namespace moloch

// =========================================================================
// Surrogate: host orchestration and C ABI
// =========================================================================
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

// accessors into a handle (moloch_api.cpp)
moloch::View<float>* moloch_internal_viewf(moloch_handle_t* h);
cudaStream_t moloch_internal_stream(moloch_handle_t* h);
int moloch_internal_nadv(moloch_handle_t* h);
int moloch_internal_nsound(moloch_handle_t* h);
int moloch_internal_attach(moloch_handle_t* h, moloch::mlp::Surrogate* s);

struct moloch_surrogate : moloch::mlp::Surrogate {};

namespace moloch {
namespace mlp {

static uint64_t sm64(uint64_t& st) {
  uint64_t z = (st += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static double u01h(uint64_t& st) { return (double)(sm64(st) >> 11) * (1.0 / 9007199254740992.0); }

#define SUR_TRY(x)                                                                     \
  do {                                                                                 \
    cudaError_t e_ = (x);                                                              \
    if (e_ != cudaSuccess) {                                                           \
      char b_[256];                                                                    \
      snprintf(b_, sizeof b_, "%s: %s", #x, cudaGetErrorString(e_));                   \
      moloch_internal_set_error(b_);                                                   \
      return MOLOCH_ERR_CUDA;                                                          \
    }                                                                                  \
  } while (0)

static int gemm(const void* A, int lda, const void* B, int ldb, float* C, int ldc, void* Cb, int ldcb,
                const float* bias, int M, int N, int K, int act, cudaStream_t st, const int* run = nullptr,
                float* Ct = nullptr, int ldct = 0) {
  launch_gemm(A, lda, B, ldb, C, ldc, Cb, ldcb, bias, M, N, K, act, st, run, Ct, ldct);
  return 1;
}

constexpr int kGrid1Max = 152 * 16;  // largest grid of the grid-stride kernels below
static int grid1(size_t n) { return (int)std::min<size_t>((n + 255) / 256, kGrid1Max); }
// k_sur_check: at most 16 x 38 blocks of 256 threads
static dim3 check_grid(int n, int m) { return dim3(std::min((n + 2047) / 2048, 16), std::min(m, 38)); }
// k_sur_features: work items of 128 columns x 64 features, one wave of
// blocks of 128 threads (5 per SM at 92 registers, 34 KB of shared memory)
// looping over the items
static dim3 feature_grid(int ncols, int kin) {
  const long items = (long)((ncols + 127) / 128) * (kin / 64);
  return dim3((unsigned)std::min<long>(items, 152 * 5));
}

static int transpose(const void* in, int rows, int cols, int ld_in, void* out, int ld_out, cudaStream_t st) {
  dim3 g((cols + 31) / 32, (rows + 31) / 32);
  k_transpose_bf16<__nv_bfloat16><<<g, dim3(32, 8), 0, st>>>((const __nv_bfloat16*)in, rows, cols, ld_in,
                                                             (__nv_bfloat16*)out, ld_out);
  return 1;
}

// forward of n rows: X -> H[0..2] (BF16, SiLU) -> Y (FP32); Z (pre-activations) optional
// Y [n][nop] row-major, or (Y == nullptr) Yt [nop][n] output-major
static int forward(Surrogate* s, const void* X, int n, void* const* H, float* const* Z, float* Y, cudaStream_t st,
                   const int* run = nullptr, float* Yt = nullptr) {
  const int hid = s->hid;
  gemm(X, s->kin, s->L[0].Wb, s->kin, Z ? Z[0] : nullptr, hid, H[0], hid, s->L[0].b, n, hid, s->kin, ACT_SILU, st, run);
  gemm(H[0], hid, s->L[1].Wb, hid, Z ? Z[1] : nullptr, hid, H[1], hid, s->L[1].b, n, hid, hid, ACT_SILU, st, run);
  gemm(H[1], hid, s->L[2].Wb, hid, Z ? Z[2] : nullptr, hid, H[2], hid, s->L[2].b, n, hid, hid, ACT_SILU, st, run);
  gemm(H[2], hid, s->L[3].Wb, hid, Y, s->nop, nullptr, 0, s->L[3].b, n, s->nop, hid, ACT_NONE, st, run, Yt, n);
  return 4;
}

// one backward pass for the batch in Xbat/Tbat after forward(Xbat, H, Z, Y):
// gradients into L[*].gW/gb, loss sum into *s->loss
static void backward(Surrogate* s, cudaStream_t st) {
  const int B = s->batch, hid = s->hid, nop = s->nop;
  const int lg = grid1((size_t)B * nop);
  k_sur_loss_grad<<<lg, 256, 0, st>>>(s->Y, s->Tbat, B, nop, s->nout, (__nv_bfloat16*)s->dY, s->lpart);
  k_sum_parts<<<1, 256, 0, st>>>(s->lpart, lg, s->loss);
  // layer 4: gW4 = dY^T H3, gb4 = colsum dY, dH3 = dY W4
  transpose(s->dY, B, nop, nop, s->dYT, B, st);
  transpose(s->H[2], B, hid, hid, s->HT[2], B, st);
  gemm(s->dYT, B, s->HT[2], B, s->L[3].gW, hid, nullptr, 0, nullptr, nop, hid, B, ACT_NONE, st);
  k_colsum_bf16<<<(nop + 255) / 256, 256, 0, st>>>((const __nv_bfloat16*)s->dY, B, nop, nop, s->L[3].gb);
  gemm(s->dY, nop, s->L[3].WT, nop, s->dH[2], hid, nullptr, 0, nullptr, B, hid, nop, ACT_NONE, st);
  // hidden layers 3, 2, 1
  for (int l = 2; l >= 0; --l) {
    k_silu_backward<<<grid1((size_t)B * hid), 256, 0, st>>>(s->dH[l], s->Z[l], (size_t)B * hid, (__nv_bfloat16*)s->dZ[l]);
    transpose(s->dZ[l], B, hid, hid, s->dZT[l], B, st);
    const void* inT;
    int kin_l;
    if (l > 0) {
      transpose(s->H[l - 1], B, hid, hid, s->HT[l - 1], B, st);
      inT = s->HT[l - 1];
      kin_l = hid;
    } else {
      transpose(s->Xbat, B, s->kin, s->kin, s->XbatT, B, st);
      inT = s->XbatT;
      kin_l = s->kin;
    }
    gemm(s->dZT[l], B, inT, B, s->L[l].gW, kin_l, nullptr, 0, nullptr, hid, kin_l, B, ACT_NONE, st);
    k_colsum_bf16<<<(hid + 255) / 256, 256, 0, st>>>((const __nv_bfloat16*)s->dZ[l], B, hid, hid, s->L[l].gb);
    if (l > 0) gemm(s->dZ[l], hid, s->L[l].WT, hid, s->dH[l - 1], hid, nullptr, 0, nullptr, B, hid, hid, ACT_NONE, st);
  }
}

static void adam_all(Surrogate* s, float lr, int t, cudaStream_t st) {
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f - powf(b1, (float)t), c2 = 1.f - powf(b2, (float)t);
  for (int l = 0; l < 4; ++l) {
    SurLayer& L = s->L[l];
    k_adam<<<grid1((size_t)L.out * L.in), 256, 0, st>>>(L.W, L.gW, L.mW, L.vW, L.out, L.in, lr, b1, b2, eps, c1, c2,
                                                      (__nv_bfloat16*)L.Wb, (__nv_bfloat16*)L.WT, L.out);
    k_adam<<<grid1(L.out), 256, 0, st>>>(L.b, L.gb, L.mb, L.vb, 1, L.out, lr, b1, b2, eps, c1, c2, nullptr, nullptr, 0);
  }
}

int sur_cycle(Surrogate* s, View<float>& v, cudaStream_t st, int nsound, int outpar) {
  const int n = v.nj * v.ni;
  k_sur_begin<<<1, 1, 0, st>>>(s->ctl, s->judge_every);
  const int* run = s->ctl + CTL_RUN;
  k_sur_features<true><<<feature_grid(n, s->kin), 128, 0, st>>>(v, nullptr, n, s->xmean, s->xstd, s->Xinf,
                                                                          s->kin, run);
  forward(s, s->Xinf, n, s->Hinf, nullptr, nullptr, st, run, s->Yinf);  // Yinf output-major
  k_sur_check<<<check_grid(n, s->nout), 256, 0, st>>>(s->Yinf, n, s->nop, s->nout, s->env, s->threshold,
                                                                 s->ctl, run);
  k_sur_decide<<<1, 1, 0, st>>>(s->ctl, s->counts);
  k_sur_judge_snapshot<<<grid1((size_t)5 * n * v.kz), 256, 0, st>>>(v, s->ctl, s->jsnap);
  const dim3 cg((v.nj + 31) / 32, (v.ni + 7) / 8);
  k_sur_vvel<<<cg, dim3(32, 8), 0, st>>>(v, s->Yinf, n, s->ymean, s->ystd, s->ctl, nsound);
  k_sur_apply<<<cg, dim3(32, 8), 0, st>>>(v, s->Yinf, n, s->ymean, s->ystd, s->ctl, outpar);
  return 11;
}

int sur_after(Surrogate* s, View<float>& v, cudaStream_t st) {
  const size_t n = (size_t)v.nj * v.ni * v.kz;
  k_sur_judge<<<grid1(n), 256, 0, st>>>(v, s->ctl, s->jsnap, s->Yinf, v.nj * v.ni, s->ymean, s->ystd, s->jacc);
  k_sur_verdict<<<1, 256, 0, st>>>(s->ctl, s->jacc, grid1(n), s->tol, s->judge_every, s->max_interval, s->counts);
  return 2;
}

static void free_sur(Surrogate* s) {
  auto F = [](void* p) { if (p) cudaFree(p); };
  for (auto& L : s->L) {
    F(L.W); F(L.b); F(L.gW); F(L.gb); F(L.mW); F(L.vW); F(L.mb); F(L.vb); F(L.Wb); F(L.WT);
  }
  F(s->xmean); F(s->xstd); F(s->ymean); F(s->ystd); F(s->Xraw); F(s->Xb); F(s->T); F(s->snap); F(s->cols);
  F(s->Xbat); F(s->XbatT); F(s->Tbat); F(s->Y); F(s->dY); F(s->dYT); F(s->loss); F(s->lpart); F(s->perm);
  for (int l = 0; l < 3; ++l) { F(s->H[l]); F(s->HT[l]); F(s->Z[l]); F(s->dH[l]); F(s->dZ[l]); F(s->dZT[l]); F(s->Hinf[l]); }
  F(s->Xinf); F(s->Yinf); F(s->ctl); F(s->counts); F(s->env); F(s->jacc); F(s->jsnap);
}

}  // namespace mlp
}  // namespace moloch

using namespace moloch::mlp;
using moloch::View;

extern "C" {

int moloch_sur_create(int kz, int capacity, int batch, unsigned long long seed, moloch_surrogate_t** out) {
  if (!out || kz < 4 || capacity < 64 || batch < 64 || batch % 64) {
    moloch_internal_set_error("sur_create: kz >= 4, capacity >= 64, batch a positive multiple of 64");
    return MOLOCH_ERR_ARG;
  }
  *out = nullptr;
  gemm_attr();  // before any capture of a step that runs the GEMM
  if (!encode_fn()) {
    moloch_internal_set_error("sur_create: cuTensorMapEncodeTiled unavailable");
    return MOLOCH_ERR_CUDA;
  }
  moloch_surrogate* s = new moloch_surrogate();
  s->kz = kz;
  s->nin = 45 * kz;
  s->kin = (s->nin + 63) / 64 * 64;
  s->nout = 5 * kz;
  s->nop = (s->nout + 63) / 64 * 64;
  s->cap = capacity;
  s->batch = batch;
  s->max_cols = 4096;
  const int hid = s->hid;
  const int ins[4] = {s->kin, hid, hid, hid}, outs[4] = {hid, hid, hid, s->nop};
  cudaError_t e = cudaSuccess;
  auto A = [&](void** p, size_t bytes) {
    if (e == cudaSuccess) e = cudaMalloc(p, bytes);
    if (e == cudaSuccess) e = cudaMemset(*p, 0, bytes);
  };
  uint64_t st = seed ? seed : 0x5EED;
  for (int l = 0; l < 4; ++l) {
    SurLayer& L = s->L[l];
    L.in = ins[l];
    L.out = outs[l];
    const size_t nw = (size_t)L.in * L.out;
    A((void**)&L.W, nw * 4); A((void**)&L.gW, nw * 4); A((void**)&L.mW, nw * 4); A((void**)&L.vW, nw * 4);
    A((void**)&L.b, L.out * 4); A((void**)&L.gb, L.out * 4); A((void**)&L.mb, L.out * 4); A((void**)&L.vb, L.out * 4);
    A(&L.Wb, nw * 2); A(&L.WT, nw * 2);
    if (e == cudaSuccess) {  // Glorot-uniform init (last layer scaled down)
      std::vector<float> w(nw);
      const int fan_in = l == 0 ? s->nin : L.in;
      const double a = std::sqrt(6.0 / (fan_in + L.out)) * (l == 3 ? 0.1 : 1.0);
      for (size_t q = 0; q < nw; ++q) {
        const int c = (int)(q % L.in);
        w[q] = (l == 0 && c >= s->nin) ? 0.f : (float)((2.0 * u01h(st) - 1.0) * a);
      }
      e = cudaMemcpy(L.W, w.data(), nw * 4, cudaMemcpyHostToDevice);
    }
  }
  const int n5 = 5 * kz;
  A((void**)&s->xmean, n5 * 4); A((void**)&s->xstd, n5 * 4); A((void**)&s->ymean, n5 * 4); A((void**)&s->ystd, n5 * 4);
  A((void**)&s->Xraw, (size_t)capacity * s->kin * 4);
  A(&s->Xb, (size_t)capacity * s->kin * 2);
  A((void**)&s->T, (size_t)capacity * s->nop * 4);
  A((void**)&s->snap, (size_t)s->max_cols * n5 * 4);
  A((void**)&s->cols, (size_t)s->max_cols * 4);
  A(&s->Xbat, (size_t)batch * s->kin * 2); A(&s->XbatT, (size_t)batch * s->kin * 2);
  A((void**)&s->Tbat, (size_t)batch * s->nop * 4); A((void**)&s->Y, (size_t)batch * s->nop * 4);
  A(&s->dY, (size_t)batch * s->nop * 2); A(&s->dYT, (size_t)batch * s->nop * 2);
  A((void**)&s->loss, 16); A((void**)&s->lpart, sizeof(float) * kGrid1Max); A((void**)&s->perm, (size_t)capacity * 4);
  for (int l = 0; l < 3; ++l) {
    A(&s->H[l], (size_t)batch * hid * 2); A(&s->HT[l], (size_t)batch * hid * 2);
    A((void**)&s->Z[l], (size_t)batch * hid * 4); A((void**)&s->dH[l], (size_t)batch * hid * 4);
    A(&s->dZ[l], (size_t)batch * hid * 2); A(&s->dZT[l], (size_t)batch * hid * 2);
  }
  A((void**)&s->ctl, CTL_COUNT * sizeof(int)); A((void**)&s->counts, 4 * sizeof(unsigned long long));
  A((void**)&s->jacc, (size_t)kGrid1Max * 10 * sizeof(double));  // per-block judge sums
  A((void**)&s->env, (size_t)s->nop * 4);
  if (e == cudaSuccess) {  // envelope 1 until moloch_sur_prepare measures it
    std::vector<float> one(s->nop, 1.f);
    e = cudaMemcpy(s->env, one.data(), s->nop * 4, cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) {  // BF16 copies of the initial weights: an Adam step with zero gradient
    adam_all(s, 0.f, 1, 0);
    e = cudaDeviceSynchronize();
  }
  if (e != cudaSuccess) {
    free_sur(s);
    delete s;
    moloch_internal_set_error(cudaGetErrorString(e));
    return MOLOCH_ERR_NOMEM;
  }
  *out = s;
  return MOLOCH_OK;
}

int moloch_sur_collect(moloch_surrogate_t* s, moloch_handle_t* h, int nsteps, int cols_per_cycle,
                       unsigned long long seed) {
  if (!s || !h || nsteps < 0 || cols_per_cycle < 1 || cols_per_cycle > s->max_cols) {
    moloch_internal_set_error("sur_collect: bad arguments");
    return MOLOCH_ERR_ARG;
  }
  View<float>* vp = moloch_internal_viewf(h);
  if (!vp || vp->kz != s->kz) {
    moloch_internal_set_error("sur_collect: needs an initialized FP32-storage handle with the surrogate's kz");
    return MOLOCH_ERR_ARG;
  }
  cudaStream_t st = moloch_internal_stream(h);
  const int ncol = vp->nj * vp->ni, nadv = moloch_internal_nadv(h);
  uint64_t rs = seed ? seed : 99;
  std::vector<int> pick(cols_per_cycle);
  for (int step = 0; step < nsteps; ++step) {
    int rc = moloch_gpu_phase(h, 0);
    if (rc) return rc;
    for (int a = 0; a < nadv; ++a) {
      const int take = std::min(cols_per_cycle, s->cap - s->npairs);
      if (take > 0) {
        for (int q = 0; q < take; ++q) pick[q] = (int)(sm64(rs) % (uint64_t)ncol);
        SUR_TRY(cudaMemcpyAsync(s->cols, pick.data(), take * sizeof(int), cudaMemcpyHostToDevice, st));
        SUR_TRY(cudaStreamSynchronize(st));
        View<float>& v = *moloch_internal_viewf(h);
        k_sur_features<false><<<feature_grid(take, s->kin), 128, 0, st>>>(v, s->cols, take, nullptr, nullptr,
                                                                   s->Xraw + (size_t)s->npairs * s->kin, s->kin,
                                                                   nullptr);
        k_sur_snapshot<<<take, 128, 0, st>>>(v, s->cols, take, s->snap);
      }
      if ((rc = moloch_gpu_phase(h, 1))) return rc;
      if (take > 0) {
        View<float>& v = *moloch_internal_viewf(h);
        k_sur_increment<<<take, 128, 0, st>>>(v, s->cols, take, s->snap, s->T + (size_t)s->npairs * s->nop, s->nop);
        s->npairs += take;
      }
      if ((rc = moloch_gpu_phase(h, 2))) return rc;
    }
    if ((rc = moloch_gpu_phase(h, 3))) return rc;
  }
  SUR_TRY(cudaStreamSynchronize(st));
  SUR_TRY(cudaGetLastError());
  return MOLOCH_OK;
}

int moloch_sur_pairs(moloch_surrogate_t* s) { return s ? s->npairs : -1; }

int moloch_sur_pair_data(moloch_surrogate_t* s, int first, int count, float* X, float* T) {
  if (!s || first < 0 || count < 0 || first + count > s->npairs || (count && (!X || !T))) {
    moloch_internal_set_error("sur_pair_data: bad arguments");
    return MOLOCH_ERR_ARG;
  }
  if (!count) return MOLOCH_OK;
  SUR_TRY(cudaMemcpy2D(X, (size_t)s->nin * 4, s->Xraw + (size_t)first * s->kin, (size_t)s->kin * 4,
                       (size_t)s->nin * 4, count, cudaMemcpyDeviceToHost));
  SUR_TRY(cudaMemcpy2D(T, (size_t)s->nout * 4, s->T + (size_t)first * s->nop, (size_t)s->nop * 4,
                       (size_t)s->nout * 4, count, cudaMemcpyDeviceToHost));
  return MOLOCH_OK;
}

// normalisation statistics, normalised BF16 features, shuffle, split
int moloch_sur_prepare(moloch_surrogate_t* s, double val_fraction, unsigned long long seed) {
  if (!s || s->npairs < 2 * s->batch) {
    moloch_internal_set_error("sur_prepare: fewer than two batches of pairs");
    return MOLOCH_ERR_STATE;
  }
  const int n = s->npairs, kz = s->kz, n5 = 5 * kz;
  std::vector<float> X((size_t)n * s->kin), T((size_t)n * s->nop);
  SUR_TRY(cudaMemcpy(X.data(), s->Xraw, X.size() * 4, cudaMemcpyDeviceToHost));
  SUR_TRY(cudaMemcpy(T.data(), s->T, T.size() * 4, cudaMemcpyDeviceToHost));
  std::vector<double> xs(n5, 0.0), xq(n5, 0.0), ys(n5, 0.0), yq(n5, 0.0);
  for (int p = 0; p < n; ++p) {
    const float* xr = &X[(size_t)p * s->kin];
    for (int f = 0; f < s->nin; ++f) { const double x = xr[f]; xs[f / 9] += x; xq[f / 9] += x * x; }
    const float* tr = &T[(size_t)p * s->nop];
    for (int q = 0; q < n5; ++q) { const double y = tr[q]; ys[q] += y; yq[q] += y * y; }
  }
  std::vector<float> xm(n5), xd(n5), ym(n5), yd(n5);
  const double nx = (double)n * 9.0;
  for (int q = 0; q < n5; ++q) {
    const double mx = xs[q] / nx, vx = std::max(xq[q] / nx - mx * mx, 0.0);
    const double my = ys[q] / n, vy = std::max(yq[q] / n - my * my, 0.0);
    xm[q] = (float)mx;
    xd[q] = (float)(std::sqrt(vx) > 1e-12 * std::max(1.0, std::fabs(mx)) ? std::sqrt(vx) : 1.0);
    ym[q] = (float)my;
    // an output that never changed in the training set (e.g. tetav at the
    // levels where the acoustic cycle leaves it alone) gets scale 0: its
    // prediction is its mean whatever the network says
    yd[q] = (float)(std::sqrt(vy) > 1e-20 ? std::sqrt(vy) : 0.0);
  }
  SUR_TRY(cudaMemcpy(s->xmean, xm.data(), n5 * 4, cudaMemcpyHostToDevice));
  SUR_TRY(cudaMemcpy(s->xstd, xd.data(), n5 * 4, cudaMemcpyHostToDevice));
  SUR_TRY(cudaMemcpy(s->ymean, ym.data(), n5 * 4, cudaMemcpyHostToDevice));
  SUR_TRY(cudaMemcpy(s->ystd, yd.data(), n5 * 4, cudaMemcpyHostToDevice));
  std::vector<float> env(s->nop, 1.f);  // largest |normalised target| per output
  for (int q = 0; q < n5; ++q) {
    if (!(yd[q] > 0.f)) {  // scale-0 outputs are not checked
      env[q] = 3.0e38f;
      continue;
    }
    double mx = 0.0;
    for (int p = 0; p < n; ++p) mx = std::max(mx, std::fabs((T[(size_t)p * s->nop + q] - ym[q]) / (double)yd[q]));
    env[q] = (float)std::max(mx, 1e-3);
  }
  SUR_TRY(cudaMemcpy(s->env, env.data(), s->nop * 4, cudaMemcpyHostToDevice));
  k_sur_normalize<<<grid1((size_t)n * s->kin), 256>>>(s->Xraw, n, s->kin, s->nin, s->xmean, s->xstd,
                                                      (__nv_bfloat16*)s->Xb, 9);
  k_sur_normalize<<<grid1((size_t)n * s->nop), 256>>>(s->T, n, s->nop, s->nout, s->ymean, s->ystd, nullptr, 1);
  // shuffle once, keep the tail as the validation split
  std::vector<int> perm(n);
  for (int q = 0; q < n; ++q) perm[q] = q;
  uint64_t rs = seed ? seed : 7;
  for (int q = n - 1; q > 0; --q) std::swap(perm[q], perm[(int)(sm64(rs) % (uint64_t)(q + 1))]);
  SUR_TRY(cudaMemcpy(s->perm, perm.data(), n * 4, cudaMemcpyHostToDevice));
  void *tx = nullptr, *tt = nullptr;
  SUR_TRY(cudaMalloc(&tx, (size_t)n * s->kin * 2));
  SUR_TRY(cudaMalloc(&tt, (size_t)n * s->nop * 4));
  k_gather_rows<__nv_bfloat16><<<grid1((size_t)n * s->kin), 256>>>((const __nv_bfloat16*)s->Xb, s->perm, n, s->kin,
                                                                   (__nv_bfloat16*)tx);
  k_gather_rows<float><<<grid1((size_t)n * s->nop), 256>>>(s->T, s->perm, n, s->nop, (float*)tt);
  SUR_TRY(cudaMemcpy(s->Xb, tx, (size_t)n * s->kin * 2, cudaMemcpyDeviceToDevice));
  SUR_TRY(cudaMemcpy(s->T, tt, (size_t)n * s->nop * 4, cudaMemcpyDeviceToDevice));
  cudaFree(tx);
  cudaFree(tt);
  s->ntrain = std::max(s->batch, (int)std::lround(n * (1.0 - val_fraction)));
  s->ntrain = std::min(s->ntrain, n);
  s->ready = true;
  SUR_TRY(cudaDeviceSynchronize());
  return MOLOCH_OK;
}

// mean squared error (normalised units) of rows [r0, r1) in whole batches
static int eval_loss(Surrogate* s, int r0, int r1, double* out, cudaStream_t st) {
  const int B = s->batch;
  double tot = 0.0;
  long long cnt = 0;
  for (int r = r0; r + B <= r1; r += B) {
    forward(s, (const __nv_bfloat16*)s->Xb + (size_t)r * s->kin, B, s->H, nullptr, s->Y, st);
    cudaMemcpyAsync(s->Tbat, s->T + (size_t)r * s->nop, (size_t)B * s->nop * 4, cudaMemcpyDeviceToDevice, st);
    const int lg = grid1((size_t)B * s->nop);
    k_sur_loss_grad<<<lg, 256, 0, st>>>(s->Y, s->Tbat, B, s->nop, s->nout, (__nv_bfloat16*)s->dY, s->lpart);
    k_sum_parts<<<1, 256, 0, st>>>(s->lpart, lg, s->loss);
    float l = 0.f;
    SUR_TRY(cudaMemcpyAsync(&l, s->loss, 4, cudaMemcpyDeviceToHost, st));
    SUR_TRY(cudaStreamSynchronize(st));
    tot += l;
    cnt += (long long)B * s->nout;
  }
  *out = cnt ? tot / cnt : 0.0;
  return MOLOCH_OK;
}

int moloch_sur_train(moloch_surrogate_t* s, int iters, float lr, unsigned long long seed, float* train_loss,
                     float* val_loss) {
  if (!s || !s->ready || iters < 0) {
    moloch_internal_set_error("sur_train: call moloch_sur_prepare first");
    return MOLOCH_ERR_STATE;
  }
  cudaStream_t st = 0;
  const int B = s->batch;
  uint64_t rs = seed ? seed : 11;
  std::vector<int> idx(B);
  for (int it = 0; it < iters; ++it) {
    for (int q = 0; q < B; ++q) idx[q] = (int)(sm64(rs) % (uint64_t)s->ntrain);
    SUR_TRY(cudaMemcpyAsync(s->perm, idx.data(), B * 4, cudaMemcpyHostToDevice, st));
    k_gather_rows<__nv_bfloat16><<<grid1((size_t)B * s->kin), 256, 0, st>>>((const __nv_bfloat16*)s->Xb, s->perm, B,
                                                                            s->kin, (__nv_bfloat16*)s->Xbat);
    k_gather_rows<float><<<grid1((size_t)B * s->nop), 256, 0, st>>>(s->T, s->perm, B, s->nop, s->Tbat);
    forward(s, s->Xbat, B, s->H, s->Z, s->Y, st);
    backward(s, st);
    // cosine decay to 10% of lr
    const float f = 0.1f + 0.9f * 0.5f * (1.f + cosf(3.14159265f * (float)it / (float)std::max(iters, 1)));
    adam_all(s, lr * f, ++s->adam_t, st);
  }
  SUR_TRY(cudaStreamSynchronize(st));
  SUR_TRY(cudaGetLastError());
  double tl = 0.0, vl = 0.0;
  int rc = eval_loss(s, 0, std::min(s->ntrain, 16 * B), &tl, st);
  if (!rc) rc = eval_loss(s, s->ntrain, s->npairs, &vl, st);
  if (train_loss) *train_loss = (float)tl;
  if (val_loss) *val_loss = (float)vl;
  return rc;
}

int moloch_sur_attach(moloch_handle_t* h, moloch_surrogate_t* s, float threshold, int judge_every, float tol) {
  if (!h) {
    moloch_internal_set_error("sur_attach: null handle");
    return MOLOCH_ERR_ARG;
  }
  if (s) {
    View<float>* vp = moloch_internal_viewf(h);
    if (!vp || vp->kz != s->kz || !s->ready) {
      moloch_internal_set_error("sur_attach: needs a trained surrogate and an FP32-storage handle with its kz");
      return MOLOCH_ERR_ARG;
    }
    if (judge_every < 0 || !(threshold >= 0.f) || !(tol >= 0.f)) {
      moloch_internal_set_error("sur_attach: threshold, tol >= 0, judge_every >= 0");
      return MOLOCH_ERR_ARG;
    }
    const int n = vp->nj * vp->ni;
    if (n > s->ninf) {
      auto F = [](void* p) { if (p) cudaFree(p); };
      F(s->Xinf); F(s->Yinf); F(s->jsnap);
      for (int l = 0; l < 3; ++l) F(s->Hinf[l]);
      s->Xinf = s->Yinf = s->jsnap = nullptr;
      s->ninf = 0;
      SUR_TRY(cudaMalloc(&s->Xinf, (size_t)n * s->kin * 2));
      SUR_TRY(cudaMalloc((void**)&s->Yinf, (size_t)n * s->nop * 4));
      SUR_TRY(cudaMalloc((void**)&s->jsnap, (size_t)5 * n * s->kz * 4));
      for (int l = 0; l < 3; ++l) SUR_TRY(cudaMalloc(&s->Hinf[l], (size_t)n * s->hid * 2));
      s->ninf = n;
    }
    s->threshold = threshold;
    s->judge_every = judge_every;
    s->tol = tol;
    s->max_interval = std::max(16 * judge_every, 1);
    // judge_every == 0: no judge, the surrogate is enabled from the start
    int ctl[CTL_COUNT] = {0};
    ctl[CTL_ENABLED] = judge_every == 0 ? 1 : 0;
    ctl[CTL_NEXTJUDGE] = 0;
    ctl[CTL_INTERVAL] = judge_every;
    SUR_TRY(cudaMemcpy(s->ctl, ctl, sizeof ctl, cudaMemcpyHostToDevice));
    SUR_TRY(cudaMemset(s->counts, 0, 4 * sizeof(unsigned long long)));
  }
  return moloch_internal_attach(h, s);
}

// cycles seen, cycles run by the plain loop (rejected, disabled or judge),
// judge cycles, judge verdicts that disabled the surrogate, the largest
// |y| / envelope since attach and the error of the last judge cycle
int moloch_sur_counts(moloch_surrogate_t* s, long long* counts4, float* max_ratio, float* last_error) {
  if (!s) return MOLOCH_ERR_ARG;
  unsigned long long c[4] = {0, 0, 0, 0};
  int ctl[CTL_COUNT];
  SUR_TRY(cudaDeviceSynchronize());
  SUR_TRY(cudaMemcpy(c, s->counts, sizeof c, cudaMemcpyDeviceToHost));
  SUR_TRY(cudaMemcpy(ctl, s->ctl, sizeof ctl, cudaMemcpyDeviceToHost));
  if (counts4)
    for (int q = 0; q < 4; ++q) counts4[q] = (long long)c[q];
  if (max_ratio) std::memcpy(max_ratio, &ctl[CTL_MAXRATIO], sizeof(float));
  if (last_error) std::memcpy(last_error, &ctl[CTL_LASTERR], sizeof(float));
  return MOLOCH_OK;
}

// host copy of a layer's FP32 weights [out][in] and bias (set != 0 uploads)
int moloch_sur_param(moloch_surrogate_t* s, int layer, float* W, float* b, int set, int* in_out) {
  if (!s || layer < 0 || layer > 3) return MOLOCH_ERR_ARG;
  SurLayer& L = s->L[layer];
  if (in_out) { in_out[0] = L.in; in_out[1] = L.out; }
  const size_t nw = (size_t)L.in * L.out;
  if (set) {
    if (W) SUR_TRY(cudaMemcpy(L.W, W, nw * 4, cudaMemcpyHostToDevice));
    if (b) SUR_TRY(cudaMemcpy(L.b, b, L.out * 4, cudaMemcpyHostToDevice));
    std::vector<float> z(nw, 0.f);  // refresh BF16 copies without moving the weights
    SUR_TRY(cudaMemcpy(L.gW, z.data(), nw * 4, cudaMemcpyHostToDevice));
    SUR_TRY(cudaMemset(L.gb, 0, L.out * 4));
    SUR_TRY(cudaMemset(L.mW, 0, nw * 4)); SUR_TRY(cudaMemset(L.vW, 0, nw * 4));
    SUR_TRY(cudaMemset(L.mb, 0, L.out * 4)); SUR_TRY(cudaMemset(L.vb, 0, L.out * 4));
    k_adam<<<grid1(nw), 256>>>(L.W, L.gW, L.mW, L.vW, L.out, L.in, 0.f, 0.9f, 0.999f, 1e-8f, 1.f, 1.f,
                               (__nv_bfloat16*)L.Wb, (__nv_bfloat16*)L.WT, L.out);
    SUR_TRY(cudaDeviceSynchronize());
  } else {
    if (W) SUR_TRY(cudaMemcpy(W, L.W, nw * 4, cudaMemcpyDeviceToHost));
    if (b) SUR_TRY(cudaMemcpy(b, L.b, L.out * 4, cudaMemcpyDeviceToHost));
  }
  return MOLOCH_OK;
}

// One forward + backward pass on a caller batch (n == batch rows): X
// [n][kin] normalised features (rounded to BF16 here), T [n][nop] targets.
// Returns the summed squared error and the gradients of one layer.
int moloch_sur_gradients(moloch_surrogate_t* s, const float* X, const float* T, int n, float* loss, int layer,
                         float* gW, float* gb) {
  if (!s || !X || !T || n != s->batch || layer < 0 || layer > 3) {
    moloch_internal_set_error("sur_gradients: n must equal the batch size");
    return MOLOCH_ERR_ARG;
  }
  std::vector<__nv_bfloat16> xb((size_t)n * s->kin);
  for (size_t q = 0; q < xb.size(); ++q) xb[q] = __float2bfloat16_rn(X[q]);
  SUR_TRY(cudaMemcpy(s->Xbat, xb.data(), xb.size() * 2, cudaMemcpyHostToDevice));
  SUR_TRY(cudaMemcpy(s->Tbat, T, (size_t)n * s->nop * 4, cudaMemcpyHostToDevice));
  forward(s, s->Xbat, n, s->H, s->Z, s->Y, 0);
  backward(s, 0);
  SUR_TRY(cudaDeviceSynchronize());
  SUR_TRY(cudaGetLastError());
  SurLayer& L = s->L[layer];
  if (loss) SUR_TRY(cudaMemcpy(loss, s->loss, 4, cudaMemcpyDeviceToHost));
  if (gW) SUR_TRY(cudaMemcpy(gW, L.gW, (size_t)L.in * L.out * 4, cudaMemcpyDeviceToHost));
  if (gb) SUR_TRY(cudaMemcpy(gb, L.gb, L.out * 4, cudaMemcpyDeviceToHost));
  return MOLOCH_OK;
}

// normalisation statistics (5 * kz each, field-major): read (set 0) or
// written (set != 0; marks the surrogate ready for attach)
int moloch_sur_stats(moloch_surrogate_t* s, float* xmean, float* xstd, float* ymean, float* ystd, int set) {
  if (!s) return MOLOCH_ERR_ARG;
  const size_t b = (size_t)5 * s->kz * sizeof(float);
  float* dev[4] = {s->xmean, s->xstd, s->ymean, s->ystd};
  float* host[4] = {xmean, xstd, ymean, ystd};
  for (int q = 0; q < 4; ++q) {
    if (!host[q]) continue;
    if (set)
      SUR_TRY(cudaMemcpy(dev[q], host[q], b, cudaMemcpyHostToDevice));
    else
      SUR_TRY(cudaMemcpy(host[q], dev[q], b, cudaMemcpyDeviceToHost));
  }
  if (set) s->ready = true;
  return MOLOCH_OK;
}

// CUDA-event times (ms) of the inference stages of one cycle on the
// handle's current state: ms[0] features, ms[1..4] the four layers, ms[5]
// the envelope check.  Changes no field (nothing is committed).
int moloch_sur_profile(moloch_surrogate_t* s, moloch_handle_t* h, double* ms, int nms) {
  View<float>* vp = moloch_internal_viewf(h);
  if (!s || !vp || !ms || nms < 6 || vp->nj * vp->ni > s->ninf) {
    moloch_internal_set_error("sur_profile: attach the surrogate to this handle first");
    return MOLOCH_ERR_ARG;
  }
  View<float>& v = *vp;
  cudaStream_t st = moloch_internal_stream(h);
  const int n = v.nj * v.ni, hid = s->hid;
  cudaEvent_t ev[7];
  for (auto& e : ev) SUR_TRY(cudaEventCreate(&e));
  cudaEventRecord(ev[0], st);
  k_sur_features<true><<<feature_grid(n, s->kin), 128, 0, st>>>(v, nullptr, n, s->xmean, s->xstd, s->Xinf,
                                                                          s->kin, nullptr);
  cudaEventRecord(ev[1], st);
  gemm(s->Xinf, s->kin, s->L[0].Wb, s->kin, nullptr, hid, s->Hinf[0], hid, s->L[0].b, n, hid, s->kin, ACT_SILU, st);
  cudaEventRecord(ev[2], st);
  gemm(s->Hinf[0], hid, s->L[1].Wb, hid, nullptr, hid, s->Hinf[1], hid, s->L[1].b, n, hid, hid, ACT_SILU, st);
  cudaEventRecord(ev[3], st);
  gemm(s->Hinf[1], hid, s->L[2].Wb, hid, nullptr, hid, s->Hinf[2], hid, s->L[2].b, n, hid, hid, ACT_SILU, st);
  cudaEventRecord(ev[4], st);
  gemm(s->Hinf[2], hid, s->L[3].Wb, hid, nullptr, 0, nullptr, 0, s->L[3].b, n, s->nop, hid, ACT_NONE, st, nullptr,
       s->Yinf, n);
  cudaEventRecord(ev[5], st);
  // the check writes slots CTL_BAD and CTL_MAXRATIO of the block it is
  // given: point it at the unused upper half of the control block
  static_assert(16 + CTL_MAXRATIO < CTL_COUNT, "control block too small");
  k_sur_check<<<check_grid(n, s->nout), 256, 0, st>>>(s->Yinf, n, s->nop, s->nout, s->env, s->threshold,
                                                                 s->ctl + 16, nullptr);
  cudaEventRecord(ev[6], st);
  SUR_TRY(cudaEventSynchronize(ev[6]));
  SUR_TRY(cudaGetLastError());
  for (int q = 0; q < 6; ++q) {
    float t = 0.f;
    cudaEventElapsedTime(&t, ev[q], ev[q + 1]);
    ms[q] = t;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  return MOLOCH_OK;
}

int moloch_sur_dims(moloch_surrogate_t* s, int* dims) {
  if (!s || !dims) return MOLOCH_ERR_ARG;
  dims[0] = s->kz; dims[1] = s->nin; dims[2] = s->kin; dims[3] = s->nout; dims[4] = s->nop; dims[5] = s->hid;
  dims[6] = s->batch; dims[7] = s->npairs; dims[8] = s->ntrain;
  return MOLOCH_OK;
}

int moloch_sur_destroy(moloch_surrogate_t* s) {
  if (!s) return MOLOCH_OK;
  cudaDeviceSynchronize();
  free_sur(s);
  delete s;
  return MOLOCH_OK;
}

}  // extern "C"
