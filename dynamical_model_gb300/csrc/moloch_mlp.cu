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

// =========================================================================
// Surrogate of one acoustic cycle (sound(), nompi/mod_moloch.F90:483-851)
// =========================================================================
#include "moloch_sur.h"

namespace moloch {
namespace mlp {

// feature x[(nb * 5 + f) * kz + k]: neighbour nb = (di + 1) * 3 + (dj + 1),
// field f = u, v, w (levels 2..kz+1), pai, tetav, level k
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

// Features of ncols columns (cols == nullptr: all columns in order).  Block
// = 32 columns x 8 feature lanes; a 64-feature slab is staged in shared
// memory so both the field reads (consecutive j) and the row writes
// (consecutive features) are coalesced.  NORM: subtract/scale with the
// dataset statistics and write BF16; else write raw FP32.
template <bool NORM>
__global__ void __launch_bounds__(256) k_sur_features(View<float> d, const int* __restrict__ cols, int ncols,
                                                      const float* __restrict__ xmean, const float* __restrict__ xstd,
                                                      void* out, int ldo) {
  __shared__ float tile[64][33];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int c0 = blockIdx.x * 32;
  const int kz = d.kz, nf = 45 * kz;
  const int cidx = c0 + tx;
  int j = 0, i = 0;
  if (cidx < ncols) {
    const int col = cols ? cols[cidx] : cidx;
    j = col % d.nj;
    i = col / d.nj;
  }
  for (int f0 = 0; f0 < ldo; f0 += 64) {
    for (int r = ty; r < 64; r += 8) {
      const int fe = f0 + r;
      float val = 0.f;
      if (cidx < ncols && fe < nf) {
        const int k = fe % kz, fk = fe / kz, fld = fk % 5, nb = fk / 5;
        const int dj = nb % 3 - 1, di = nb / 3 - 1;
        int jj = j + dj, ii = i + di;
        jj = jj < 0 ? jj + d.nj : (jj >= d.nj ? jj - d.nj : jj);
        ii = ii < 0 ? ii + d.ni : (ii >= d.ni ? ii - d.ni : ii);
        val = sur_field(d, fld, jj, ii, k);
        if (NORM) val = (val - xmean[fld * kz + k]) / xstd[fld * kz + k];
      }
      tile[r][tx] = val;
    }
    __syncthreads();
    // write rows: column c0 + cc, features f0 .. f0+63
    for (int q = tx + 32 * ty; q < 32 * 64; q += 256) {
      const int cc = q / 64, r = q % 64;
      if (c0 + cc < ncols && f0 + r < ldo) {
        if (NORM)
          reinterpret_cast<__nv_bfloat16*>(out)[(size_t)(c0 + cc) * ldo + f0 + r] = __float2bfloat16_rn(tile[r][cc]);
        else
          reinterpret_cast<float*>(out)[(size_t)(c0 + cc) * ldo + f0 + r] = tile[r][cc];
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

// in-place normalisation of a row-major [n][ld] FP32 array by per-column
// statistics (the first m columns), with optional BF16 copy
__global__ void k_sur_normalize(float* __restrict__ a, int n, int ld, int m, const float* __restrict__ mean,
                                const float* __restrict__ stdv, __nv_bfloat16* __restrict__ ab, int period) {
  const size_t tot = (size_t)n * ld;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < tot; q += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(q % ld);
    float v = a[q];
    if (c < m) {
      const int s = c % period;
      v = (v - mean[s]) / stdv[s];
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
// the padding), BF16; accumulates the squared error into *loss
__global__ void k_sur_loss_grad(const float* __restrict__ Y, const float* __restrict__ T, int n, int ld, int m,
                                __nv_bfloat16* __restrict__ dY, float* __restrict__ loss) {
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
  if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, acc);
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

// acceptance check of one surrogate cycle: every increment finite and its
// normalised size within the threshold.  k_sur_check marks *bad; the
// one-thread k_sur_decide turns it into *flag = 1 (accept) / 0 (fall back to
// the plain sound loop), counts, and clears *bad for the next cycle.
__global__ void k_sur_check(const float* __restrict__ Y, int n, int ld, int m, float threshold, int* __restrict__ bad) {
  const size_t tot = (size_t)n * ld;
  int b = 0;
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < tot; q += (size_t)gridDim.x * blockDim.x) {
    const int c = (int)(q % ld);
    if (c < m && !(fabsf(Y[q]) <= threshold)) b = 1;  // also catches NaN
  }
  if (__any_sync(0xffffffffu, b) && (threadIdx.x & 31) == 0) atomicOr(bad, 1);
}
__global__ void k_sur_decide(int* __restrict__ bad, int* __restrict__ flag, unsigned long long* __restrict__ counts) {
  const int b = *bad;
  *flag = b ? 0 : 1;
  counts[0] += 1;
  if (b) counts[1] += 1;
  *bad = 0;
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
                                                  const int* __restrict__ flag, int nsound) {
  if (!*flag) return;
  const int jj = blockIdx.x * 32 + threadIdx.x, ii = blockIdx.y * 8 + threadIdx.y;
  const int nj = d.nj, ni = d.ni, kz = d.kz;
  if (jj >= nj || ii >= ni) return;
  const size_t pl = d.pl, c = jj + (size_t)nj * ii;
  const int jp = jj == nj - 1 ? 0 : jj + 1, ip = ii == ni - 1 ? 0 : ii + 1;
  const size_t ce = jp + (size_t)nj * ii, cn = jj + (size_t)nj * ip;
  const float* __restrict__ u = d.ubuf[d.cur];
  const float* __restrict__ v = d.vbuf[d.cur];
  const float fr = (float)(nsound - 1) / (float)nsound;
  auto inc = [&](size_t col, int f, int k) { const int q = f * kz + k; return Y[col * ld + q] * ystd[q] + ymean[q]; };
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
// column; u, v go to the buffer the plain loop leaves them in after nsound
// substeps.
__global__ void __launch_bounds__(256) k_sur_apply(View<float> d, const float* __restrict__ Y, int ld,
                                                   const float* __restrict__ ymean, const float* __restrict__ ystd,
                                                   const int* __restrict__ flag, int nsound) {
  if (!*flag) return;
  const int jj = blockIdx.x * 32 + threadIdx.x, ii = blockIdx.y * 8 + threadIdx.y;
  const int nj = d.nj, ni = d.ni, kz = d.kz;
  if (jj >= nj || ii >= ni) return;
  const size_t pl = d.pl, c = jj + (size_t)nj * ii;
  const float* __restrict__ yr = Y + c * ld;
  const float* u = d.ubuf[d.cur];
  const float* v = d.vbuf[d.cur];
  float* uo = d.ubuf[d.cur ^ (nsound & 1)];
  float* vo = d.vbuf[d.cur ^ (nsound & 1)];
  auto inc = [&](int f, int k) { const int q = f * kz + k; return yr[q] * ystd[q] + ymean[q]; };
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
#include <mutex>
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

static int g_gemm_attr_done = 0;
static int gemm(const void* A, int lda, const void* B, int ldb, float* C, int ldc, void* Cb, int ldcb,
                const float* bias, int M, int N, int K, int act, cudaStream_t st) {
  if (!g_gemm_attr_done) {
    cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
    g_gemm_attr_done = 1;
  }
  dim3 grid((M + kTileM - 1) / kTileM, (N + kTileN - 1) / kTileN);
  k_gemm_tc<<<grid, 128, kSmem, st>>>((const __nv_bfloat16*)A, lda, (const __nv_bfloat16*)B, ldb, C, ldc,
                                       (__nv_bfloat16*)Cb, ldcb, bias, M, N, K, act);
  return 1;
}

static int grid1(size_t n) { return (int)std::min<size_t>((n + 255) / 256, 152 * 16); }

static int transpose(const void* in, int rows, int cols, int ld_in, void* out, int ld_out, cudaStream_t st) {
  dim3 g((cols + 31) / 32, (rows + 31) / 32);
  k_transpose_bf16<__nv_bfloat16><<<g, dim3(32, 8), 0, st>>>((const __nv_bfloat16*)in, rows, cols, ld_in,
                                                             (__nv_bfloat16*)out, ld_out);
  return 1;
}

// forward of n rows: X -> H[0..2] (BF16, SiLU) -> Y (FP32); Z (pre-activations) optional
static int forward(Surrogate* s, const void* X, int n, void* const* H, float* const* Z, float* Y, cudaStream_t st) {
  const int hid = s->hid;
  gemm(X, s->kin, s->L[0].Wb, s->kin, Z ? Z[0] : nullptr, hid, H[0], hid, s->L[0].b, n, hid, s->kin, ACT_SILU, st);
  gemm(H[0], hid, s->L[1].Wb, hid, Z ? Z[1] : nullptr, hid, H[1], hid, s->L[1].b, n, hid, hid, ACT_SILU, st);
  gemm(H[1], hid, s->L[2].Wb, hid, Z ? Z[2] : nullptr, hid, H[2], hid, s->L[2].b, n, hid, hid, ACT_SILU, st);
  gemm(H[2], hid, s->L[3].Wb, hid, Y, s->nop, nullptr, 0, s->L[3].b, n, s->nop, hid, ACT_NONE, st);
  return 4;
}

// one backward pass for the batch in Xbat/Tbat after forward(Xbat, H, Z, Y):
// gradients into L[*].gW/gb, loss sum into *s->loss
static void backward(Surrogate* s, cudaStream_t st) {
  const int B = s->batch, hid = s->hid, nop = s->nop;
  cudaMemsetAsync(s->loss, 0, sizeof(float), st);
  k_sur_loss_grad<<<grid1((size_t)B * nop), 256, 0, st>>>(s->Y, s->Tbat, B, nop, s->nout, (__nv_bfloat16*)s->dY, s->loss);
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

int sur_cycle(Surrogate* s, View<float>& v, cudaStream_t st, int nsound) {
  const int n = v.nj * v.ni;
  k_sur_features<true><<<(n + 31) / 32, dim3(32, 8), 0, st>>>(v, nullptr, n, s->xmean, s->xstd, s->Xinf, s->kin);
  forward(s, s->Xinf, n, s->Hinf, nullptr, s->Yinf, st);
  k_sur_check<<<grid1((size_t)n * s->nop), 256, 0, st>>>(s->Yinf, n, s->nop, s->nout, s->threshold, s->bad);
  k_sur_decide<<<1, 1, 0, st>>>(s->bad, s->flag, s->counts);
  const dim3 cg((v.nj + 31) / 32, (v.ni + 7) / 8);
  k_sur_vvel<<<cg, dim3(32, 8), 0, st>>>(v, s->Yinf, s->nop, s->ymean, s->ystd, s->flag, nsound);
  k_sur_apply<<<cg, dim3(32, 8), 0, st>>>(v, s->Yinf, s->nop, s->ymean, s->ystd, s->flag, nsound);
  return 9;
}

static void free_sur(Surrogate* s) {
  auto F = [](void* p) { if (p) cudaFree(p); };
  for (auto& L : s->L) {
    F(L.W); F(L.b); F(L.gW); F(L.gb); F(L.mW); F(L.vW); F(L.mb); F(L.vb); F(L.Wb); F(L.WT);
  }
  F(s->xmean); F(s->xstd); F(s->ymean); F(s->ystd); F(s->Xraw); F(s->Xb); F(s->T); F(s->snap); F(s->cols);
  F(s->Xbat); F(s->XbatT); F(s->Tbat); F(s->Y); F(s->dY); F(s->dYT); F(s->loss); F(s->perm);
  for (int l = 0; l < 3; ++l) { F(s->H[l]); F(s->HT[l]); F(s->Z[l]); F(s->dH[l]); F(s->dZ[l]); F(s->dZT[l]); F(s->Hinf[l]); }
  F(s->Xinf); F(s->Yinf); F(s->flag); F(s->bad); F(s->counts);
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
  if (!g_gemm_attr_done) {  // before any capture of a step that runs the GEMM
    cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem);
    g_gemm_attr_done = 1;
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
  A((void**)&s->loss, 16); A((void**)&s->perm, (size_t)capacity * 4);
  for (int l = 0; l < 3; ++l) {
    A(&s->H[l], (size_t)batch * hid * 2); A(&s->HT[l], (size_t)batch * hid * 2);
    A((void**)&s->Z[l], (size_t)batch * hid * 4); A((void**)&s->dH[l], (size_t)batch * hid * 4);
    A(&s->dZ[l], (size_t)batch * hid * 2); A(&s->dZT[l], (size_t)batch * hid * 2);
  }
  A((void**)&s->flag, 16); A((void**)&s->bad, 16); A((void**)&s->counts, 16);
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
        k_sur_features<false><<<(take + 31) / 32, dim3(32, 8), 0, st>>>(v, s->cols, take, nullptr, nullptr,
                                                                       s->Xraw + (size_t)s->npairs * s->kin, s->kin);
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
    for (int f = 0; f < s->nin; ++f) { const double x = xr[f]; xs[f % n5] += x; xq[f % n5] += x * x; }
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
    yd[q] = (float)(std::sqrt(vy) > 1e-30 ? std::sqrt(vy) : 1.0);
  }
  SUR_TRY(cudaMemcpy(s->xmean, xm.data(), n5 * 4, cudaMemcpyHostToDevice));
  SUR_TRY(cudaMemcpy(s->xstd, xd.data(), n5 * 4, cudaMemcpyHostToDevice));
  SUR_TRY(cudaMemcpy(s->ymean, ym.data(), n5 * 4, cudaMemcpyHostToDevice));
  SUR_TRY(cudaMemcpy(s->ystd, yd.data(), n5 * 4, cudaMemcpyHostToDevice));
  k_sur_normalize<<<grid1((size_t)n * s->kin), 256>>>(s->Xraw, n, s->kin, s->nin, s->xmean, s->xstd,
                                                      (__nv_bfloat16*)s->Xb, n5);
  k_sur_normalize<<<grid1((size_t)n * s->nop), 256>>>(s->T, n, s->nop, s->nout, s->ymean, s->ystd, nullptr, n5);
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
    cudaMemsetAsync(s->loss, 0, 4, st);
    cudaMemcpyAsync(s->Tbat, s->T + (size_t)r * s->nop, (size_t)B * s->nop * 4, cudaMemcpyDeviceToDevice, st);
    k_sur_loss_grad<<<grid1((size_t)B * s->nop), 256, 0, st>>>(s->Y, s->Tbat, B, s->nop, s->nout,
                                                                (__nv_bfloat16*)s->dY, s->loss);
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

int moloch_sur_attach(moloch_handle_t* h, moloch_surrogate_t* s, float threshold) {
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
    const int n = vp->nj * vp->ni;
    if (n > s->ninf) {
      auto F = [](void* p) { if (p) cudaFree(p); };
      F(s->Xinf); F(s->Yinf);
      for (int l = 0; l < 3; ++l) F(s->Hinf[l]);
      SUR_TRY(cudaMalloc(&s->Xinf, (size_t)n * s->kin * 2));
      SUR_TRY(cudaMalloc((void**)&s->Yinf, (size_t)n * s->nop * 4));
      for (int l = 0; l < 3; ++l) SUR_TRY(cudaMalloc(&s->Hinf[l], (size_t)n * s->hid * 2));
      s->ninf = n;
    }
    s->threshold = threshold;
  }
  return moloch_internal_attach(h, s);
}

int moloch_sur_counts(moloch_surrogate_t* s, long long* cycles, long long* fallbacks) {
  if (!s) return MOLOCH_ERR_ARG;
  unsigned long long c[2] = {0, 0};
  SUR_TRY(cudaDeviceSynchronize());
  SUR_TRY(cudaMemcpy(c, s->counts, sizeof c, cudaMemcpyDeviceToHost));
  if (cycles) *cycles = (long long)c[0];
  if (fallbacks) *fallbacks = (long long)c[1];
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
