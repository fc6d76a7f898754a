// Persistent ensemble step (types and program format in moloch_persist.h).
//
// The kernel bodies are those of moloch_kernels.cuh, compiled here a third
// time with the flags of moloch_kernels_fast.cu, so they round as in the
// per-kernel launches (the two modes agree bit for bit).  One launch writes
// arrays in one phase and reads them in the next: the gpu-scope fences of
// the grid barrier order the phases, and every array pointer a body uses
// comes from the member's view in shared memory, none from a kernel
// parameter, as in the per-kernel batched launches.
//
// Blocks are 32 x 8 threads.  Point bodies (32 x 8 tiles) run as in their
// own kernels; the 32 x 4 column bodies get tiles 8 rows high (see
// TK_COLUMN8); the warp-strip bodies get 8 strips per item, one per warp,
// with the momentum strips' cp.async rings in dynamic shared memory.  The
// kernel is built for 2, 3 and 4 resident blocks per SM (register budgets
// of 128, 80 and 64; the ensemble autotuner picks one).  Body variants that
// need far more than the budget of 3 blocks in FP32 or 2 in FP64 (FP32
// k-marching momentum, FP64 fused divergence/damping strips, horizontal WAF
// strips, 5 or 10 vertical-WAF fields per thread) are not carried.
//
// Grid barrier: thread 0 of each block fences, takes the arrival counter,
// and the last arrival resets the counter and bumps the generation; the
// others poll the generation with a limit of Args::spin SM cycles, after
// which they set *Args::err and leave.  A block that sees *err set leaves at
// its next barrier, and a launch that starts with *err set returns at once,
// so a failed step never waits longer than one limit per block.
#define MOLOCH_KNS kpersist
#define MOLOCH_NR_DDIV 1  // FP64 WAF limiter quotient by Newton-Raphson (div_nr)
#include "../../include/moloch_gb300.h"
#include "moloch_kernels.cuh"
#include "moloch_persist.h"

#include <algorithm>

namespace moloch {
namespace persist {

using namespace moloch::kpersist;

template <class T>
__host__ __device__ constexpr bool has_fused_divdamp() { return sizeof(T) == 4; }
template <class T>
__host__ __device__ constexpr bool has_momentum_km() { return sizeof(T) == 8; }
constexpr int kWarps = 8;

template <class T>
__device__ __forceinline__ void run_item(const View<T>& d, const Phase& ph, const int4 t, MomSlots<T>* ring) {
  switch (ph.kind) {
    case PH_PREDIAG: b_prediag<T>(d, t.y, t.z, t.w, ph.a0, ph.a1); break;
    case PH_DIVDAMP_STRIP:
      if constexpr (has_fused_divdamp<T>()) b_divdamp_strip<T>(d, t.y, t.z, ph.a0, threadIdx.y, kWarps);
      break;
    case PH_DIV: b_sound_div<T>(d, t.y, t.z, t.w); break;
    case PH_DIV_KM: b_sound_div_km<T>(d, t.y, t.z, t.w); break;
    case PH_DAMP: b_sound_damp<T>(d, t.y, t.z, t.w); break;
    case PH_DAMP_KM: b_sound_damp_km<T>(d, t.y, t.z, t.w); break;
    case PH_COLUMN: b_sound_column<T, 1>(d, t.y, t.z, t.w, ph.a0, ph.a1, ph.a2); break;
    case PH_LAP_FILTER: b_lap_filter<T>(d, t.y, t.z, t.w); break;
    case PH_PAI_UPDATE: b_pai_update<T>(d, t.y, t.z, t.w); break;
    case PH_MOM_STRIP: b_momentum_strip<T>(d, t.y, t.z, ph.a0, ring[threadIdx.y], threadIdx.y, kWarps); break;
    case PH_MOM: b_sound_momentum<T>(d, t.y, t.z, t.w); break;
    case PH_MOM_KM:
      if constexpr (has_momentum_km<T>()) b_sound_momentum_km<T>(d, t.y, t.z, t.w);
      break;
    case PH_WAF_VERTICAL1: b_waf_vertical<T, 1>(d, t.y, t.z, t.w); break;
    case PH_WAF_VERTICAL2: b_waf_vertical<T, 2>(d, t.y, t.z, t.w); break;
    case PH_WAF_HORIZONTAL: b_waf_horizontal<T>(d, t.y, t.z, t.w); break;
    case PH_STAG: b_stag_from_x<T>(d, t.y, t.z, t.w); break;
    case PH_POSTDIAG: b_postdiag<T>(d, t.y, t.z, t.w); break;
    default: break;
  }
}

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// barrier after phase p; false when the step is abandoned (a wait gave up
// here or elsewhere, or this block is the test hook's)
template <class T>
__device__ __forceinline__ bool grid_barrier(const Args<T>& a, const int p, int* s_ok) {
  __syncthreads();
  if (threadIdx.x == 0 && threadIdx.y == 0) {
    int ok = 1;
    if ((int)blockIdx.x == a.skip_block && p == a.skip_barrier) {
      ok = 0;  // leave without arriving: the others' waits run out
    } else {
      volatile unsigned int* gen = &a.ctl->gen;
      const unsigned int g0 = *gen;
      __threadfence();  // this block's writes before its arrival
      const unsigned int arrived = atomicAdd(&a.ctl->count, 1u);
      if (arrived == gridDim.x - 1) {
        atomicExch(&a.ctl->count, 0u);
        __threadfence();
        atomicAdd(&a.ctl->gen, 1u);
      } else {
        const long long t0 = clock64();
        while (*gen == g0) {
          if (*(volatile int*)a.err) { ok = 0; break; }
          if (clock64() - t0 > a.spin) { atomicExch(a.err, 1); ok = 0; break; }
          __nanosleep(32);
        }
      }
      __threadfence();  // the other blocks' writes before this block's next loads
    }
    *s_ok = ok;
  }
  __syncthreads();
  return *s_ok != 0;
}

template <class T, int MINB>
__global__ void __launch_bounds__(256, MINB) k_ensemble_persistent(const __grid_constant__ Args<T> a) {
  extern __shared__ __align__(16) unsigned char persist_smem[];
  MomSlots<T>* ring = reinterpret_cast<MomSlots<T>*>(persist_smem);  // one per warp
  __shared__ View<T> sv;
  __shared__ int s_item[2];
  __shared__ int s_ok;
  if (*(volatile int*)a.err) return;  // an earlier step gave up: nothing runs until the host clears it
  const int tid = threadIdx.x + 32 * threadIdx.y;
  const bool stamp = a.stamps != nullptr && blockIdx.x == 0 && tid == 0;
  if (stamp) a.stamps[0] = globaltimer_ns();
  int have = -1;  // which view sv holds
  for (int p = 0; p < a.nphases; ++p) {
    const Phase ph = a.prog[p];
    // chunks of ph.chunk items; the claim of the next chunk is in flight
    // while this one runs.  Claim slots alternate: thread 0 rewrites a slot
    // one chunk after the others read it, with a barrier between.
    if (tid == 0) s_item[0] = atomicAdd(&a.ctl->q[p], ph.chunk);
    __syncthreads();
    for (int it = 0;; ++it) {
      const int start = s_item[it & 1];
      if (start >= ph.ntiles) break;
      if (tid == 0) s_item[(it + 1) & 1] = atomicAdd(&a.ctl->q[p], ph.chunk);
      const int end = min(start + ph.chunk, ph.ntiles);
      for (int item = start; item < end; ++item) {
        const int4 t = ph.tiles[item];
        const int vid = ph.par * a.nmembers + t.x;
        if (vid != have) {  // block-uniform
          __syncthreads();  // every thread is done with the previous view
          copy_view(&sv, a.views + vid);
          __syncthreads();
          have = vid;
        }
        run_item<T>(sv, ph, t, ring);
      }
      __syncthreads();  // the next claim is visible
    }
    if (!grid_barrier(a, p, &s_ok)) return;
    if (stamp) a.stamps[p + 1] = globaltimer_ns();
  }
}

template <class T>
bool supports(int hz_levels, int kmarch, int vfields) {
  if (hz_levels >= 16 || (vfields != 1 && vfields != 2)) return false;
  if (kmarch & (32 | 512)) return false;  // the staged column solve and the two-level strips run as own launches
  if ((kmarch & 16) && !has_fused_divdamp<T>()) return false;
  if ((kmarch & 4) && !(kmarch & 8) && !has_momentum_km<T>()) return false;
  return true;
}

template <class T>
int program(const Batch<T>& b, const PhaseFlags& fl, int fcur, int grid, std::vector<Phase>& out) {
  out.clear();
  if (b.hstrip || !supports<T>(4, b.kmarch, b.vfields) || grid < 1) return 1;
  int cur = 0;
  auto P = [&](int kind, int tk, int a0 = 0, int a1 = 0, int a2 = 0) {
    Phase ph;
    ph.kind = kind;
    ph.ntiles = b.ntiles[tk];
    ph.tiles = b.tiles[tk];
    ph.par = cur * 2 + fcur;
    ph.a0 = a0;
    ph.a1 = a1;
    ph.a2 = a2;
    ph.chunk = std::max(1, ph.ntiles / (8 * grid));
    out.push_back(ph);
  };
  // the order of the per-kernel launches (blaunch_step)
  P(PH_PREDIAG, TK_POINT, fl.filterpai, fl.filtertheta);
  for (int a = 0; a < fl.nadv; ++a) {
    for (int ns = 1; ns <= fl.nsound; ++ns) {
      const int last = ns == fl.nsound;
      if (b.kmarch & 16) {
        P(PH_DIVDAMP_STRIP, TK_DSTRIP8, kDDR);
        cur ^= 1;  // the damped u, v are in the other buffer
      } else {
        if (b.kmarch & 1) P(PH_DIV_KM, TK_CHUNK); else P(PH_DIV, TK_POINT);
        if (b.kmarch & 2) P(PH_DAMP_KM, TK_CHUNK); else P(PH_DAMP, TK_POINT);
      }
      if (fl.divfilter) {
        P(PH_COLUMN, TK_COLUMN8, ns, last, 1);
        P(PH_LAP_FILTER, TK_POINT);
        P(PH_PAI_UPDATE, TK_POINT);
      } else {
        P(PH_COLUMN, TK_COLUMN8, ns, last, 0);
      }
      if (b.kmarch & 8) P(PH_MOM_STRIP, TK_MSTRIP8, kMomR);
      else if (b.kmarch & 4) P(PH_MOM_KM, TK_CHUNK);
      else P(PH_MOM, TK_POINT);
      cur ^= 1;
    }
    P(b.vfields == 2 ? PH_WAF_VERTICAL2 : PH_WAF_VERTICAL1, TK_VERTICAL8);
    P(PH_WAF_HORIZONTAL, TK_HORIZONTAL);
    fcur ^= 1;
    P(PH_STAG, TK_POINT);
    cur = 0;
  }
  P(PH_POSTDIAG, TK_COLUMN8);
  return (int)out.size() <= kMaxPhases ? 0 : 2;
}

template <class T>
static size_t ring_bytes() { return sizeof(MomSlots<T>) * kWarps; }

// the kernel instantiated for 2, 3 and 4 resident blocks per SM (register
// budgets of 128, 80 and 64 per thread)
template <class T>
static const void* kernel_of(int variant) {
  switch (variant) {
    case 0: return (const void*)k_ensemble_persistent<T, 2>;
    case 2: return (const void*)k_ensemble_persistent<T, 4>;
    default: return (const void*)k_ensemble_persistent<T, 3>;
  }
}

template <class T>
int blocks_per_sm(int variant, size_t* smem) {
  const size_t s = ring_bytes<T>();
  if (smem) *smem = s;
  const void* k = kernel_of<T>(variant);
  if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s) != cudaSuccess) return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, 256, s) != cudaSuccess) return 0;
  return nb;
}

template <class T>
cudaError_t launch(const Args<T>& a, int variant, int grid, size_t smem, cudaStream_t st) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(32, 8);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  switch (variant) {
    case 0: return cudaLaunchKernelEx(&cfg, k_ensemble_persistent<T, 2>, a);
    case 2: return cudaLaunchKernelEx(&cfg, k_ensemble_persistent<T, 4>, a);
    default: return cudaLaunchKernelEx(&cfg, k_ensemble_persistent<T, 3>, a);
  }
}

template bool supports<float>(int, int, int);
template bool supports<double>(int, int, int);
template int program<float>(const Batch<float>&, const PhaseFlags&, int, int, std::vector<Phase>&);
template int program<double>(const Batch<double>&, const PhaseFlags&, int, int, std::vector<Phase>&);
template int blocks_per_sm<float>(int, size_t*);
template int blocks_per_sm<double>(int, size_t*);
template cudaError_t launch<float>(const Args<float>&, int, int, size_t, cudaStream_t);
template cudaError_t launch<double>(const Args<double>&, int, int, size_t, cudaStream_t);

}  // namespace persist
}  // namespace moloch
