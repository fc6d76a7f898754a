// Implicit w (Thomas, one thread per column) + Exner/theta/pai update of
// sound() for FP32 storage (nompi/mod_moloch.F90:634-728, :843-849) with
// every array crossing HBM once.
//
// The one-thread-per-column kernel (b_sound_column) reads the down-sweep's
// inputs, writes an FP32 stash of the recurrence, and in the
// back-substitution reads the stash and six of the inputs again; at
// 512 x 512 x 60 about 175 K columns are in flight, so level k is read again
// 2k+1 level steps later, long after L2 evicted it.  Here:
//   * a persistent CTA per SM walks tiles of 32 (j) x 4 (i) columns, one
//     compute warp per row of 32 columns, one thread per column;
//   * a producer warp stages chunks of kKCT levels of every input with 3-D
//     TMA boxes (32 x 4 x kKCT) into a ring of shared-memory stages, running
//     ahead through the down-sweep chunks, the back-substitution chunks and
//     the next tile's chunks, so the loads never wait on the recurrence;
//   * the values the back-substitution needs -- the recurrence's wp, ww,
//     the old w, and zdiv2b, fmz, qv, tetav, pai of each level -- go into
//     the thread's own TMEM lane (8 words a level, 8 kz <= 512 columns),
//     which stands in for registers that cannot be indexed by level.
// The arithmetic per level is that of b_sound_column<float> (FP64 pivots in
// complement form, FP32 right-hand side and back-substitution).
//
// Waits are bounded by View::spin_cycles SM cycles; a wait that gives up
// sets *View::kerr, the CTA stops, waits (bounded) for its copies in
// flight, frees TMEM and returns.
#pragma once

#include "moloch_tc.cuh"

namespace moloch {
namespace MOLOCH_KNS {

constexpr int kKCT = 8;                          // levels per staged chunk
constexpr int kTmStages = 4;                     // ring depth
constexpr int kTmSlots = 9;                      // arrays per stage (down-sweep)
constexpr int kTmSlotBytes = kKCT * 4 * 32 * 4;  // one 32 x 4 x kKCT FP32 box
constexpr int kTmStageBytes = kTmSlots * kTmSlotBytes;
constexpr int kTmSmem = kTmStages * kTmStageBytes + 128;  // + alignment slack
constexpr int kTmThreads = 160;                  // 4 compute warps + producer warp
constexpr int kTmMaxKz = 64;                     // 8 words x kz TMEM columns

// tensor maps of the staged arrays (tetav, pai, qv, qc depend on the
// advected-field buffer set, so the host keeps one set per parity)
enum ColMap { CM_W = 0, CM_FMZF, CM_QV, CM_TET, CM_PAI, CM_QSAT, CM_ZD, CM_FMZ, CM_T, CM_QC, CM_QWL, CM_QWI, CM_S,
              CM_COUNT };
struct ColumnMaps {
  CUtensorMap m[CM_COUNT];
};

__device__ __forceinline__ uint32_t fbits(float x) { return __float_as_uint(x); }
__device__ __forceinline__ float bitsf(uint32_t x) { return __uint_as_float(x); }

template <class T>
__global__ void __launch_bounds__(kTmThreads, 1)
    k_sound_column_tm(View<T> d, const __grid_constant__ ColumnMaps maps, int nsound, int last) {
  static_assert(sizeof(T) == 4, "FP32 storage only");
  if (d.sur_skip && *d.sur_skip) return;  // the surrogate took this cycle
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full[kTmStages], empty[kTmStages];
  __shared__ uint32_t tmem_base;
  __shared__ int s_fail, s_issued, s_consumed;
  __shared__ int s_last_job[kTmStages];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 127) & ~(uintptr_t)127);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nj = d.nj, ni = d.ni, kz = d.kz;
  const size_t pl = d.pl;
  const int nbx = (nj + 31) / 32, nby = (ni + 3) / 4, ntiles = nbx * nby;
  const int nd = (kz - 1 + kKCT - 1) / kKCT;  // down-sweep chunks: kk = kz-1 .. 1
  const int nu = (kz + kKCT - 1) / kKCT;      // back-substitution chunks: m = 0 .. kz-1
  const int jpt = nd + nu;                    // jobs per tile
  const int my_tiles = blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  const int njobs = my_tiles * jpt;
  const long long lim = d.spin_cycles;

  if (warp == 0) tc::tmem_alloc(&tmem_base, 512);
  if (tid == 128) {
    for (int s = 0; s < kTmStages; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 4);
      s_last_job[s] = -1;
    }
    s_fail = 0;
    s_issued = 0;
    s_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tbase = tmem_base;

  if (warp == 4) {
    // ---- producer: one thread issues every TMA box of this CTA's jobs
    if (lane == 0) {
      const uint32_t down_bytes = 9u * kTmSlotBytes, up_bytes = (last ? 5u : 3u) * kTmSlotBytes;
      for (int g = 0; g < njobs; ++g) {
        const int s = g % kTmStages;
        if (g >= kTmStages && !tc::mbar_wait_cycles(&empty[s], ((g / kTmStages) - 1) & 1, lim)) {
          s_fail = 1;
          break;
        }
        if (*(volatile int*)&s_fail) break;
        const int t = blockIdx.x + (g / jpt) * gridDim.x, c = g % jpt;
        const int x = (t % nbx) * 32, y = (t / nbx) * 4;
        uint8_t* st = smem + s * kTmStageBytes;
        if (g == d.fault_skip_job) {  // test hook: leave this job unissued
          s_issued = g + 1;
          continue;
        }
        if (c < nd) {
          const int kk_lo = kz - 1 - c * kKCT - (kKCT - 1);
          tc::mbar_arrive_expect_tx(&full[s], down_bytes);
          // levels kk of w, fmzf, qv and kk-1 of the others share a slot index
          tc::tma_load_3d(st + 0 * kTmSlotBytes, &maps.m[CM_W], x, y, kk_lo, &full[s]);
          tc::tma_load_3d(st + 1 * kTmSlotBytes, &maps.m[CM_FMZF], x, y, kk_lo, &full[s]);
          tc::tma_load_3d(st + 2 * kTmSlotBytes, &maps.m[CM_QV], x, y, kk_lo, &full[s]);
          tc::tma_load_3d(st + 3 * kTmSlotBytes, &maps.m[CM_TET], x, y, kk_lo - 1, &full[s]);
          tc::tma_load_3d(st + 4 * kTmSlotBytes, &maps.m[CM_PAI], x, y, kk_lo - 1, &full[s]);
          tc::tma_load_3d(st + 5 * kTmSlotBytes, &maps.m[CM_QSAT], x, y, kk_lo - 1, &full[s]);
          tc::tma_load_3d(st + 6 * kTmSlotBytes, &maps.m[CM_ZD], x, y, kk_lo - 1, &full[s]);
          tc::tma_load_3d(st + 7 * kTmSlotBytes, &maps.m[CM_FMZ], x, y, kk_lo - 1, &full[s]);
          tc::tma_load_3d(st + 8 * kTmSlotBytes, &maps.m[CM_T], x, y, kk_lo - 1, &full[s]);
        } else {
          const int m0 = (c - nd) * kKCT;
          tc::mbar_arrive_expect_tx(&full[s], up_bytes);
          tc::tma_load_3d(st + 0 * kTmSlotBytes, &maps.m[CM_QC], x, y, m0, &full[s]);
          tc::tma_load_3d(st + 1 * kTmSlotBytes, &maps.m[CM_QWL], x, y, m0, &full[s]);
          tc::tma_load_3d(st + 2 * kTmSlotBytes, &maps.m[CM_QWI], x, y, m0, &full[s]);
          if (last) {
            tc::tma_load_3d(st + 3 * kTmSlotBytes, &maps.m[CM_S], x, y, m0, &full[s]);
            tc::tma_load_3d(st + 4 * kTmSlotBytes, &maps.m[CM_FMZF], x, y, m0, &full[s]);
          }
        }
        s_last_job[s] = g;
        s_issued = g + 1;
      }
    }
  } else {
    // ---- compute warps: warp w holds row i = 4 by + w of the tile, lane = j
    const uint32_t trow = tbase + ((uint32_t)(warp * 32) << 16);
    const T ns = T(nsound), ns1 = T(nsound - 1);
    const T zcs2 = d.zcs2, dts = d.dts, egdts = d.egdts, dtrdz = d.dtrdz;
    const T rdrcv = T(kRdrcv);
    const T* __restrict__ FF = d.ffilt;
    int g = 0;  // job counter, in the producer's order
    bool fail = false;
    auto wait_full = [&](int job) -> const float* {
      const int s = job % kTmStages;
      bool ok = tc::mbar_wait_cycles(&full[s], (job / kTmStages) & 1, lim);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) {
        if (lane == 0) s_fail = 1;
        fail = true;
        return nullptr;
      }
      return reinterpret_cast<const float*>(smem + s * kTmStageBytes);
    };
    auto release = [&](int job) {
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&empty[job % kTmStages]);
    };
    // slot a, level index q (0 .. kKCT-1) of this thread's column
    const int sl = warp * 32 + lane;
    auto S_ = [&](const float* st, int a, int q) { return st[a * (kTmSlotBytes / 4) + q * 128 + sl]; };

    for (int tl = 0; tl < my_tiles && !fail; ++tl) {
      const int t = blockIdx.x + tl * gridDim.x;
      const int jj = (t % nbx) * 32 + lane, ii = (t / nbx) * 4 + warp;
      const bool own = jj < nj && ii < ni;
      const size_t c = own ? (size_t)jj + (size_t)nj * ii : 0;
      // level kz-1 values the down-sweep starts from, surface w, and qv(0)
      // for the record of level 0 (columns outside the domain read column 0)
      size_t o = (size_t)(kz - 1) * pl;
      T zd_k = d.zdiv2b[c + o], tk = d.tetav[c + o], pk = d.pai[c + o], fk = d.fmz[c + o], qsk = d.qsat[c + o];
      const T wsurf = d.w[c + (size_t)kz * pl];
      const T qv0 = d.q[0][c];
      float wkp1 = wsurf;
      double cwp1 = 1.0;  // 1 - wwkw(kz+1)

      // (b) down-sweep k = kz .. 2 (reference order)
      for (int cc = 0; cc < nd; ++cc, ++g) {
        const float* st = wait_full(g);
        if (!st) break;
        const int kk_hi = kz - 1 - cc * kKCT, kk_lo = kk_hi - (kKCT - 1);
        for (int kk = kk_hi; kk >= kk_lo && kk >= 1; --kk) {
          const int q = kk - kk_lo;
          const T wk = S_(st, 0, q), fz = S_(st, 1, q), qvk = S_(st, 2, q), ff = FF[kk];
          const T tkm = S_(st, 3, q), pkm = S_(st, 4, q), qskm = S_(st, 5, q), zd_km = S_(st, 6, q);
          const T fkm = S_(st, 7, q), tm = S_(st, 8, q);
          T zrom1w = ((T(0.5) * T(kCpd)) * fz) * (tkm + tk);
          zrom1w = zrom1w - (((((T(kCpd) * wk) * fz) * fz) * ns) * dtrdz) * (tkm - tk);
          if (qvk > T(0.96) * qsk && wk > T(0.1)) {
            const T zqs = T(0.5) * (qsk + qskm);
            const T zdth = ((((((T(kEgrav) * wk) * ns1) * dts) * T(kWlhv)) * T(kWlhv)) * zqs) /
                           ((((T(kCpd) * pkm) * T(kRwat)) * tm) * tm);
            zrom1w = zrom1w + zdth * fz;
          }
          T zwexpl = (wk - (zrom1w * dtrdz) * (pkm - pk)) - egdts;
          zwexpl = zwexpl + ((T(kRdrcv) * zrom1w) * dtrdz) * (pkm * zd_km - pk * zd_k);
          const T zu_t = ((zcs2 * fkm) * zrom1w) * pkm + ff;
          const T zd_t = ((zcs2 * fk) * zrom1w) * pk + ff;
          // FP64 pivot recurrence in complement form (as b_sound_column)
          const double zu = widen_f32(zu_t), zdd = widen_f32(zd_t);
          const double tt = fma(zdd, cwp1, 1.0);
          const double den = tt + zu;
          float r;
          asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(narrow_trunc(den)));
          const double q0 = widen_f32(narrow_trunc(tt) * r);
          const double rem = fma(-den, q0, tt);
          cwp1 = q0 + widen_f32(r * narrow_trunc(rem));
          const float wpk = r * (zwexpl + zd_t * wkp1);
          const float wwk = r * zu_t;
          // record of level kk: zdiv2b, fmz, qv, tetav, pai, old w, wp, ww
          const uint32_t rec[8] = {fbits(zd_k), fbits(fk), fbits(qvk), fbits(tk), fbits(pk), fbits(wk), fbits(wpk),
                                   fbits(wwk)};
          tc::tmem_st8(trow + (uint32_t)(8 * kk), rec);
          wkp1 = wpk;
          zd_k = zd_km; tk = tkm; pk = pkm; fk = fkm; qsk = qskm;
        }
        release(g);
      }
      if (fail) break;
      {  // record of level 0 (no recurrence values)
        const uint32_t rec[8] = {fbits(zd_k), fbits(fk), fbits(qv0), fbits(tk), fbits(pk), 0u, 0u, 0u};
        tc::tmem_st8(trow, rec);
      }
      tc::tmem_wait_st();

      // (c) back-substitution (:681-686) fused with the Exner/theta update
      // of the level above (:690-728); w(1) = 0 always (init_moloch :260-262)
      uint32_t cur[8], nxt[8];
      tc::tmem_ld8(trow, cur);
      tc::tmem_wait_ld8(cur);
      T fzd = bitsf(cur[0]), ffmz = bitsf(cur[1]), fqv = bitsf(cur[2]), ftet = bitsf(cur[3]), fpai = bitsf(cur[4]);
      if (kz > 1) tc::tmem_ld8(trow + 8u, nxt);
      float wlo_d = 0.f;
      T wlo = T(0);
      int kk = 1;
      for (int cc = 0; cc < nu; ++cc, ++g) {
        const float* st = wait_full(g);
        if (!st) break;
        const int m0 = cc * kKCT;
        for (; kk <= kz && kk - 1 < m0 + kKCT; ++kk) {
          const int m = kk - 1, q = m - m0;
          T wn;
          if (kk < kz) {
            tc::tmem_wait_ld8(nxt);
#pragma unroll
            for (int e = 0; e < 8; ++e) cur[e] = nxt[e];
            if (kk + 1 < kz) tc::tmem_ld8(trow + (uint32_t)(8 * (kk + 1)), nxt);
            wlo_d = bitsf(cur[6]) + bitsf(cur[7]) * wlo_d;
            wn = (T)wlo_d;
            if (own) {
              const size_t qq = c + (size_t)kk * pl;
              d.deltaw[qq] = (-bitsf(cur[5])) + wn;
              d.w[qq] = wn;
            }
          } else {
            wn = wsurf;
          }
          // finalize level m = kk-1 with w(m) = wlo, w(m+1) = wn
          const T fqc = S_(st, 0, q), fqwl = S_(st, 1, q), fqwi = S_(st, 2, q);
          T zd = fzd;
          zd = zd + (dtrdz * ffmz) * (wlo - wn);
          zd = (zd * ((T(1) + T(0.86) * fqv) + T(3.2) * fqc)) / ((T(1) + T(0.96) * fqv) + T(4.8) * fqc);
          if (own) {
            const size_t qm = c + (size_t)m * pl;
            d.tetav[qm] = ftet * (T(1) + (rdrcv * zd) * ((T(0.25) * fqv + T(4.2) * fqwl) + T(2.1) * fqwi));
            if (jj == nj - 1) d.ep_j[ii + (size_t)ni * m] = fpai;
            if (ii == ni - 1) d.ep_i[jj + (size_t)nj * m] = fpai;
            d.pai[qm] = fpai * (T(1) - rdrcv * zd);
            if (last) d.s[qm] = m == 0 ? T(0) : (wlo + S_(st, 3, q)) * S_(st, 4, q);  // Equation 10 (:843-849)
          }
          wlo = wn;
          if (kk < kz) {
            fzd = bitsf(cur[0]); ffmz = bitsf(cur[1]); fqv = bitsf(cur[2]); ftet = bitsf(cur[3]); fpai = bitsf(cur[4]);
          }
        }
        release(g);
      }
      if (fail) break;
      if (last && own) d.s[c + (size_t)kz * pl] = T(0);
    }
    // no TMEM load or store of this thread may be in flight when TMEM is
    // freed (a wait that gave up can leave one of either)
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    if (lane == 0 && warp == 0) s_consumed = g;  // jobs every compute warp has finished (or gave up at)
  }
  tc::tc_fence_before();
  __syncthreads();
  if (tid == 128 && s_fail) {
    // a wait gave up: flag it and let the copies still in flight land
    // before the CTA's shared memory is released (bounded)
    atomicExch(d.kerr, 1);
    for (int s = 0; s < kTmStages; ++s) {
      const int j = s_last_job[s];
      if (j >= s_consumed) tc::mbar_wait_cycles(&full[s], (j / kTmStages) & 1, lim);
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (warp == 0) tc::tmem_dealloc(tbase, 512);
}

}  // namespace MOLOCH_KNS
}  // namespace moloch
