// Implicit w (Thomas, one thread per column) + Exner/theta/pai update of
// sound() for FP32 storage (nompi/mod_moloch.F90:634-728, :843-849), staged
// by TMA, with the column state the back-substitution needs kept on chip.
//
// The one-thread-per-column kernel (b_sound_column) reads the down-sweep's
// inputs, writes an FP32 stash of the recurrence, and in the
// back-substitution reads the stash and six of the inputs again; at
// 512 x 512 x 60 about 175 K columns are in flight, so level k is read again
// 2k+1 level steps later, long after L2 evicted it (1.49x the algorithmic
// DRAM bytes).  Here:
//   * a persistent CTA per SM walks tiles of 32 (j) x 8 (i) columns, eight
//     compute warps (one per row of 32 columns, two per SM sub-partition,
//     so two FP64 pivot chains interleave), one thread per column;
//   * a producer warp stages chunks of kKCT levels of every input with 3-D
//     TMA boxes (32 x 8 x kKCT) into a ring of shared-memory stages, running
//     ahead through the down-sweep chunks, the back-substitution chunks and
//     the next tile's chunks, so loads never wait on the recurrence;
//   * the recurrence's wp, ww, the old w and zdiv2b of each level go into
//     the thread's own TMEM lane (4 words a level: warps w and w+4 share a
//     lane quarter and take 256 columns each), which stands in for
//     registers that cannot be indexed by level;
//   * fmz, qv, tetav, pai, which the back-substitution reads again, are
//     loaded with an L2 evict_last policy in the down-sweep (the resident
//     set of all CTAs is 152 x 256 columns x 60 levels x 16 B = 37 MB at
//     this size) and every other load and store with evict_first, so the
//     re-reads hit L2.
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

constexpr int kKCT = 8;                          // levels per staged chunk (a multiple of 4)
constexpr int kTmStages = 3;                     // ring depth
constexpr int kTmSlots = 9;                      // arrays per stage
constexpr int kTmRows = 8;                       // rows (i) per tile = compute warps
constexpr int kTmSlotBytes = kKCT * kTmRows * 32 * 4;  // one 32 x 8 x kKCT FP32 box
constexpr int kTmStageBytes = kTmSlots * kTmSlotBytes;
constexpr int kTmSmem = kTmStages * kTmStageBytes + 128;  // + alignment slack
constexpr int kTmThreads = 32 * (kTmRows + 1);   // compute warps + producer warp
constexpr int kTmMaxKz = 64;                     // 4 words x kz TMEM columns per warp

// tensor maps of the staged arrays (tetav, pai, qv, qc depend on the
// advected-field buffer set, so the host keeps one set per parity)
enum ColMap { CM_W = 0, CM_FMZF, CM_QV, CM_TET, CM_PAI, CM_QSAT, CM_ZD, CM_FMZ, CM_T, CM_QC, CM_QWL, CM_QWI, CM_S,
              CM_COUNT };
struct ColumnMaps {
  CUtensorMap m[CM_COUNT];
};
// box shapes: k_sound_column_tm, k_sound_column_tw with 12 and 16 rows
constexpr int kColumnMapConfigs = 3;

// FP32 <-> FP64 conversions on the integer pipe for values known to lie in
// the FP32 normal range -- in the pivot recurrence zu, zd > 0, tt, den >= 1,
// q0 in (0, 1] -- giving the bits widen_f32 / narrow_trunc give there,
// without their zero, subnormal, infinity and NaN cases (which cost most of
// their operations, all on the recurrence's dependency chain).  The
// quotient's residual may be zero: narrow_residual flushes magnitudes below
// the FP32 normal range to zero.
__device__ __forceinline__ double widen_normal(float x) {
  const unsigned b = __float_as_uint(x);
  const unsigned hi = (((b & 0x7fffffffu) >> 3) + 0x38000000u) | (b & 0x80000000u);
  return __hiloint2double((int)hi, (int)(b << 29));
}
__device__ __forceinline__ float narrow_normal(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned m = (__funnelshift_l(lo, hi, 3) - (896u << 23)) & 0x7fffffffu;
  return __uint_as_float(m | (hi & 0x80000000u));
}
__device__ __forceinline__ float narrow_residual(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned m = (__funnelshift_l(lo, hi, 3) - (896u << 23)) & 0x7fffffffu;
  return __uint_as_float(((hi & 0x7fffffffu) < 0x38100000u ? 0u : m) | (hi & 0x80000000u));
}

__device__ __forceinline__ uint32_t fbits(float x) { return __float_as_uint(x); }
__device__ __forceinline__ float bitsf(uint32_t x) { return __uint_as_float(x); }

template <class T, int LAST>
__global__ void __launch_bounds__(kTmThreads, 1)
    k_sound_column_tm(View<T> d, const __grid_constant__ ColumnMaps maps, int nsound) {
  constexpr bool last = LAST != 0;  // the last substep also completes s (Equation 10)
  static_assert(sizeof(T) == 4, "FP32 storage only");
  if (d.sur_skip && *d.sur_skip) return;  // the surrogate took this cycle
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full[kTmStages], empty[kTmStages];
  __shared__ uint32_t tmem_base;
  __shared__ int s_fail, s_consumed;
  __shared__ int s_last_job[kTmStages];
  __shared__ float s_ff[kTmMaxKz];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 127) & ~(uintptr_t)127);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nj = d.nj, ni = d.ni, kz = d.kz;
  const size_t pl = d.pl;
  const int nbx = (nj + 31) / 32, nby = (ni + kTmRows - 1) / kTmRows, ntiles = nbx * nby;
  const int nd = (kz - 1 + kKCT - 1) / kKCT;  // down-sweep chunks: kk = kz-1 .. 1
  const int nu = (kz + kKCT - 1) / kKCT;      // back-substitution chunks: kk = 1 .. kz
  const int jpt = nd + nu;                    // jobs per tile
  const int my_tiles = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  const int njobs = my_tiles * jpt;
  const long long lim = d.spin_cycles;

  if (warp == 0) tc::tmem_alloc(&tmem_base, 512);
  if (tid == 32 * kTmRows) {
    for (int q = 0; q < kTmStages; ++q) {
      tc::mbar_init(&full[q], 1);
      tc::mbar_init(&empty[q], kTmRows);
      s_last_job[q] = -1;
    }
    s_fail = 0;
    s_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int k = tid; k < kz; k += blockDim.x) s_ff[k] = d.ffilt[k];
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tbase = tmem_base;

  if (warp == kTmRows) {
    // ---- producer: one thread issues every TMA box of this CTA's jobs
    if (lane == 0) {
      const uint64_t keep = tc::policy_evict_last(), once = tc::policy_evict_first();
      const uint32_t down_bytes = 9u * kTmSlotBytes, up_bytes = (last ? 9u : 7u) * kTmSlotBytes;
      for (int g = 0; g < njobs; ++g) {
        const int q = g % kTmStages;
        if (g >= kTmStages && !tc::mbar_wait_cycles(&empty[q], ((g / kTmStages) - 1) & 1, lim)) {
          s_fail = 1;
          break;
        }
        if (*(volatile int*)&s_fail) break;
        if (g == d.fault_skip_job) continue;  // test hook: leave this job unissued
        const int t = (int)blockIdx.x + (g / jpt) * (int)gridDim.x, c = g % jpt;
        const int x = (t % nbx) * 32, y = (t / nbx) * kTmRows;
        uint8_t* stg = smem + q * kTmStageBytes;
        auto box = [&](int slot, int map, int z, uint64_t pol) {
          tc::tma_load_3d_hint(stg + slot * kTmSlotBytes, &maps.m[map], x, y, z, &full[q], pol);
        };
        if (c < nd) {
          const int kk_lo = kz - 1 - c * kKCT - (kKCT - 1);
          tc::mbar_arrive_expect_tx(&full[q], down_bytes);
          // level kk of w, fmzf, qv and level kk-1 of the others share a
          // slot index; fmz, qv, tetav, pai are read again by the
          // back-substitution and stay in L2
          box(0, CM_W, kk_lo, once);
          box(1, CM_FMZF, kk_lo, once);
          box(2, CM_QV, kk_lo, keep);
          box(3, CM_TET, kk_lo - 1, keep);
          box(4, CM_PAI, kk_lo - 1, keep);
          box(5, CM_QSAT, kk_lo - 1, once);
          box(6, CM_ZD, kk_lo - 1, once);
          box(7, CM_FMZ, kk_lo - 1, keep);
          box(8, CM_T, kk_lo - 1, once);
        } else {
          const int m0 = (c - nd) * kKCT;
          tc::mbar_arrive_expect_tx(&full[q], up_bytes);
          box(0, CM_FMZ, m0, once);
          box(1, CM_QV, m0, once);
          box(2, CM_TET, m0, once);
          box(3, CM_PAI, m0, once);
          box(4, CM_QC, m0, once);
          box(5, CM_QWL, m0, once);
          box(6, CM_QWI, m0, once);
          if (last) {
            box(7, CM_S, m0, once);
            box(8, CM_FMZF, m0, once);
          }
        }
        s_last_job[q] = g;
      }
    }
  } else {
    // ---- compute warps: warp w holds row i = 8 by + w of the tile, lane = j;
    // its TMEM: lane quarter w % 4, columns 256 (w / 4) .. +255, 4 per level
    const uint32_t trow = tbase + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)((warp >> 2) * 256);
    const uint64_t once = tc::policy_evict_first();
    const T ns = T(nsound), ns1 = T(nsound - 1);
    const T zcs2 = d.zcs2, dts = d.dts, egdts = d.egdts, dtrdz = d.dtrdz;
    const T rdrcv = T(kRdrcv);
    int g = 0;  // job counter, in the producer's order
    bool fail = false;
    auto wait_full = [&](int job) -> const float* {
      const int q = job % kTmStages;
      bool ok = tc::mbar_wait_cycles(&full[q], (job / kTmStages) & 1, lim);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) {
        if (lane == 0) s_fail = 1;
        fail = true;
        return nullptr;
      }
      return reinterpret_cast<const float*>(smem + q * kTmStageBytes);
    };
    auto release = [&](int job) {
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&empty[job % kTmStages]);
    };
    // slot a, level index q (0 .. kKCT-1) of this thread's column
    const int sl = warp * 32 + lane;
    auto S_ = [&](const float* st, int a, int q) { return st[a * (kTmSlotBytes / 4) + q * (kTmRows * 32) + sl]; };
    // the values a tile starts from: level kz-1 of zdiv2b, tetav, pai, fmz,
    // qsat and the surface w (columns outside the domain read column 0)
    struct Init { T zd, tk, pk, fk, qsk, wsurf; };
    auto load_init = [&](int t, Init& v) {
      const int jj = (t % nbx) * 32 + lane, ii = (t / nbx) * kTmRows + warp;
      const size_t c = (jj < nj && ii < ni) ? (size_t)jj + (size_t)nj * ii : 0;
      const size_t o = (size_t)(kz - 1) * pl;
      v.zd = d.zdiv2b[c + o]; v.tk = d.tetav[c + o]; v.pk = d.pai[c + o]; v.fk = d.fmz[c + o];
      v.qsk = d.qsat[c + o]; v.wsurf = d.w[c + (size_t)kz * pl];
    };
    Init nx{};
    if (my_tiles > 0) load_init((int)blockIdx.x, nx);
    const int nfull = (kz - 1) / kKCT;  // back-substitution chunks whose levels all lie below kz

    for (int tl = 0; tl < my_tiles && !fail; ++tl) {
      const int t = (int)blockIdx.x + tl * (int)gridDim.x;
      const int jj = (t % nbx) * 32 + lane, ii = (t / nbx) * kTmRows + warp;
      const bool own = jj < nj && ii < ni;
      const size_t c = own ? (size_t)jj + (size_t)nj * ii : 0;
      T zd_k = nx.zd, tk = nx.tk, pk = nx.pk, fk = nx.fk, qsk = nx.qsk;
      const T wsurf = nx.wsurf;
      float wkp1 = wsurf;
      double cwp1 = 1.0;  // 1 - wwkw(kz+1)

      // one level kk of the down-sweep from slot index q; the record of
      // level kk (wp, ww, old w, zdiv2b) goes to rec[0..3]
      auto dn_level = [&](const float* st, const int q, const int kk, uint32_t* rec) {
        const T wk = S_(st, 0, q), fz = S_(st, 1, q), qvk = S_(st, 2, q), ff = s_ff[kk];
        const T tkm = S_(st, 3, q), pkm = S_(st, 4, q), qskm = S_(st, 5, q), zd_km = S_(st, 6, q);
        const T fkm = S_(st, 7, q), tm = S_(st, 8, q);
        T zrom1w = ((T(0.5) * T(kCpd)) * fz) * (tkm + tk);
        zrom1w = zrom1w - (((((T(kCpd) * wk) * fz) * fz) * ns) * dtrdz) * (tkm - tk);
        zrom1w = zrom1w_moist(zrom1w, qvk, qsk, qskm, wk, fz, pkm, tm, ns1, dts);
        T zwexpl = (wk - (zrom1w * dtrdz) * (pkm - pk)) - egdts;
        zwexpl = zwexpl + ((T(kRdrcv) * zrom1w) * dtrdz) * prod_sub(pkm, zd_km, pk, zd_k);
        const T zu_t = ((zcs2 * fkm) * zrom1w) * pkm + ff;
        const T zd_t = ((zcs2 * fk) * zrom1w) * pk + ff;
        // FP64 pivot recurrence in complement form (as b_sound_column), with
        // the conversions specialised to the ranges they see here
        const double zu = widen_normal(zu_t), zdd = widen_normal(zd_t);
        const double tt = fma(zdd, cwp1, 1.0);
        const double den = tt + zu;
        float r;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(narrow_normal(den)));
        const double q0 = widen_normal(narrow_normal(tt) * r);
        const double rem = fma(-den, q0, tt);
        cwp1 = q0 + widen_normal(r * narrow_residual(rem));
        const float wpk = r * (zwexpl + zd_t * wkp1);
        rec[0] = fbits(wpk); rec[1] = fbits(r * zu_t); rec[2] = fbits(wk); rec[3] = fbits(zd_k);
        wkp1 = wpk;
        zd_k = zd_km; tk = tkm; pk = pkm; fk = fkm; qsk = qskm;
      };

      // (b) down-sweep k = kz .. 2 (reference order)
      for (int cc = 0; cc < nd; ++cc, ++g) {
        const float* st = wait_full(g);
        if (!st) break;
        const int kk_hi = kz - 1 - cc * kKCT, kk_lo = kk_hi - (kKCT - 1);
        if (kk_lo >= 1) {  // a whole chunk: four levels, one TMEM store
          uint32_t rec[4 * kKCT];
#pragma unroll
          for (int u = 0; u < kKCT; ++u) dn_level(st, kKCT - 1 - u, kk_hi - u, rec + 4 * (kKCT - 1 - u));
#pragma unroll
          for (int h = 0; h < kKCT / 4; ++h) tc::tmem_st16p(trow + (uint32_t)(4 * kk_lo + 16 * h), rec + 16 * h);
        } else {
          for (int kk = kk_hi; kk >= 1; --kk) {
            uint32_t rec[4];
            dn_level(st, kk - kk_lo, kk, rec);
            tc::tmem_st4(trow + (uint32_t)(4 * kk), rec[0], rec[1], rec[2], rec[3]);
          }
        }
        release(g);
      }
      if (fail) break;
      tc::tmem_st4(trow, 0u, 0u, 0u, fbits(zd_k));  // level 0: zdiv2b only
      tc::tmem_wait_st();
      // the next tile's starting values, loaded while this one finishes
      if (tl + 1 < my_tiles) load_init(t + (int)gridDim.x, nx);

      // (c) back-substitution (:681-686) fused with the Exner/theta update
      // of the level above (:690-728); w(1) = 0 always (init_moloch :260-262).
      // Chunk cc holds levels kk = 4 cc + 1 .. 4 cc + 4; the records of a
      // whole chunk (all kk < kz) are 16 consecutive TMEM columns, loaded
      // one chunk ahead.
      float wlo_d = 0.f;
      T wlo = T(0), fzd;
      {
        uint32_t r0[4];
        tc::tmem_ld4(trow, r0);
        tc::tmem_wait_ld4(r0);
        fzd = bitsf(r0[3]);
      }
      uint32_t cur[4 * kKCT], nxt[4 * kKCT];
      if (nfull > 0) {
#pragma unroll
        for (int h = 0; h < kKCT / 4; ++h) tc::tmem_ld16p(trow + 4u + 16u * h, nxt + 16 * h);
      }
      T* __restrict__ pw = d.w + c;
      T* __restrict__ pdw = d.deltaw + c;
      T* __restrict__ ptet = d.tetav + c;
      T* __restrict__ ppai = d.pai + c;
      T* __restrict__ psv = d.s + c;
      // level kk (record rec when kk < kz) and the finalize of level kk-1
      auto up_level = [&](const float* st, const int q, const int kk, const uint32_t* rec) {
        const int m = kk - 1;
        T wn, zd_next = T(0);
        if (rec) {
          wlo_d = bitsf(rec[0]) + bitsf(rec[1]) * wlo_d;
          wn = (T)wlo_d;
          zd_next = bitsf(rec[3]);
          if (own) {
            const size_t qq = (size_t)kk * pl;
            tc::st_hint(pdw + qq, (-bitsf(rec[2])) + wn, once);
            tc::st_hint(pw + qq, wn, once);
          }
        } else {
          wn = wsurf;
        }
        const T ffmz = S_(st, 0, q), fqv = S_(st, 1, q), ftet = S_(st, 2, q), fpai = S_(st, 3, q);
        const T fqc = S_(st, 4, q), fqwl = S_(st, 5, q), fqwi = S_(st, 6, q);
        T zd = fzd;
        zd = zd + (dtrdz * ffmz) * (wlo - wn);
        zd = div_corr(zd * ((T(1) + T(0.86) * fqv) + T(3.2) * fqc), (T(1) + T(0.96) * fqv) + T(4.8) * fqc);
        if (own) {
          const size_t qm = (size_t)m * pl;
          tc::st_hint(ptet + qm,
                      ftet * (T(1) + (rdrcv * zd) * (prod_add(T(0.25), fqv, T(4.2), fqwl) + T(2.1) * fqwi)), once);
          if (jj == nj - 1) d.ep_j[ii + (size_t)ni * m] = fpai;
          if (ii == ni - 1) d.ep_i[jj + (size_t)nj * m] = fpai;
          tc::st_hint(ppai + qm, fpai * (T(1) - rdrcv * zd), once);
          if (last) tc::st_hint(psv + qm, m == 0 ? T(0) : (wlo + S_(st, 7, q)) * S_(st, 8, q), once);  // Eq. 10
        }
        wlo = wn;
        fzd = zd_next;
      };
      for (int cc = 0; cc < nu; ++cc, ++g) {
        const float* st = wait_full(g);
        if (!st) break;
        const int kk0 = cc * kKCT + 1;
        if (cc < nfull) {
#pragma unroll
          for (int h = 0; h < kKCT / 4; ++h) tc::tmem_wait_ld16p(nxt + 16 * h);
#pragma unroll
          for (int e = 0; e < 4 * kKCT; ++e) cur[e] = nxt[e];
          if (cc + 1 < nfull) {
#pragma unroll
            for (int h = 0; h < kKCT / 4; ++h) tc::tmem_ld16p(trow + (uint32_t)(4 * (kk0 + kKCT) + 16 * h), nxt + 16 * h);
          }
#pragma unroll
          for (int u = 0; u < kKCT; ++u) up_level(st, u, kk0 + u, cur + 4 * u);
        } else {
          for (int kk = kk0; kk <= kz && kk < kk0 + kKCT; ++kk) {
            if (kk < kz) {
              uint32_t rec[4];
              tc::tmem_ld4(trow + (uint32_t)(4 * kk), rec);
              tc::tmem_wait_ld4(rec);
              up_level(st, kk - kk0, kk, rec);
            } else {
              up_level(st, kk - kk0, kk, nullptr);
            }
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
    if (lane == 0 && warp == 0) s_consumed = g;  // first job warp 0 did not finish
  }
  tc::tc_fence_before();
  __syncthreads();
  if (tid == 32 * kTmRows && s_fail) {
    // a wait gave up: flag it and let the copies still in flight land
    // before the CTA's shared memory is released (bounded)
    atomicExch(d.kerr, 1);
    for (int q = 0; q < kTmStages; ++q) {
      const int j = s_last_job[q];
      if (j >= s_consumed) tc::mbar_wait_cycles(&full[q], (j / kTmStages) & 1, lim);
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (warp == 0) tc::tmem_dealloc(tbase, 512);
}


// ---- the same solve with two words of column state a level in TMEM ------
// k_sound_column_tm keeps four words a level in TMEM (wp, ww, the old w,
// zdiv2b), which allows two compute warps a lane quarter, eight a CTA: the
// serial chains then leave the SM issuing in about 40 % of its cycles.
// k_sound_column_tw keeps only wp and ww there.  The old w and zdiv2b are
// staged a second time for the back-substitution, like fmz, qv, tetav and
// pai (all six are loaded with L2 evict_last in the down-sweep, so the
// second read hits L2), and ROWS / 4 warps share a lane quarter: 12 or 16
// compute warps, one row of the 32 x ROWS column tile each, in chunks of
// four levels.  The arithmetic per level is that of k_sound_column_tm, so
// the results are bit-identical to it.
template <int ROWS>
struct TwCfg {
  static constexpr int rows = ROWS;
  static constexpr int kct = 4;                        // levels per staged chunk
  static constexpr int stages = ROWS <= 12 ? 3 : 2;    // ring depth within 227 KB
  static constexpr int slots = 11;                     // arrays per stage (back-substitution, last substep)
  static constexpr int slot_bytes = kct * ROWS * 32 * 4;
  static constexpr int stage_bytes = slots * slot_bytes;
  static constexpr int smem = stages * stage_bytes + 128;
  static constexpr int threads = 32 * (ROWS + 1);
  static constexpr int bank = 128;                     // TMEM columns per warp: 2 words x 64 levels
  static_assert(ROWS % 4 == 0 && (ROWS / 4) * bank <= 512, "TMEM holds 512 columns a lane");
};

// The arrays and scalars of the domain a column tile belongs to
template <class T>
struct TwDom {
  const T *zdiv2b, *fmz, *qsat, *ffilt;
  T *w, *deltaw, *tetav, *pai, *s, *ep_j, *ep_i;
  int nj, ni, kz;
  size_t pl;
  T zcs2, dts, egdts, dtrdz;
};
template <class T>
__device__ __forceinline__ TwDom<T> tw_dom(const View<T>& d) {
  TwDom<T> v;
  v.zdiv2b = d.zdiv2b; v.fmz = d.fmz; v.qsat = d.qsat; v.ffilt = d.ffilt;
  v.w = d.w; v.deltaw = d.deltaw; v.tetav = d.tetav; v.pai = d.pai; v.s = d.s; v.ep_j = d.ep_j; v.ep_i = d.ep_i;
  v.nj = d.nj; v.ni = d.ni; v.kz = d.kz; v.pl = d.pl;
  v.zcs2 = d.zcs2; v.dts = d.dts; v.egdts = d.egdts; v.dtrdz = d.dtrdz;
  return v;
}

// The body of k_sound_column_tw (one domain: BATCH false, the tiles of
// that domain computed from the tile number) and of kb_sound_column_tw
// (an ensemble: BATCH true, tile t is tiles[t] = {member, tile x, tile y},
// the member's view in views[member] and its tensor maps in
// cms[2 member + fcur]).  A CTA walks tiles blockIdx.x, + gridDim.x, ...;
// the producer and the compute warps count the same jobs (the chunks of
// each tile, which depend on the tile's kz).
template <class T, int LAST, int ROWS, bool BATCH>
__device__ __forceinline__ void column_tw_body(const View<T>* views, const ColumnMaps* cms, const int4* tiles,
                                               int ntiles_in, int fcur, int nsound, int* kerr, long long lim,
                                               int skip_job) {
  using C = TwCfg<ROWS>;
  constexpr int KC = C::kct, NST = C::stages, SLOTF = C::slot_bytes / 4;
  constexpr bool last = LAST != 0;  // the last substep also completes s (Equation 10)
  static_assert(sizeof(T) == 4, "FP32 storage only");
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full[NST], empty[NST];
  __shared__ uint32_t tmem_base;
  __shared__ int s_fail, s_consumed;
  __shared__ int s_last_job[NST];
  __shared__ float s_ff[kTmMaxKz];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 127) & ~(uintptr_t)127);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // one domain: tiles of nbx x nby
  const int nbx1 = BATCH ? 1 : (views[0].nj + 31) / 32;
  const int ntiles = BATCH ? ntiles_in : nbx1 * ((views[0].ni + ROWS - 1) / ROWS);
  struct Tile { int m, x, y; };
  auto tile_of = [&](int t) -> Tile {
    if constexpr (BATCH) {
      const int4 q = tiles[t];
      return {q.x, q.y * 32, q.z * ROWS};
    } else {
      return {0, (t % nbx1) * 32, (t / nbx1) * ROWS};
    }
  };

  if (warp == 0) tc::tmem_alloc(&tmem_base, 512);
  if (tid == 32 * ROWS) {
    for (int q = 0; q < NST; ++q) {
      tc::mbar_init(&full[q], 1);
      tc::mbar_init(&empty[q], ROWS);
      s_last_job[q] = -1;
    }
    s_fail = 0;
    s_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if constexpr (!BATCH)
    for (int k = tid; k < views[0].kz; k += blockDim.x) s_ff[k] = views[0].ffilt[k];
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tbase = tmem_base;

  if (warp == ROWS) {
    // ---- producer: one thread issues every TMA box of this CTA's jobs
    if (lane == 0) {
      const uint64_t keep = tc::policy_evict_last(), once = tc::policy_evict_first();
      const uint32_t down_bytes = 9u * C::slot_bytes, up_bytes = (last ? 11u : 9u) * C::slot_bytes;
      int g = 0;
      bool stop = false;
      for (int t = (int)blockIdx.x; t < ntiles && !stop; t += (int)gridDim.x) {
        const Tile tl = tile_of(t);
        const int kz = views[tl.m].kz;
        const int nd = (kz - 1 + KC - 1) / KC, jpt = nd + (kz + KC - 1) / KC;
        const CUtensorMap* mp = (BATCH ? cms[2 * tl.m + fcur] : cms[0]).m;
        for (int c = 0; c < jpt; ++c, ++g) {
          const int q = g % NST;
          if (g >= NST && !tc::mbar_wait_cycles(&empty[q], ((g / NST) - 1) & 1, lim)) {
            s_fail = 1;
            stop = true;
            break;
          }
          if (*(volatile int*)&s_fail) {
            stop = true;
            break;
          }
          if (g == skip_job) continue;  // test hook: leave this job unissued
          uint8_t* stg = smem + q * C::stage_bytes;
          auto box = [&](int slot, int map, int z, uint64_t pol) {
            tc::tma_load_3d_hint(stg + slot * C::slot_bytes, &mp[map], tl.x, tl.y, z, &full[q], pol);
          };
          if (c < nd) {
            const int kk_lo = kz - 1 - c * KC - (KC - 1);
            tc::mbar_arrive_expect_tx(&full[q], down_bytes);
            // level kk of w, fmzf, qv and level kk-1 of the others share a
            // slot index; w, qv, tetav, pai, zdiv2b, fmz are read again by
            // the back-substitution and stay in L2
            box(0, CM_W, kk_lo, keep);
            box(1, CM_FMZF, kk_lo, once);
            box(2, CM_QV, kk_lo, keep);
            box(3, CM_TET, kk_lo - 1, keep);
            box(4, CM_PAI, kk_lo - 1, keep);
            box(5, CM_QSAT, kk_lo - 1, once);
            box(6, CM_ZD, kk_lo - 1, keep);
            box(7, CM_FMZ, kk_lo - 1, keep);
            box(8, CM_T, kk_lo - 1, once);
          } else {
            // levels m = m0 .. m0+KC-1 of the arrays of the update, level
            // m+1 of the old w
            const int m0 = (c - nd) * KC;
            tc::mbar_arrive_expect_tx(&full[q], up_bytes);
            box(0, CM_FMZ, m0, once);
            box(1, CM_QV, m0, once);
            box(2, CM_TET, m0, once);
            box(3, CM_PAI, m0, once);
            box(4, CM_QC, m0, once);
            box(5, CM_QWL, m0, once);
            box(6, CM_QWI, m0, once);
            box(7, CM_W, m0 + 1, once);
            box(8, CM_ZD, m0, once);
            if (last) {
              box(9, CM_S, m0, once);
              box(10, CM_FMZF, m0, once);
            }
          }
          s_last_job[q] = g;
        }
      }
    }
  } else {
    // ---- compute warps: warp w holds row i = y + w of the tile, lane = j;
    // its TMEM: lane quarter w % 4, columns 128 (w / 4) .., 2 per level
    const uint32_t trow = tbase + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)((warp >> 2) * C::bank);
    const uint64_t once = tc::policy_evict_first();
    const T ns = T(nsound), ns1 = T(nsound - 1);
    const T rdrcv = T(kRdrcv);
    int g = 0;  // job counter, in the producer's order
    bool fail = false;
    auto wait_full = [&](int job) -> const float* {
      const int q = job % NST;
      bool ok = tc::mbar_wait_cycles(&full[q], (job / NST) & 1, lim);
      ok = __all_sync(0xffffffffu, ok);
      if (!ok) {
        if (lane == 0) s_fail = 1;
        fail = true;
        return nullptr;
      }
      return reinterpret_cast<const float*>(smem + q * C::stage_bytes);
    };
    auto release = [&](int job) {
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&empty[job % NST]);
    };
    // slot a, level index q (0 .. KC-1) of this thread's column
    const int sl = warp * 32 + lane;
    auto S_ = [&](const float* st, int a, int q) { return st[a * SLOTF + q * (ROWS * 32) + sl]; };
    // the values a tile starts from: level kz-1 of zdiv2b, tetav, pai, fmz,
    // qsat and the surface w (columns outside the domain read column 0)
    struct Init { T zd, tk, pk, fk, qsk, wsurf; };
    auto load_init = [&](int t, Init& v) {
      const Tile tl = tile_of(t);
      const TwDom<T> dm = tw_dom(views[tl.m]);
      const int jj = tl.x + lane, ii = tl.y + warp;
      const size_t c = (jj < dm.nj && ii < dm.ni) ? (size_t)jj + (size_t)dm.nj * ii : 0;
      const size_t o = (size_t)(dm.kz - 1) * dm.pl;
      v.zd = dm.zdiv2b[c + o]; v.tk = dm.tetav[c + o]; v.pk = dm.pai[c + o]; v.fk = dm.fmz[c + o];
      v.qsk = dm.qsat[c + o]; v.wsurf = dm.w[c + (size_t)dm.kz * dm.pl];
    };
    Init nx{};
    if ((int)blockIdx.x < ntiles) load_init((int)blockIdx.x, nx);

    for (int t = (int)blockIdx.x; t < ntiles && !fail; t += (int)gridDim.x) {
      const Tile tl = tile_of(t);
      const TwDom<T> v = tw_dom(views[tl.m]);
      const int nj = v.nj, ni = v.ni, kz = v.kz;
      const size_t pl = v.pl;
      const T zcs2 = v.zcs2, dts = v.dts, egdts = v.egdts, dtrdz = v.dtrdz;
      const int nd = (kz - 1 + KC - 1) / KC;  // down-sweep chunks: kk = kz-1 .. 1
      const int nu = (kz + KC - 1) / KC;      // back-substitution chunks: kk = 1 .. kz
      const int nfull = (kz - 1) / KC;        // back-substitution chunks whose levels all lie below kz
      const int jj = tl.x + lane, ii = tl.y + warp;
      const bool own = jj < nj && ii < ni;
      const size_t c = own ? (size_t)jj + (size_t)nj * ii : 0;
      T zd_k = nx.zd, tk = nx.tk, pk = nx.pk, fk = nx.fk, qsk = nx.qsk;
      const T wsurf = nx.wsurf;
      float wkp1 = wsurf;
      double cwp1 = 1.0;  // 1 - wwkw(kz+1)
      auto ffilt = [&](int kk) -> T {
        if constexpr (BATCH) return v.ffilt[kk];
        else return s_ff[kk];
      };

      // one level kk of the down-sweep from slot index q; the record of
      // level kk (wp, ww) goes to rec[0..1]
      auto dn_level = [&](const float* st, const int q, const int kk, uint32_t* rec) {
        const T wk = S_(st, 0, q), fz = S_(st, 1, q), qvk = S_(st, 2, q), ff = ffilt(kk);
        const T tkm = S_(st, 3, q), pkm = S_(st, 4, q), qskm = S_(st, 5, q), zd_km = S_(st, 6, q);
        const T fkm = S_(st, 7, q), tm = S_(st, 8, q);
        T zrom1w = ((T(0.5) * T(kCpd)) * fz) * (tkm + tk);
        zrom1w = zrom1w - (((((T(kCpd) * wk) * fz) * fz) * ns) * dtrdz) * (tkm - tk);
        zrom1w = zrom1w_moist(zrom1w, qvk, qsk, qskm, wk, fz, pkm, tm, ns1, dts);
        T zwexpl = (wk - (zrom1w * dtrdz) * (pkm - pk)) - egdts;
        zwexpl = zwexpl + ((T(kRdrcv) * zrom1w) * dtrdz) * prod_sub(pkm, zd_km, pk, zd_k);
        const T zu_t = ((zcs2 * fkm) * zrom1w) * pkm + ff;
        const T zd_t = ((zcs2 * fk) * zrom1w) * pk + ff;
        const double zu = widen_normal(zu_t), zdd = widen_normal(zd_t);
        const double tt = fma(zdd, cwp1, 1.0);
        const double den = tt + zu;
        float r;
        asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(narrow_normal(den)));
        const double q0 = widen_normal(narrow_normal(tt) * r);
        const double rem = fma(-den, q0, tt);
        cwp1 = q0 + widen_normal(r * narrow_residual(rem));
        const float wpk = r * (zwexpl + zd_t * wkp1);
        rec[0] = fbits(wpk); rec[1] = fbits(r * zu_t);
        wkp1 = wpk;
        zd_k = zd_km; tk = tkm; pk = pkm; fk = fkm; qsk = qskm;
      };

      // (b) down-sweep k = kz .. 2 (reference order)
      for (int cc = 0; cc < nd; ++cc, ++g) {
        const float* st = wait_full(g);
        if (!st) break;
        const int kk_hi = kz - 1 - cc * KC, kk_lo = kk_hi - (KC - 1);
        if (kk_lo >= 1) {  // a whole chunk: one TMEM store of its 8 words
          uint32_t rec[2 * KC];
#pragma unroll
          for (int u = 0; u < KC; ++u) dn_level(st, KC - 1 - u, kk_hi - u, rec + 2 * (KC - 1 - u));
          tc::tmem_st8p(trow + (uint32_t)(2 * kk_lo), rec);
        } else {
          for (int kk = kk_hi; kk >= 1; --kk) {
            uint32_t rec[2];
            dn_level(st, kk - kk_lo, kk, rec);
            tc::tmem_st2(trow + (uint32_t)(2 * kk), rec[0], rec[1]);
          }
        }
        release(g);
      }
      if (fail) break;
      tc::tmem_wait_st();
      // the next tile's starting values, loaded while this one finishes
      if (t + (int)gridDim.x < ntiles) load_init(t + (int)gridDim.x, nx);

      // (c) back-substitution (:681-686) fused with the Exner/theta update
      // of the level above (:690-728); w(1) = 0 always (init_moloch :260-262).
      // Chunk cc holds levels kk = 4 cc + 1 .. 4 cc + 4; the records of a
      // whole chunk (all kk < kz) are 8 consecutive TMEM columns, loaded one
      // chunk ahead.
      float wlo_d = 0.f;
      T wlo = T(0);
      uint32_t cur[2 * KC], nxt[2 * KC];
      if (nfull > 0) tc::tmem_ld8p(trow + 2u, nxt);
      T* __restrict__ pw = v.w + c;
      T* __restrict__ pdw = v.deltaw + c;
      T* __restrict__ ptet = v.tetav + c;
      T* __restrict__ ppai = v.pai + c;
      T* __restrict__ psv = v.s + c;
      // level kk (record rec when kk < kz) and the update of level kk-1
      auto up_level = [&](const float* st, const int q, const int kk, const uint32_t* rec) {
        const int m = kk - 1;
        T wn;
        if (rec) {
          wlo_d = bitsf(rec[0]) + bitsf(rec[1]) * wlo_d;
          wn = (T)wlo_d;
          if (own) {
            const size_t qq = (size_t)kk * pl;
            tc::st_hint(pdw + qq, (-S_(st, 7, q)) + wn, once);
            tc::st_hint(pw + qq, wn, once);
          }
        } else {
          wn = wsurf;
        }
        const T ffmz = S_(st, 0, q), fqv = S_(st, 1, q), ftet = S_(st, 2, q), fpai = S_(st, 3, q);
        const T fqc = S_(st, 4, q), fqwl = S_(st, 5, q), fqwi = S_(st, 6, q);
        T zd = S_(st, 8, q);
        zd = zd + (dtrdz * ffmz) * (wlo - wn);
        zd = div_corr(zd * ((T(1) + T(0.86) * fqv) + T(3.2) * fqc), (T(1) + T(0.96) * fqv) + T(4.8) * fqc);
        if (own) {
          const size_t qm = (size_t)m * pl;
          tc::st_hint(ptet + qm,
                      ftet * (T(1) + (rdrcv * zd) * (prod_add(T(0.25), fqv, T(4.2), fqwl) + T(2.1) * fqwi)), once);
          if (jj == nj - 1) v.ep_j[ii + (size_t)ni * m] = fpai;
          if (ii == ni - 1) v.ep_i[jj + (size_t)nj * m] = fpai;
          tc::st_hint(ppai + qm, fpai * (T(1) - rdrcv * zd), once);
          if (last) tc::st_hint(psv + qm, m == 0 ? T(0) : (wlo + S_(st, 9, q)) * S_(st, 10, q), once);  // Eq. 10
        }
        wlo = wn;
      };
      for (int cc = 0; cc < nu; ++cc, ++g) {
        const float* st = wait_full(g);
        if (!st) break;
        const int kk0 = cc * KC + 1;
        if (cc < nfull) {
          tc::tmem_wait_ld8p(nxt);
#pragma unroll
          for (int e = 0; e < 2 * KC; ++e) cur[e] = nxt[e];
          if (cc + 1 < nfull) tc::tmem_ld8p(trow + (uint32_t)(2 * (kk0 + KC)), nxt);
#pragma unroll
          for (int u = 0; u < KC; ++u) up_level(st, u, kk0 + u, cur + 2 * u);
        } else {
          for (int kk = kk0; kk <= kz && kk < kk0 + KC; ++kk) {
            if (kk < kz) {
              uint32_t rec[2];
              tc::tmem_ld2(trow + (uint32_t)(2 * kk), rec);
              tc::tmem_wait_ld2(rec);
              up_level(st, kk - kk0, kk, rec);
            } else {
              up_level(st, kk - kk0, kk, nullptr);
            }
          }
        }
        release(g);
      }
      if (fail) break;
      if (last && own) v.s[c + (size_t)kz * pl] = T(0);
    }
    // no TMEM load or store of this thread may be in flight when TMEM is
    // freed (a wait that gave up can leave one of either)
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
    if (lane == 0 && warp == 0) s_consumed = g;  // first job warp 0 did not finish
  }
  tc::tc_fence_before();
  __syncthreads();
  if (tid == 32 * ROWS && s_fail) {
    // a wait gave up: flag it and let the copies still in flight land
    // before the CTA's shared memory is released (bounded)
    atomicExch(kerr, 1);
    for (int q = 0; q < NST; ++q) {
      const int j = s_last_job[q];
      if (j >= s_consumed) tc::mbar_wait_cycles(&full[q], (j / NST) & 1, lim);
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (warp == 0) tc::tmem_dealloc(tbase, 512);
}

template <class T, int LAST, int ROWS>
__global__ void __launch_bounds__(TwCfg<ROWS>::threads, 1)
    k_sound_column_tw(const __grid_constant__ View<T> d, const __grid_constant__ ColumnMaps maps, int nsound) {
  if (d.sur_skip && *d.sur_skip) return;  // the surrogate took this cycle
  column_tw_body<T, LAST, ROWS, false>(&d, &maps, nullptr, 0, 0, nsound, d.kerr, d.spin_cycles, d.fault_skip_job);
}

// An ensemble's column tiles in one persistent launch: the tile table
// lists (member, tile x, tile y) heaviest member first; cms holds each
// member's tensor maps for the 12-row boxes, two buffer-set parities per
// member.  A wait that gives up sets *kerr (the ensemble's error word).
template <class T, int LAST, int ROWS>
__global__ void __launch_bounds__(TwCfg<ROWS>::threads, 1)
    kb_sound_column_tw(const View<T>* __restrict__ views, const ColumnMaps* __restrict__ cms,
                       const int4* __restrict__ tiles, int ntiles, int fcur, int nsound, int* kerr, long long lim) {
  column_tw_body<T, LAST, ROWS, true>(views, cms, tiles, ntiles, fcur, nsound, kerr, lim, -1);
}

}  // namespace MOLOCH_KNS
}  // namespace moloch
