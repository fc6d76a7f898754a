// Momentum update of sound(), Equations 17 and 18 (nompi/mod_moloch.F90:
// 730-837), for FP32 storage: tiles of 32 (j) x 8 (i) columns marching down
// all levels, each level's neighbourhood staged by TMA.
//
// The warp-strip kernel (b_momentum_strip) spends most of its issue slots
// on per-lane cp.async copies, shuffles for the east/west neighbours and the
// 2-D metric fields reloaded on every level; here one thread per column
// takes its metric terms once, and every level's u, v, tetav, pai and
// deltaw arrive as one 40 x 10 TMA box each (the tile with a one-point halo,
// its x origin rounded down to a 16-byte boundary) in a ring of kMtStages
// levels, so a point reads its neighbours from shared memory.
//
// Halo entries a TMA box cannot give -- periodic images across the domain
// edges, and the reference's stale halos (u, v before divdamp, pai before
// its update, kept in the edge buffers) -- are written into the staged
// level by the tile's threads before it is used, in the precedence of
// b_sound_momentum: for v the north row then the west column (the west
// value wins at the corner), for u the south row then the east column.
//
// Waits are bounded by View::spin_cycles SM cycles; a wait that gives up
// sets *View::kerr; the decision is taken CTA-wide, the CTA waits (bounded)
// for its copies in flight and returns.
#pragma once

#include "moloch_tc.cuh"

namespace moloch {
namespace MOLOCH_KNS {

constexpr int kMtRows = 8;                       // rows (i) per tile = warps
constexpr int kMtBoxJ = 40, kMtBoxI = kMtRows + 2;
constexpr int kMtSlotBytes = 1664;               // 40 x 10 x 4 B rounded up to 128 B
constexpr int kMtArrays = 5;                     // u, v, tetav, pai, deltaw
constexpr int kMtStageBytes = kMtArrays * kMtSlotBytes;
constexpr int kMtStages = 4;                     // levels in the ring
constexpr int kMtSmem = kMtStages * kMtStageBytes + 128;
constexpr int kMtThreads = 32 * kMtRows;

// tensor maps: u, v of both buffers of the pair, tetav and pai of both
// advected-field sets, deltaw; a launch takes the five it needs
enum MomMap { MM_U0 = 0, MM_U1, MM_V0, MM_V1, MM_T0, MM_T1, MM_P0, MM_P1, MM_DW, MM_COUNT };
struct MomentumMaps {
  CUtensorMap m[MM_COUNT];
};
struct MomentumSel {
  CUtensorMap u, v, tet, pai, dw;
};

template <class T>
__global__ void __launch_bounds__(kMtThreads, 3) k_momentum_tm(View<T> d, const __grid_constant__ MomentumSel maps) {
  static_assert(sizeof(T) == 4, "FP32 storage only");
  if (d.sur_skip && *d.sur_skip) return;  // the surrogate took this cycle
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full[kMtStages];
  __shared__ int s_issued;
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 127) & ~(uintptr_t)127);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nj = d.nj, ni = d.ni, kz = d.kz;
  const size_t pl = d.pl;
  const int j0 = blockIdx.x * 32, i0 = blockIdx.y * kMtRows;
  const int jj = j0 + lane, ii = i0 + warp;
  const bool own = jj < nj && ii < ni;
  const long long lim = d.spin_cycles;
  // tiles whose halo crosses a domain edge (or whose last column or row is
  // the domain's) take their halo from the edge buffers and periodic images
  const bool w_edge = j0 == 0, s_edge = i0 == 0;
  const bool e_edge = j0 + 32 >= nj, n_edge = i0 + kMtRows >= ni;
  const bool edge = w_edge || s_edge || e_edge || n_edge;
  const int ecol = (e_edge ? nj - j0 : 32) + 4;      // smem column of the east halo used
  const int nrow = (n_edge ? ni - i0 : kMtRows) + 1;  // smem row of the north halo used

  if (tid == 0) {
    for (int q = 0; q < kMtStages; ++q) tc::mbar_init(&full[q], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // level l of the ring (0 .. kz): u, v, tetav, pai of level l (l < kz) and
  // deltaw of level l; x origin j0 - 4 (16-byte aligned), y origin i0 - 1
  auto issue = [&](int l) {
    const int q = l % kMtStages;
    uint8_t* st = smem + q * kMtStageBytes;
    const uint32_t n = l < kz ? 5u : 1u;
    tc::mbar_arrive_expect_tx(&full[q], n * (uint32_t)(kMtBoxJ * kMtBoxI * 4));
    if (l < kz) {
      tc::tma_load_3d(st + 0 * kMtSlotBytes, &maps.u, j0 - 4, i0 - 1, l, &full[q]);
      tc::tma_load_3d(st + 1 * kMtSlotBytes, &maps.v, j0 - 4, i0 - 1, l, &full[q]);
      tc::tma_load_3d(st + 2 * kMtSlotBytes, &maps.tet, j0 - 4, i0 - 1, l, &full[q]);
      tc::tma_load_3d(st + 3 * kMtSlotBytes, &maps.pai, j0 - 4, i0 - 1, l, &full[q]);
    }
    tc::tma_load_3d(st + 4 * kMtSlotBytes, &maps.dw, j0 - 4, i0 - 1, l, &full[q]);
  };
  if (tid == 0) {
    int n = 0;
    for (int l = 0; l < kMtStages && l <= kz; ++l, ++n) issue(l);
    s_issued = n;
  }

  // halo entries of staged level l that TMA could not give (edge tiles)
  auto patch = [&](int l) {
    float* st = reinterpret_cast<float*>(smem + (l % kMtStages) * kMtStageBytes);
    float* U = st;
    float* V = st + 1 * (kMtSlotBytes / 4);
    float* TT = st + 2 * (kMtSlotBytes / 4);
    float* P = st + 3 * (kMtSlotBytes / 4);
    float* DW = st + 4 * (kMtSlotBytes / 4);
    const size_t o = (size_t)l * pl;
    // rows: south row (r = 0), columns c = 0 .. 39 (j = j0 - 4 + c, wrapped)
    if (s_edge) {
      for (int c = tid; c < kMtBoxJ; c += blockDim.x) {
        const int j = wrap2(j0 - 4 + c, nj);
        if (l < kz) {
          U[c] = d.eu_i[j + (size_t)nj * l];
          P[c] = d.ep_i[j + (size_t)nj * l];
          TT[c] = d.tetav[o + j + (size_t)nj * (ni - 1)];
        }
        DW[c] = d.deltaw[o + j + (size_t)nj * (ni - 1)];
      }
    }
    if (n_edge && l < kz)
      for (int c = tid; c < kMtBoxJ; c += blockDim.x) V[nrow * kMtBoxJ + c] = d.ev_i[wrap2(j0 - 4 + c, nj) + (size_t)nj * l];
    __syncthreads();  // corners: the column patches below win
    if (w_edge) {
      for (int r = tid; r < kMtBoxI; r += blockDim.x) {
        const int i = wrap2(i0 - 1 + r, ni);
        if (l < kz) {
          V[r * kMtBoxJ + 3] = d.ev_j[i + (size_t)ni * l];
          P[r * kMtBoxJ + 3] = d.ep_j[i + (size_t)ni * l];
          TT[r * kMtBoxJ + 3] = d.tetav[o + (nj - 1) + (size_t)nj * i];
        }
        DW[r * kMtBoxJ + 3] = d.deltaw[o + (nj - 1) + (size_t)nj * i];
      }
    }
    if (e_edge && l < kz)
      for (int r = tid; r < kMtBoxI; r += blockDim.x) U[r * kMtBoxJ + ecol] = d.eu_j[wrap2(i0 - 1 + r, ni) + (size_t)ni * l];
    // these generic writes precede the TMA that later refills the slot
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  };

  // the column's 2-D terms, once
  const size_t c = own ? (size_t)jj + (size_t)nj * ii : 0;
  const T dts = d.dts, egdts = d.egdts;
  const T hcpd = T(0.5) * T(kCpd);
  const T zcx = d.dtrdx * d.mu[c];
  const T zcy = d.rotllr ? d.dtrdy : d.dtrdy * d.mv[c];
  const T corx = (d.coru[c] * dts) * T(0.25), cory = (d.corv[c] * dts) * T(0.25);
  const T hxc = d.hx[c], hyc = d.hy[c];
  T* __restrict__ uo = d.ubuf[d.cur ^ 1] + c;
  T* __restrict__ vo = d.vbuf[d.cur ^ 1] + c;
  const int sc = (warp + 1) * kMtBoxJ + lane + 4;  // this point in a staged box

  bool ok = true;
  int consumed = 0;  // levels whose copies are known to have landed
  for (int k = 0; k < kz; ++k) {
    const int q0 = k % kMtStages, q1 = (k + 1) % kMtStages;
    bool w = tc::mbar_wait_cycles(&full[q0], (k / kMtStages) & 1, lim) &&
             tc::mbar_wait_cycles(&full[q1], ((k + 1) / kMtStages) & 1, lim);
    ok = __syncthreads_and(w);
    if (!ok) break;
    consumed = k + 2;
    if (edge) {
      if (k == 0) patch(0);
      patch(k + 1);
      __syncthreads();
    }
    const float* s0 = reinterpret_cast<const float*>(smem + q0 * kMtStageBytes);
    const float* s1 = reinterpret_cast<const float*>(smem + q1 * kMtStageBytes);
    const float* U = s0;
    const float* V = s0 + 1 * (kMtSlotBytes / 4);
    const float* TT = s0 + 2 * (kMtSlotBytes / 4);
    const float* P = s0 + 3 * (kMtSlotBytes / 4);
    const float* D0 = s0 + 4 * (kMtSlotBytes / 4);
    const float* D1 = s1 + 4 * (kMtSlotBytes / 4);
    const int sw = sc - 1, ss = sc - kMtBoxJ, sn = sc + kMtBoxJ;
    const T gzh = d.gzitakh[k];
    const T dw_c = D0[sc], dw_c1 = D1[sc];
    const T tc_ = TT[sc], pc = P[sc];
    // Equation 17
    {
      const T zfz = egdts + T(0.25) * (((D0[sw] + D1[sw]) + dw_c) + dw_c1);
      const T zrom1u = hcpd * (TT[sw] + tc_);
      const T zcor1u = corx * (((V[sc] + V[sw]) + V[sn - 1]) + V[sn]);
      const T un = ((U[sc] + zcor1u) - (zfz * hxc) * gzh) - (zcx * zrom1u) * (pc - P[sw]);
      if (own) uo[(size_t)k * pl] = un;
    }
    // Equation 18
    {
      const T zfz = egdts + T(0.25) * (((D0[ss] + D1[ss]) + dw_c) + dw_c1);
      const T zrom1v = hcpd * (TT[ss] + tc_);
      const T zcor1v = cory * (((U[sc] + U[ss]) + U[sc + 1]) + U[ss + 1]);
      const T vn = ((V[sc] - zcor1v) - (zfz * hyc) * gzh) - (zcy * zrom1v) * (pc - P[ss]);
      if (own) vo[(size_t)k * pl] = vn;
    }
    __syncthreads();  // level k's slot is free
    if (tid == 0 && k + kMtStages <= kz) {
      issue(k + kMtStages);
      s_issued = k + kMtStages + 1;
    }
  }
  if (!ok) {
    // a wait gave up: flag it and let the copies still in flight land
    // before the CTA's shared memory is released (bounded)
    if (tid == 0) {
      atomicExch(d.kerr, 1);
      for (int l = consumed; l < s_issued; ++l) tc::mbar_wait_cycles(&full[l % kMtStages], (l / kMtStages) & 1, lim);
    }
  }
}

}  // namespace MOLOCH_KNS
}  // namespace moloch
