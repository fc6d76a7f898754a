// Horizontal divergence, Equation 10 and divdamp of sound() (nompi/
// mod_moloch.F90:514-597, :853-895, :627-630) in one pass, for FP32
// storage: tiles of 32 (j) x 8 (i) columns marching down all levels, each
// level's neighbourhood staged by TMA.  The arithmetic of b_divdamp_strip.
//
// Per level the tile's u, v, rfw, rfs and fmz arrive as 40 x 11 TMA boxes
// (columns j0-4 .. j0+35, rows i0-1 .. i0+9) in a ring of kDtStages levels;
// the divergence zdiv2a of the 34 x 10 points the damping reads (the tile
// and a one-point rim) is formed in shared memory, then every point damps
// u, v into the other buffer of the pair and writes zdiv2b, s(k) and, on the
// lowest level, the surface w and s.  s(k+1) of one level is s(k) of the
// next, carried in a register.  The 2-D metric terms of the box are staged
// once per tile with periodic wrap; in tiles whose box leaves the domain,
// the cells outside it are replaced by their periodic images before use.
// The boundary points store the pre-damping edge values the momentum step
// reads as the stale ud/vd halo (:730-735).
//
// Waits are bounded by View::spin_cycles SM cycles; a wait that gives up
// sets *View::kerr; the decision is taken CTA-wide, the CTA waits (bounded)
// for its copies in flight and returns.
#pragma once

#include "moloch_tc.cuh"

namespace moloch {
namespace MOLOCH_KNS {

constexpr int kDtRows = 8;                       // rows (i) per tile = warps
constexpr int kDtBoxJ = 40, kDtBoxI = kDtRows + 3;
constexpr int kDtBoxElems = kDtBoxJ * kDtBoxI;   // 440
constexpr int kDtSlotBytes = 1792;               // 440 x 4 B rounded up to 128 B
constexpr int kDtArrays = 5;                     // u, v, rfw, rfs, fmz
constexpr int kDtStageBytes = kDtArrays * kDtSlotBytes;
constexpr int kDtStages = 4;                     // levels in the ring
constexpr int kDtZJ = 34, kDtZI = kDtRows + 2;   // zdiv2a region: columns j0-1 .. j0+32, rows i0-1 .. i0+8
constexpr int kDtSmem = kDtStages * kDtStageBytes + 128;
constexpr int kDtThreads = 32 * kDtRows;

enum DivMap { DM_U0 = 0, DM_U1, DM_V0, DM_V1, DM_RFW, DM_RFS, DM_FMZ, DM_COUNT };
struct DivdampMaps {
  CUtensorMap m[DM_COUNT];
};
struct DivdampSel {
  CUtensorMap u, v, rfw, rfs, fmz;
};

template <class T>
__global__ void __launch_bounds__(kDtThreads, 3) k_divdamp_tm(View<T> d, const __grid_constant__ DivdampSel maps) {
  static_assert(sizeof(T) == 4, "FP32 storage only");
  if (d.sur_skip && *d.sur_skip) return;  // the surrogate took this cycle
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full[kDtStages];
  __shared__ int s_issued;
  __shared__ float zs_[kDtZI * kDtZJ];
  // 2-D terms of the box, periodic: hx, hy, mx (mx2 without rotation), rmu, rmv
  __shared__ float m2[5][kDtBoxElems];
  uint8_t* smem = (uint8_t*)(((uintptr_t)smem_raw + 127) & ~(uintptr_t)127);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nj = d.nj, ni = d.ni, kz = d.kz;
  const size_t pl = d.pl;
  const int j0 = blockIdx.x * 32, i0 = blockIdx.y * kDtRows;
  const int jj = j0 + lane, ii = i0 + warp;
  const bool own = jj < nj && ii < ni;
  const long long lim = d.spin_cycles;
  const bool rot = d.rotllr;
  // the box leaves the domain somewhere: cells outside take periodic images
  const bool edge = j0 - 4 < 0 || j0 + 35 >= nj || i0 - 1 < 0 || i0 + kDtRows + 1 >= ni;

  if (tid == 0) {
    for (int q = 0; q < kDtStages; ++q) tc::mbar_init(&full[q], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int e = tid; e < kDtBoxElems; e += blockDim.x) {
    const int r = e / kDtBoxJ, cc = e - r * kDtBoxJ;
    const size_t q = (size_t)wrap2(j0 - 4 + cc, nj) + (size_t)nj * wrap2(i0 - 1 + r, ni);
    m2[0][e] = d.hx[q];
    m2[1][e] = d.hy[q];
    m2[2][e] = rot ? d.mx[q] : d.mx2[q];
    m2[3][e] = rot ? T(0) : d.rmu[q];
    m2[4][e] = d.rmv[q];
  }
  __syncthreads();
  auto issue = [&](int l) {
    const int q = l % kDtStages;
    uint8_t* st = smem + q * kDtStageBytes;
    tc::mbar_arrive_expect_tx(&full[q], 5u * (uint32_t)(kDtBoxElems * 4));
    tc::tma_load_3d(st + 0 * kDtSlotBytes, &maps.u, j0 - 4, i0 - 1, l, &full[q]);
    tc::tma_load_3d(st + 1 * kDtSlotBytes, &maps.v, j0 - 4, i0 - 1, l, &full[q]);
    tc::tma_load_3d(st + 2 * kDtSlotBytes, &maps.rfw, j0 - 4, i0 - 1, l, &full[q]);
    tc::tma_load_3d(st + 3 * kDtSlotBytes, &maps.rfs, j0 - 4, i0 - 1, l, &full[q]);
    tc::tma_load_3d(st + 4 * kDtSlotBytes, &maps.fmz, j0 - 4, i0 - 1, l, &full[q]);
  };
  if (tid == 0) {
    int n = 0;
    for (int l = 0; l < kDtStages && l < kz; ++l, ++n) issue(l);
    s_issued = n;
  }
  // cells of staged level l outside the domain: periodic images (edge tiles)
  auto patch = [&](int l) {
    float* st = reinterpret_cast<float*>(smem + (l % kDtStages) * kDtStageBytes);
    const size_t o = (size_t)l * pl;
    const T* src[5] = {d.ubuf[d.cur] + o, d.vbuf[d.cur] + o, d.rfw + o, d.rfs + o, d.fmz + o};
    for (int e = tid; e < kDtBoxElems; e += blockDim.x) {
      const int r = e / kDtBoxJ, cc = e - r * kDtBoxJ;
      const int gj = j0 - 4 + cc, gi = i0 - 1 + r;
      if (gj >= 0 && gj < nj && gi >= 0 && gi < ni) continue;
      const size_t q = (size_t)wrap2(gj, nj) + (size_t)nj * wrap2(gi, ni);
#pragma unroll
      for (int a = 0; a < 5; ++a) st[a * (kDtSlotBytes / 4) + e] = src[a][q];
    }
    // these generic writes precede the TMA that later refills the slot
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  };

  const size_t c = own ? (size_t)jj + (size_t)nj * ii : 0;
  const T dtrdx = d.dtrdx, dtrdy = d.dtrdy, dtrdz = d.dtrdz, ddamp2 = d.ddamp2;
  const T muc = d.mu[c];
  const T mvc = rot ? T(0) : d.mv[c];
  T* __restrict__ uo = d.ubuf[d.cur ^ 1] + c;
  T* __restrict__ vo = d.vbuf[d.cur ^ 1] + c;
  const int sc = (warp + 1) * kDtBoxJ + lane + 4;  // this point in a staged box
  const T hx0 = m2[0][sc], hx1 = m2[0][sc + 1], hy0 = m2[1][sc], hy1 = m2[1][sc + kDtBoxJ];
  T s_k = d.s[c];  // s at the top level is never computed here

  bool ok = true;
  int consumed = 0;
  for (int k = 0; k < kz; ++k) {
    const bool has_dn = k < kz - 1;  // level k+1 exists
    const int q0 = k % kDtStages, q1 = (k + 1) % kDtStages;
    bool w = tc::mbar_wait_cycles(&full[q0], (k / kDtStages) & 1, lim) &&
             (!has_dn || tc::mbar_wait_cycles(&full[q1], ((k + 1) / kDtStages) & 1, lim));
    ok = __syncthreads_and(w);
    if (!ok) break;
    consumed = has_dn ? k + 2 : k + 1;
    if (edge) {
      if (k == 0) patch(0);
      if (has_dn) patch(k + 1);
      __syncthreads();
    }
    const float* s0 = reinterpret_cast<const float*>(smem + q0 * kDtStageBytes);
    const float* U = s0;
    const float* V = s0 + 1 * (kDtSlotBytes / 4);
    const float* RFW = s0 + 2 * (kDtSlotBytes / 4);
    const float* RFS = s0 + 3 * (kDtSlotBytes / 4);
    const float* FMZ = s0 + 4 * (kDtSlotBytes / 4);
    // zdiv2a (Equation 16) on the tile and its rim
    for (int e = tid; e < kDtZI * kDtZJ; e += blockDim.x) {
      const int zr = e / kDtZJ, zc = e - zr * kDtZJ;
      const int b = zr * kDtBoxJ + zc + 3;  // the point (j0 - 1 + zc, i0 - 1 + zr) in a box
      const T uk = U[b], uk_e = U[b + 1], vk = V[b], vn = V[b + kDtBoxJ];
      T z;
      if (rot) {
        const T zum = (dtrdx * uk) * RFW[b];
        const T zup = (dtrdx * uk_e) * RFW[b + 1];
        const T zvm = ((dtrdy * vk) * RFS[b]) * m2[4][b];
        const T zvp = ((dtrdy * vn) * RFS[b + kDtBoxJ]) * m2[4][b + kDtBoxJ];
        z = (FMZ[b] * m2[2][b]) * ((zup - zum) + (zvp - zvm));
      } else {
        const T zum = ((dtrdx * uk) * m2[3][b]) * RFW[b];
        const T zup = ((dtrdx * uk_e) * m2[3][b + 1]) * RFW[b + 1];
        const T zvm = ((dtrdy * vk) * m2[4][b]) * RFS[b];
        const T zvp = ((dtrdy * vn) * m2[4][b + kDtBoxJ]) * RFS[b + kDtBoxJ];
        z = (m2[2][b] * FMZ[b]) * ((zup - zum) + (zvp - zvm));
      }
      zs_[e] = z;
    }
    __syncthreads();
    // s(k+1) (Equation 10), or the surface w and s on the lowest level
    const T u0 = U[sc], v0 = V[sc], ue = U[sc + 1], vn = V[sc + kDtBoxJ];
    T s_k1, ws = T(0);
    if (has_dn) {
      const float* s1 = reinterpret_cast<const float*>(smem + q1 * kDtStageBytes);
      const T up = s1[sc], up_e = s1[sc + 1];
      const T vp = s1[(kDtSlotBytes / 4) + sc], vp_n = s1[(kDtSlotBytes / 4) + sc + kDtBoxJ];
      const T zuh = (up + u0) * hx0 + (up_e + ue) * hx1;
      const T zvh = (vp + v0) * hy0 + (vp_n + vn) * hy1;
      s_k1 = -((T(0.25) * (zuh + zvh)) * d.gzitak[k + 1]);
    } else {
      const T zuh = u0 * hx0 + ue * hx1;
      const T zvh = v0 * hy0 + vn * hy1;
      ws = T(0.5) * (zuh + zvh);
      s_k1 = -ws;
    }
    if (own) {
      const int zp = (warp + 1) * kDtZJ + lane + 1;  // this point in the zdiv2a region
      const T zc = zs_[zp], zw = zs_[zp - 1], ze = zs_[zp + 1], zsv = zs_[zp - kDtZJ], zn = zs_[zp + kDtZJ];
      const size_t o = (size_t)k * pl;
      if (k > 0) d.s[o + c] = s_k;
      if (!has_dn) {
        d.w[c + (size_t)kz * pl] = ws;
        d.s[c + (size_t)kz * pl] = -ws;
      }
      if (jj == 0) d.eu_j[ii + (size_t)ni * k] = u0;
      if (ii == ni - 1) d.eu_i[jj + (size_t)nj * k] = u0;
      if (jj == nj - 1) d.ev_j[ii + (size_t)ni * k] = v0;
      if (ii == 0) d.ev_i[jj + (size_t)nj * k] = v0;
      const T cd = d.cdamp[k];
      uo[o] = u0 + ((cd * muc) * (zc - zw));
      if (rot)
        vo[o] = v0 + cd * (zc - zsv);
      else
        vo[o] = v0 + ((cd * mvc) * (zc - zsv));
      const T p2d = T(0.125) * (((zw + ze) + zsv) + zn) - T(0.5) * zc;
      T zd = zc + ddamp2 * p2d;
      zd = zd + (FMZ[sc] * dtrdz) * (s_k - s_k1);
      d.zdiv2b[o + c] = zd;
    }
    s_k = s_k1;
    __syncthreads();  // level k's slot and the zdiv2a region are free
    if (tid == 0 && k + kDtStages < kz) {
      issue(k + kDtStages);
      s_issued = k + kDtStages + 1;
    }
  }
  if (!ok && tid == 0) {
    // a wait gave up: flag it and let the copies still in flight land
    // before the CTA's shared memory is released (bounded)
    atomicExch(d.kerr, 1);
    for (int l = consumed; l < s_issued; ++l) tc::mbar_wait_cycles(&full[l % kDtStages], (l / kDtStages) & 1, lim);
  }
}

}  // namespace MOLOCH_KNS
}  // namespace moloch
