// MOLOCH step kernels for sm_103a.  Included by one .cu file per arithmetic
// build (MOLOCH_KNS names the namespace): the exact FP64 build is compiled
// with --fmad=false so every expression keeps the reference's evaluation
// order; the fast build allows multiply-add contraction and also carries the
// FP32-storage instantiation.
//
// Kernel map (reference: nompi/mod_moloch.F90):
//   k_prediag          :289-323  p, qsat, tvirt, qwltot, qwitot, tetav
//   k_sound_div        :514-597  u/v halo + surface w + s (Eq. 10) + zdiv2 (Eq. 16)
//   k_sound_column     :853-895 + :627-728  divdamp, vertical s term, implicit w
//                      (Thomas, one thread per column), Exner/theta update,
//                      nompi pai halo order, s completion (:843-849)
//   k_lap_filter       :423-440 divergence_filter (mo_divfilter)
//   k_pai_update       :716-728 (split form used when the filter is on)
//   k_sound_momentum   :730-837  Equations 17, 18
//   k_stag_to_x        :1327-1341, :1389-1417  (u,v,w) -> (ux,vx,wx)
//   k_waf_vertical     :966-1073  two vertical WAF passes, all 10 fields
//   k_waf_meridional   :1075-1136 meridional WAF flux + update -> p0
//   k_waf_zonal        :1138-1187 zonal WAF flux + update -> pp
//   k_stag_from_x      :1343-1387  (ux,vx,wx) -> (u,v,w)
//   k_filter_increment :442-481 + :333-353 filtpai / filttheta
//   k_postdiag         :355-391  tvirt, t, p, rho, ps, qsat
//   k_diag_*           :395-411  max/min of ps, u, v; NaN/Inf check; FP64 column sums
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#include "moloch_constants.h"
#include "moloch_view.h"

#ifndef MOLOCH_KNS
#error "MOLOCH_KNS must name the namespace of this kernel build"
#endif

namespace moloch {
namespace MOLOCH_KNS {

constexpr int kColBX = 32;  // column kernels: 32 j x 4 i threads
constexpr int kColBY = 4;
constexpr int kPtBX = 32;   // point kernels: 32 j x 8 i threads
constexpr int kPtBY = 8;
constexpr int kTileBI = 8;  // WAF tile rows

template <class T>
struct FieldPtrs {
  T* f[kNumAdvected];
};

// ---- small device helpers ---------------------------------------------
__device__ __forceinline__ int wm1(int x, int n) { return x == 0 ? n - 1 : x - 1; }
__device__ __forceinline__ int wp1(int x, int n) { return x == n - 1 ? 0 : x + 1; }
__device__ __forceinline__ int wm2(int x, int n) { int y = x - 2; return y < 0 ? y + n : y; }
__device__ __forceinline__ int wp2(int x, int n) { int y = x + 2; return y >= n ? y - n : y; }
__device__ __forceinline__ int wrapn(int x, int n) { int y = x % n; return y < 0 ? y + n : y; }

__device__ __forceinline__ double dpow(double a, double b) { return pow(a, b); }
__device__ __forceinline__ float dpow(float a, float b) { return powf(a, b); }
__device__ __forceinline__ double dexp(double a) { return exp(a); }
__device__ __forceinline__ float dexp(float a) { return expf(a); }
__device__ __forceinline__ double dabs(double a) { return fabs(a); }
__device__ __forceinline__ float dabs(float a) { return fabsf(a); }
__device__ __forceinline__ double dcopysign(double a, double b) { return copysign(a, b); }
__device__ __forceinline__ float dcopysign(float a, float b) { return copysignf(a, b); }

// Fortran MAX/MIN of two values as the algorithm uses them
template <class T> __device__ __forceinline__ T fmax2(T a, T b) { return a > b ? a : b; }
template <class T> __device__ __forceinline__ T fmin2(T a, T b) { return a < b ? a : b; }
// superbee limiter b = max(0, min(2, max(r, min(2r, 1))))   (:994)
template <class T> __device__ __forceinline__ T superbee(T r) {
  return fmax2(T(0), fmin2(T(2), fmax2(r, fmin2(T(2) * r, T(1)))));
}
// sign(max(abs(z), minden), z)   (:992)
template <class T> __device__ __forceinline__ T safeden(T z) {
  return dcopysign(fmax2(dabs(z), T(kMinden)), z);
}

// pfesat / pfwsat (:119-181)
template <class T>
__device__ __forceinline__ T pfwsat(T t, T p) {
  T tl = t - T(kTzero);
  if (tl > T(100)) tl = T(100);
  if (tl < T(-75)) tl = T(-75);
  T td = tl, esat;
  if (td >= T(0)) {
    esat = T(kEsA0) + td * (T(kEsA1) + td * (T(kEsA2) + td * (T(kEsA3) + td * (T(kEsA4) +
           td * (T(kEsA5) + td * (T(kEsA6) + td * (T(kEsA7) + td * T(kEsA8))))))));
  } else {
    esat = T(kEsC0) + td * (T(kEsC1) + td * (T(kEsC2) + td * (T(kEsC3) + td * (T(kEsC4) +
           td * (T(kEsC5) + td * (T(kEsC6) + td * (T(kEsC7) + td * T(kEsC8))))))));
  }
  T lim = T(0.15) * p;
  T es = esat < lim ? esat : lim;
  return T(kEp2) * (es / (p - es));
}

// ---- pre-diagnostics (:289-323) ----------------------------------------
template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY) k_prediag(View<T> d, int filterpai, int filtertheta) {
  int jj = blockIdx.x * kPtBX + threadIdx.x;
  int ii = blockIdx.y * kPtBY + threadIdx.y;
  if (jj >= d.nj || ii >= d.ni) return;
  size_t c = (size_t)jj + (size_t)d.nj * ii + (size_t)blockIdx.z * d.pl;
  T pai = d.pai[c], t = d.t[c];
  T qv = d.q[0][c], qc = d.q[1][c], qi = d.q[2][c], qr = d.q[3][c], qs = d.q[4][c];
  T p = dpow(pai, T(kCpovr)) * T(kP00);
  d.p[c] = p;
  d.qsat[c] = pfwsat(t, p);
  T tv = t * ((((T(1) + T(kEp1) * qv) - qc) - qi) - qr - qs);
  d.tvirt[c] = tv;
  d.qwltot[c] = qc + qr;
  d.qwitot[c] = qi + qs;
  T tet = tv / pai;
  d.tetav[c] = tet;
  if (filterpai) d.pf[c] = pai;
  if (filtertheta) d.tf[c] = tet;
}

// ---- sound: halo, surface w, s (Eq. 10), horizontal divergence (Eq. 16) ---
// One thread per column.  Writes the pre-divdamp u/v edge values that the
// momentum step later reads as the stale ud/vd halo ring (:730-735).
template <class T>
__global__ void __launch_bounds__(kColBX* kColBY) k_sound_div(View<T> d) {
  int jj = blockIdx.x * kColBX + threadIdx.x;
  int ii = blockIdx.y * kColBY + threadIdx.y;
  const int nj = d.nj, ni = d.ni, kz = d.kz, pl = d.pl;
  if (jj >= nj || ii >= ni) return;
  const int jp = wp1(jj, nj), ip = wp1(ii, ni);
  const T* __restrict__ u = d.ubuf[d.cur];
  const T* __restrict__ v = d.vbuf[d.cur];
  const size_t c = (size_t)jj + (size_t)nj * ii;
  const size_t ce = (size_t)jp + (size_t)nj * ii;  // (j+1, i)
  const size_t cn = (size_t)jj + (size_t)nj * ip;  // (j, i+1)
  const T hx0 = d.hx[c], hx1 = d.hx[ce], hy0 = d.hy[c], hy1 = d.hy[cn];
  const T mxv = d.rotllr ? d.mx[c] : d.mx2[c];
  const T rmv0 = d.rmv[c], rmv1 = d.rmv[cn];
  const T rmu0 = d.rmu[c], rmu1 = d.rmu[ce];
  const T dtrdx = d.dtrdx, dtrdy = d.dtrdy;
  T u0p = T(0), u1p = T(0), v0p = T(0), v1p = T(0);
  for (int kk = 0; kk < kz; ++kk) {
    const size_t o = (size_t)kk * pl;
    const T u0 = u[c + o], u1 = u[ce + o], v0 = v[c + o], v1 = v[cn + o];
    if (kk > 0) {  // s(k), k = 2..kz  (:557-570)
      T zuh = (u0 + u0p) * hx0 + (u1 + u1p) * hx1;
      T zvh = (v0 + v0p) * hy0 + (v1 + v1p) * hy1;
      d.s[c + o] = -((T(0.25) * (zuh + zvh)) * d.gzitak[kk]);
    }
    const T f = d.fmz[c + o];
    const T zrfmzum = d.rfw[c + o], zrfmzup = d.rfw[ce + o];
    const T zrfmzvm = d.rfs[c + o], zrfmzvp = d.rfs[cn + o];
    T zum, zup, zvm, zvp;
    if (d.rotllr) {
      zum = (dtrdx * u0) * zrfmzum;
      zup = (dtrdx * u1) * zrfmzup;
      zvm = ((dtrdy * v0) * zrfmzvm) * rmv0;
      zvp = ((dtrdy * v1) * zrfmzvp) * rmv1;
      d.zdiv2a[c + o] = (f * mxv) * ((zup - zum) + (zvp - zvm));
    } else {
      zum = ((dtrdx * u0) * rmu0) * zrfmzum;
      zup = ((dtrdx * u1) * rmu1) * zrfmzup;
      zvm = ((dtrdy * v0) * rmv0) * zrfmzvm;
      zvp = ((dtrdy * v1) * rmv1) * zrfmzvp;
      d.zdiv2a[c + o] = (mxv * f) * ((zup - zum) + (zvp - zvm));
    }
    // stale-halo edges (values before divdamp)
    if (jj == 0) d.eu_j[ii + (size_t)ni * kk] = u0;
    if (ii == ni - 1) d.eu_i[jj + (size_t)nj * kk] = u0;
    if (jj == nj - 1) d.ev_j[ii + (size_t)ni * kk] = v0;
    if (ii == 0) d.ev_i[jj + (size_t)nj * kk] = v0;
    u0p = u0; u1p = u1; v0p = v0; v1p = v1;
  }
  // surface w(kz+1), s(kz+1)  (:536-549); u0p.. hold level kz
  T zuh = u0p * hx0 + u1p * hx1;
  T zvh = v0p * hy0 + v1p * hy1;
  T ws = T(0.5) * (zuh + zvh);
  d.w[c + (size_t)kz * pl] = ws;
  d.s[c + (size_t)kz * pl] = -ws;
}

// ---- sound: divdamp + implicit w + Exner/theta (one thread per column) ----
// defer_pai: store the final divergence in zdiv2b and leave pai to
// k_pai_update (used when the divergence filter runs in between).
template <class T>
__global__ void __launch_bounds__(kColBX* kColBY)
    k_sound_column(View<T> d, int nsound, int last, int defer_pai) {
  int jj = blockIdx.x * kColBX + threadIdx.x;
  int ii = blockIdx.y * kColBY + threadIdx.y;
  const int nj = d.nj, ni = d.ni, kz = d.kz, pl = d.pl;
  if (jj >= nj || ii >= ni) return;
  const int jm = wm1(jj, nj), jp = wp1(jj, nj), im = wm1(ii, ni), ip = wp1(ii, ni);
  T* __restrict__ u = d.ubuf[d.cur];
  T* __restrict__ v = d.vbuf[d.cur];
  const size_t c = (size_t)jj + (size_t)nj * ii;
  const size_t cw = (size_t)jm + (size_t)nj * ii, ce = (size_t)jp + (size_t)nj * ii;
  const size_t cs = (size_t)jj + (size_t)nj * im, cn = (size_t)jj + (size_t)nj * ip;
  const T mu = d.mu[c], mv = d.mv[c];
  const T ddamp2 = d.ddamp2, dtrdz = d.dtrdz;

  // (a) divdamp (:853-895) and the vertical s contribution (:627-630)
  for (int kk = 0; kk < kz; ++kk) {
    const size_t o = (size_t)kk * pl;
    const T zc = d.zdiv2a[c + o], zw = d.zdiv2a[cw + o], ze = d.zdiv2a[ce + o];
    const T zs = d.zdiv2a[cs + o], zn = d.zdiv2a[cn + o];
    const T cd = d.cdamp[kk];
    u[c + o] = u[c + o] + ((cd * mu) * (zc - zw));
    if (d.rotllr)
      v[c + o] = v[c + o] + cd * (zc - zs);
    else
      v[c + o] = v[c + o] + ((cd * mv) * (zc - zs));
    T p2d = T(0.125) * (((zw + ze) + zs) + zn) - T(0.5) * zc;
    T zd = zc + ddamp2 * p2d;
    zd = zd + (d.fmz[c + o] * dtrdz) * (d.s[c + o] - d.s[c + o + pl]);
    d.zdiv2b[c + o] = zd;
  }

  // (b) Thomas down-sweep, k = kz .. 2  (:634-678); pivots in FP64
  const T ns = T(nsound), ns1 = T(nsound - 1);
  const T zcs2 = d.zcs2, dts = d.dts, egdts = d.egdts;
  double wkp1 = (double)d.w[c + (size_t)kz * pl];  // w(kz+1) from k_sound_div
  const T wsurf = d.w[c + (size_t)kz * pl];
  double wwp1 = 0.0;                                // wwkw(kz+1) = 0
  T zd_k = d.zdiv2b[c + (size_t)(kz - 1) * pl];
  T tk = d.tetav[c + (size_t)(kz - 1) * pl];
  T pk = d.pai[c + (size_t)(kz - 1) * pl];
  T fk = d.fmz[c + (size_t)(kz - 1) * pl];
  T qsk = d.qsat[c + (size_t)(kz - 1) * pl];
  for (int kk = kz - 1; kk >= 1; --kk) {
    const size_t o = (size_t)kk * pl, om = (size_t)(kk - 1) * pl;
    const T wk = d.w[c + o];
    const T fz = d.fmzf[c + o];
    const T tkm = d.tetav[c + om];
    T zrom1w = ((T(0.5) * T(kCpd)) * fz) * (tkm + tk);
    zrom1w = zrom1w - (((((T(kCpd) * wk) * fz) * fz) * ns) * dtrdz) * (tkm - tk);
    const T pkm = d.pai[c + om];
    const T qskm = d.qsat[c + om];
    if (d.q[0][c + o] > T(0.96) * qsk && wk > T(0.1)) {
      T zqs = T(0.5) * (qsk + qskm);
      T tm = d.t[c + om];
      T zdth = ((((((T(kEgrav) * wk) * ns1) * dts) * T(kWlhv)) * T(kWlhv)) * zqs) /
               ((((T(kCpd) * pkm) * T(kRwat)) * tm) * tm);
      zrom1w = zrom1w + zdth * fz;
    }
    const T zd_km = d.zdiv2b[c + om];
    T zwexpl = (wk - (zrom1w * dtrdz) * (pkm - pk)) - egdts;
    zwexpl = zwexpl + ((T(kRdrcv) * zrom1w) * dtrdz) * (pkm * zd_km - pk * zd_k);
    const T fkm = d.fmz[c + om];
    const T ff = d.ffilt[kk];
    const double zu = (double)(((zcs2 * fkm) * zrom1w) * pkm + ff);
    const double zdd = (double)(((zcs2 * fk) * zrom1w) * pk + ff);
    const double zrapp = 1.0 / (((1.0 + zdd) + zu) - zdd * wwp1);
    const double wpk = zrapp * ((double)zwexpl + zdd * wkp1);
    const double wwk = zrapp * zu;
    d.wp[c + o] = wpk;
    d.wwkw[c + o] = wwk;
    wkp1 = wpk; wwp1 = wwk;
    zd_k = zd_km; tk = tkm; pk = pkm; fk = fkm; qsk = qskm;
  }

  // (c) back-substitution (:681-686) fused with the Exner/theta update of
  // the level above (:690-728); w(1) = 0 always (init_moloch :260-262)
  const T rdrcv = T(kRdrcv);
  T wlo = T(0);  // w(k-1) at the time level k is solved
  auto finalize = [&](int kk, T wl, T wh) {
    const size_t o = (size_t)kk * pl;
    T zd = d.zdiv2b[c + o];
    zd = zd + (dtrdz * d.fmz[c + o]) * (wl - wh);
    const T qv = d.q[0][c + o], qc = d.q[1][c + o];
    zd = (zd * ((T(1) + T(0.86) * qv) + T(3.2) * qc)) / ((T(1) + T(0.96) * qv) + T(4.8) * qc);
    d.tetav[c + o] =
        d.tetav[c + o] * (T(1) + (rdrcv * zd) * ((T(0.25) * qv + T(4.2) * d.qwltot[c + o]) +
                                                 T(2.1) * d.qwitot[c + o]));
    if (defer_pai) {
      d.zdiv2b[c + o] = zd;
    } else {
      const T pold = d.pai[c + o];
      if (jj == nj - 1) d.ep_j[ii + (size_t)ni * kk] = pold;
      if (ii == ni - 1) d.ep_i[jj + (size_t)nj * kk] = pold;
      d.pai[c + o] = pold * (T(1) - rdrcv * zd);
    }
    if (last) {  // complete Equation 10 (:843-849)
      if (kk == 0)
        d.s[c + o] = T(0);
      else
        d.s[c + o] = (wl + d.s[c + o]) * d.fmzf[c + o];
    }
  };
  for (int kk = 1; kk < kz; ++kk) {
    const size_t o = (size_t)kk * pl;
    const double wn_d = d.wp[c + o] + d.wwkw[c + o] * (double)wlo;
    const T wn = (T)wn_d;
    const T wold = d.w[c + o];
    d.deltaw[c + o] = (-wold) + wn;
    d.w[c + o] = wn;
    finalize(kk - 1, wlo, wn);
    wlo = wn;
  }
  finalize(kz - 1, wlo, wsurf);
  if (last) d.s[c + (size_t)kz * pl] = T(0);
}

// ---- 5-point Laplacian filter of one field, out of place ----------------
// out = a + coef(k) * (0.125*(aW+aE+aS+aN) - 0.5*a)   (:423-481)
// coef(k) = anu2 * xknu(k) when use_xknu, else the constant c0.
template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY)
    k_lap_filter(View<T> d, const T* __restrict__ a, T* __restrict__ out, int use_xknu, T c0) {
  int jj = blockIdx.x * kPtBX + threadIdx.x;
  int ii = blockIdx.y * kPtBY + threadIdx.y;
  const int nj = d.nj, ni = d.ni;
  if (jj >= nj || ii >= ni) return;
  const size_t o = (size_t)blockIdx.z * d.pl;
  const size_t c = jj + (size_t)nj * ii;
  T aw = a[o + wm1(jj, nj) + (size_t)nj * ii], ae = a[o + wp1(jj, nj) + (size_t)nj * ii];
  T as = a[o + jj + (size_t)nj * wm1(ii, ni)], an = a[o + jj + (size_t)nj * wp1(ii, ni)];
  T ac = a[o + c];
  T p2d = T(0.125) * (((aw + ae) + as) + an) - T(0.5) * ac;
  T coef = use_xknu ? d.anu2 * d.xknu[blockIdx.z] : c0;
  out[o + c] = ac + coef * p2d;
}

// pai update with the nompi halo order (:716-728), split form
template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY) k_pai_update(View<T> d, const T* __restrict__ zd) {
  int jj = blockIdx.x * kPtBX + threadIdx.x;
  int ii = blockIdx.y * kPtBY + threadIdx.y;
  const int nj = d.nj, ni = d.ni, kk = blockIdx.z;
  if (jj >= nj || ii >= ni) return;
  const size_t c = jj + (size_t)nj * ii + (size_t)kk * d.pl;
  const T pold = d.pai[c];
  if (jj == nj - 1) d.ep_j[ii + (size_t)ni * kk] = pold;
  if (ii == ni - 1) d.ep_i[jj + (size_t)nj * kk] = pold;
  d.pai[c] = pold * (T(1) - T(kRdrcv) * zd[c]);
}

// filtpai / filttheta on the step increment (:333-353, :442-481):
// x = a - ref; a = ((x + nupaitq * lap(x)) + ref), written to out
template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY)
    k_filter_increment(View<T> d, const T* __restrict__ a, const T* __restrict__ ref, T* __restrict__ out) {
  int jj = blockIdx.x * kPtBX + threadIdx.x;
  int ii = blockIdx.y * kPtBY + threadIdx.y;
  const int nj = d.nj, ni = d.ni;
  if (jj >= nj || ii >= ni) return;
  const size_t o = (size_t)blockIdx.z * d.pl;
  auto X = [&](int j, int i) {
    size_t q = o + j + (size_t)nj * i;
    return a[q] - ref[q];
  };
  T xw = X(wm1(jj, nj), ii), xe = X(wp1(jj, nj), ii), xs = X(jj, wm1(ii, ni)), xn = X(jj, wp1(ii, ni));
  T xc = X(jj, ii);
  T p2d = T(0.125) * (((xw + xe) + xs) + xn) - T(0.5) * xc;
  const size_t c = o + jj + (size_t)nj * ii;
  out[c] = (xc + T(kNupaitq) * p2d) + ref[c];
}

// ---- sound: momentum, Equations 17 and 18 (:737-837) --------------------
template <class T>
__global__ void __launch_bounds__(kColBX* kColBY) k_sound_momentum(View<T> d) {
  int jj = blockIdx.x * kColBX + threadIdx.x;
  int ii = blockIdx.y * kColBY + threadIdx.y;
  const int nj = d.nj, ni = d.ni, kz = d.kz, pl = d.pl;
  if (jj >= nj || ii >= ni) return;
  const int jm = wm1(jj, nj), jp = wp1(jj, nj), im = wm1(ii, ni), ip = wp1(ii, ni);
  const T* __restrict__ u = d.ubuf[d.cur];
  const T* __restrict__ v = d.vbuf[d.cur];
  T* __restrict__ uo = d.ubuf[d.cur ^ 1];
  T* __restrict__ vo = d.vbuf[d.cur ^ 1];
  const size_t c = (size_t)jj + (size_t)nj * ii;
  const size_t cw = (size_t)jm + (size_t)nj * ii, ce = (size_t)jp + (size_t)nj * ii;
  const size_t cs = (size_t)jj + (size_t)nj * im, cn = (size_t)jj + (size_t)nj * ip;
  const size_t cwn = (size_t)jm + (size_t)nj * ip, ces = (size_t)jp + (size_t)nj * im;
  const T dts = d.dts, egdts = d.egdts;
  const T zcx = d.dtrdx * d.mu[c];
  const T zcy = d.rotllr ? d.dtrdy : d.dtrdy * d.mv[c];
  const T hx = d.hx[c], hy = d.hy[c];
  const T cu = (d.coru[c] * dts) * T(0.25);
  const T cv = (d.corv[c] * dts) * T(0.25);
  const T hcpd = T(0.5) * T(kCpd);
  T dw_c = d.deltaw[c], dw_w = d.deltaw[cw], dw_s = d.deltaw[cs];  // level k
  for (int kk = 0; kk < kz; ++kk) {
    const size_t o = (size_t)kk * pl, o1 = (size_t)(kk + 1) * pl;
    const T dw_c1 = d.deltaw[c + o1], dw_w1 = d.deltaw[cw + o1], dw_s1 = d.deltaw[cs + o1];
    const T tc = d.tetav[c + o];
    const T pc = d.pai[c + o];
    const T gzh = d.gzitakh[kk];
    // Equation 17
    {
      T zfz = egdts + T(0.25) * (((dw_w + dw_w1) + dw_c) + dw_c1);
      T zrom1u = hcpd * (d.tetav[cw + o] + tc);
      T vdc = v[c + o];
      T vdw = jj == 0 ? d.ev_j[ii + (size_t)ni * kk] : v[cw + o];
      T vdwn = jj == 0 ? d.ev_j[ip + (size_t)ni * kk]
                       : (ii == ni - 1 ? d.ev_i[jm + (size_t)nj * kk] : v[cwn + o]);
      T vdn = ii == ni - 1 ? d.ev_i[jj + (size_t)nj * kk] : v[cn + o];
      T zcor1u = cu * (((vdc + vdw) + vdwn) + vdn);
      T paw = jj == 0 ? d.ep_j[ii + (size_t)ni * kk] : d.pai[cw + o];
      uo[c + o] = ((u[c + o] + zcor1u) - (zfz * hx) * gzh) - (zcx * zrom1u) * (pc - paw);
    }
    // Equation 18
    {
      T zfz = egdts + T(0.25) * (((dw_s + dw_s1) + dw_c) + dw_c1);
      T zrom1v = hcpd * (d.tetav[cs + o] + tc);
      T udc = u[c + o];
      T uds = ii == 0 ? d.eu_i[jj + (size_t)nj * kk] : u[cs + o];
      T ude = jj == nj - 1 ? d.eu_j[ii + (size_t)ni * kk] : u[ce + o];
      T udes = jj == nj - 1 ? d.eu_j[im + (size_t)ni * kk]
                            : (ii == 0 ? d.eu_i[jp + (size_t)nj * kk] : u[ces + o]);
      T zcor1v = cv * (((udc + uds) + ude) + udes);
      T pas = ii == 0 ? d.ep_i[jj + (size_t)nj * kk] : d.pai[cs + o];
      vo[c + o] = ((v[c + o] - zcor1v) - (zfz * hy) * gzh) - (zcy * zrom1v) * (pc - pas);
    }
    dw_c = dw_c1; dw_w = dw_w1; dw_s = dw_s1;
  }
}

// ---- advection: staggered -> cross points (:1327-1341, :1389-1417) -----
template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY) k_stag_to_x(View<T> d) {
  int jj = blockIdx.x * kPtBX + threadIdx.x;
  int ii = blockIdx.y * kPtBY + threadIdx.y;
  const int nj = d.nj, ni = d.ni, kz = d.kz, kk = blockIdx.z;
  if (jj >= nj || ii >= ni) return;
  const T* __restrict__ u = d.ubuf[d.cur];
  const T* __restrict__ v = d.vbuf[d.cur];
  const size_t o = (size_t)kk * d.pl;
  const size_t c = jj + (size_t)nj * ii;
  const size_t rowj = (size_t)nj * ii;
  d.ux[o + c] = T(0.5625) * (u[o + rowj + wp1(jj, nj)] + u[o + c]) -
                T(0.0625) * (u[o + rowj + wp2(jj, nj)] + u[o + rowj + wm1(jj, nj)]);
  d.vx[o + c] = T(0.5625) * (v[o + jj + (size_t)nj * wp1(ii, ni)] + v[o + c]) -
                T(0.0625) * (v[o + jj + (size_t)nj * wp2(ii, ni)] + v[o + jj + (size_t)nj * wm1(ii, ni)]);
  const T* __restrict__ w = d.w;
  const size_t pl = d.pl;
  T wxv;
  if (kk == 0)
    wxv = T(0.5) * (w[c + pl] + w[c]);
  else if (kk == kz - 1)
    wxv = T(0.5) * (w[c + (size_t)kz * pl] + w[c + (size_t)(kz - 1) * pl]);
  else
    wxv = T(0.5625) * (w[c + (kk + 1) * pl] + w[c + kk * pl]) -
          T(0.0625) * (w[c + (kk + 2) * pl] + w[c + (kk - 1) * pl]);
  d.wx[o + c] = wxv;
}

// ---- advection: vertical WAF, two passes at dt/2 (:966-1073) ------------
// One thread per column streams k with a 4-value window.  Pass 2 works in
// place on wz: each level is read before it is overwritten.
template <class T>
__device__ __forceinline__ void waf_vpass(const T* src, T* dst, const T* __restrict__ s,
                                          const T* __restrict__ wafu, const T* __restrict__ wafd,
                                          size_t c, size_t pl, int kz, T dtrdz) {
  T a = src[c];
  T b = a;
  T cc = src[c + (kz > 1 ? pl : 0)];
  T wfw_k = T(0);
  T s_k = s[c];
  for (int k = 1; k <= kz; ++k) {  // 1-based level
    const size_t o = (size_t)(k - 1) * pl;
    const T s_k1 = s[c + (size_t)k * pl];  // s(k+1)
    const int k2 = k + 2 <= kz ? k + 2 : kz;
    const T dd = src[c + (size_t)(k2 - 1) * pl];
    T wfw_k1 = T(0);
    if (k <= kz - 1) {
      const T zamu = s_k1 * dtrdz;
      T is, num;
      if (zamu >= T(0)) {
        is = T(1); num = cc - dd;  // k1 = k+1, k1p1 = min(k+2, kz)
      } else {
        is = T(-1); num = a - b;   // k1 = max(k-1, 1), k1p1 = k
      }
      const T zzden = safeden(b - cc);
      const T r = num / zzden;
      const T bb = superbee(r);
      const T zphi = (is + zamu * bb) - is * bb;
      wfw_k1 = (T(0.5) * s_k1) * ((T(1) + zphi) * cc + (T(1) - zphi) * b);
    }
    const T zrfmu = wafu[c + o], zrfmd = wafd[c + o];
    const T zdv = (s_k * zrfmu - s_k1 * zrfmd) * b;
    dst[c + o] = ((b - wfw_k * zrfmu) + wfw_k1 * zrfmd) + zdv;
    a = b; b = cc; cc = dd; wfw_k = wfw_k1; s_k = s_k1;
  }
}


template <class T>
__global__ void __launch_bounds__(kColBX* kColBY) k_waf_vertical(View<T> d, FieldPtrs<T> fp) {
  int jj = blockIdx.x * kColBX + threadIdx.x;
  int ii = blockIdx.y * kColBY + threadIdx.y;
  const int nj = d.nj, ni = d.ni, kz = d.kz;
  if (jj >= nj || ii >= ni) return;
  const int f = blockIdx.z;
  const size_t pl = d.pl;
  const size_t c = jj + (size_t)nj * ii;
  T* wz = d.wz + (size_t)f * pl * kz;
  waf_vpass<T>(fp.f[f], wz, d.s, d.wafu, d.wafd, c, pl, kz, d.dtrdz_a);  // pp -> wz
  waf_vpass<T>(wz, wz, d.s, d.wafu, d.wafd, c, pl, kz, d.dtrdz_a);        // wz -> wz
}

// ---- advection: meridional WAF (:1075-1136) -----------------------------
// Block = 32 j x kTileBI i points of one level; the wz rows i-2..i+BI+1 and
// the BI+1 fluxes live in shared memory; all 10 fields reuse the velocity
// and metric terms loaded once per thread.
template <class T>
__global__ void __launch_bounds__(kPtBX* kTileBI) k_waf_meridional(View<T> d, FieldPtrs<T> fp) {
  constexpr int BI = kTileBI;
  __shared__ T wzt[BI + 4][kPtBX];
  __shared__ T flx[BI + 1][kPtBX];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int nj = d.nj, ni = d.ni, kz = d.kz;
  const size_t pl = d.pl;
  const int j0 = blockIdx.x * kPtBX, i0 = blockIdx.y * BI, kk = blockIdx.z;
  const int jj = j0 + tx;
  const bool jok = jj < nj;
  const int jc = jok ? jj : nj - 1;
  const size_t ko = (size_t)kk * pl;
  const T* __restrict__ v = d.vbuf[d.cur];
  const T dtrdy = d.dtrdy_a;
  // flux rows owned by this thread: q = ty, and q = BI for ty == 0
  T fv[2], fz[2], frm[2];
  bool fok[2];
  for (int n = 0; n < 2; ++n) {
    int q = n == 0 ? ty : BI;
    int ii = i0 + q;  // flux zpby at 1-based i = ii+1 (between ii-1 and ii)
    fok[n] = (n == 0 || ty == 0) && ii <= ni;
    int iv = ii < ni ? ii : ii - ni;
    size_t cq = jc + (size_t)nj * (fok[n] ? iv : 0);
    fv[n] = fok[n] ? v[ko + cq] : T(0);
    frm[n] = fok[n] ? d.rmv[cq] : T(1);
    fz[n] = d.rotllr ? fv[n] * dtrdy : (fv[n] * frm[n]) * dtrdy;
  }
  // output point
  const int io = i0 + ty;
  const bool ook = jok && io < ni;
  const int ion = io + 1 < ni ? io + 1 : 0;
  const size_t co = jc + (size_t)nj * (io < ni ? io : 0);
  const size_t con = jc + (size_t)nj * (io < ni ? ion : 0);
  const T zrfmn = d.wafn[ko + co], zrfms = d.wafs[ko + co];
  const T vs = v[ko + co], vn = v[ko + con];
  const T rmvs = d.rmv[co], rmvn = d.rmv[con], mx2 = d.mx2[co];
  for (int f = 0; f < kNumAdvected; ++f) {
    const T* __restrict__ wzf = d.wz + (size_t)f * pl * kz;
    for (int r = ty; r < BI + 4; r += BI) wzt[r][tx] = wzf[ko + jc + (size_t)nj * wrapn(i0 - 2 + r, ni)];
    __syncthreads();
    for (int n = 0; n < 2; ++n) {
      if (!fok[n]) continue;
      const int q = n == 0 ? ty : BI;
      const int r = q + 2;
      const T zamu = fz[n];
      T is, num;
      if (zamu > T(0)) {
        is = T(1); num = wzt[r - 1][tx] - wzt[r - 2][tx];   // ih = i-1, ihm1 = i-2
      } else {
        is = T(-1); num = wzt[r + 1][tx] - wzt[r][tx];      // ih = i+1, ihm1 = i
      }
      const T zzden = safeden(wzt[r][tx] - wzt[r - 1][tx]);
      const T rr = num / zzden;
      const T bb = superbee(rr);
      const T zphi = (is + zamu * bb) - is * bb;
      const T fl = (T(1) + zphi) * wzt[r - 1][tx] + (T(1) - zphi) * wzt[r][tx];
      flx[q][tx] = d.rotllr ? (T(0.5) * fv[n]) * fl : ((T(0.5) * fv[n]) * frm[n]) * fl;
    }
    __syncthreads();
    if (ook) {
      T* __restrict__ ppf = fp.f[f];
      const T pp = ppf[ko + co];
      T p0;
      if (d.rotllr) {
        const T zdv = (vn * zrfmn - vs * zrfms) * pp;
        p0 = ((wzt[ty + 2][tx] + flx[ty][tx] * zrfms) - flx[ty + 1][tx] * zrfmn) + zdv;
      } else {
        const T zdv = ((vn * rmvn) * zrfmn - (vs * rmvs) * zrfms) * pp;
        p0 = wzt[ty + 2][tx] + mx2 * (((flx[ty][tx] * zrfms) - flx[ty + 1][tx] * zrfmn) + zdv);
      }
      d.p0[(size_t)f * pl * kz + ko + co] = p0;
    }
    __syncthreads();
  }
}

// ---- advection: zonal WAF (:1138-1187), update of pp in place -----------
template <class T>
__global__ void __launch_bounds__(kPtBX* kTileBI) k_waf_zonal(View<T> d, FieldPtrs<T> fp) {
  constexpr int BI = kTileBI;
  constexpr int BX = kPtBX;
  __shared__ T p0t[BI][BX + 4];
  __shared__ T flx[BI][BX + 1];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int nj = d.nj, ni = d.ni, kz = d.kz;
  const size_t pl = d.pl;
  const int j0 = blockIdx.x * BX, i0 = blockIdx.y * BI, kk = blockIdx.z;
  const int ii = i0 + ty;
  const bool iok = ii < ni;
  const int ic = iok ? ii : ni - 1;
  const size_t ko = (size_t)kk * pl;
  const size_t row = (size_t)nj * ic;
  const T* __restrict__ u = d.ubuf[d.cur];
  const T dtrdx = d.dtrdx_a;
  T fu[2], fz[2], frm[2];
  bool fok[2];
  for (int n = 0; n < 2; ++n) {
    int q = n == 0 ? tx : BX;
    int jq = j0 + q;  // flux zpbw at 1-based j = jq+1
    fok[n] = (n == 0 || tx == 0) && jq <= nj;
    int ju = jq < nj ? jq : jq - nj;
    size_t cq = (fok[n] ? ju : 0) + row;
    fu[n] = fok[n] ? u[ko + cq] : T(0);
    T m = fok[n] ? (d.rotllr ? d.mu[cq] : d.rmu[cq]) : T(1);
    frm[n] = m;
    fz[n] = (fu[n] * m) * dtrdx;
  }
  const int jo = j0 + tx;
  const bool ook = iok && jo < nj;
  const int joe = jo + 1 < nj ? jo + 1 : 0;
  const size_t co = (jo < nj ? jo : 0) + row;
  const size_t coe = (jo < nj ? joe : 0) + row;
  const T zrfme = d.wafe[ko + co], zrfmw = d.wafw[ko + co];
  const T uw = u[ko + co], ue = u[ko + coe];
  const T rmuw = d.rmu[co], rmue = d.rmu[coe], mx2 = d.mx2[co];
  for (int f = 0; f < kNumAdvected; ++f) {
    const T* __restrict__ p0f = d.p0 + (size_t)f * pl * kz;
    for (int x = tx; x < BX + 4; x += BX) p0t[ty][x] = p0f[ko + row + wrapn(j0 - 2 + x, nj)];
    __syncthreads();
    for (int n = 0; n < 2; ++n) {
      if (!fok[n]) continue;
      const int q = n == 0 ? tx : BX;
      const int x = q + 2;
      const T zamu = fz[n];
      T is, num;
      if (zamu > T(0)) {
        is = T(1); num = p0t[ty][x - 1] - p0t[ty][x - 2];
      } else {
        is = T(-1); num = p0t[ty][x + 1] - p0t[ty][x];
      }
      const T zzden = safeden(p0t[ty][x] - p0t[ty][x - 1]);
      const T rr = num / zzden;
      const T bb = superbee(rr);
      const T zphi = (is + zamu * bb) - is * bb;
      const T fl = (T(1) + zphi) * p0t[ty][x - 1] + (T(1) - zphi) * p0t[ty][x];
      flx[ty][q] = d.rotllr ? (T(0.5) * fu[n]) * fl : ((T(0.5) * fu[n]) * frm[n]) * fl;
    }
    __syncthreads();
    if (ook) {
      T* __restrict__ ppf = fp.f[f];
      const T pp = ppf[ko + co];
      const T p0 = p0t[ty][tx + 2];
      T out;
      if (d.rotllr) {
        const T zdv = (ue * zrfme - uw * zrfmw) * pp;
        out = ((p0 + flx[ty][tx] * zrfmw) - flx[ty][tx + 1] * zrfme) + zdv;
      } else {
        const T zdv = ((ue * rmue) * zrfme - (uw * rmuw) * zrfmw) * pp;
        out = p0 + mx2 * (((flx[ty][tx] * zrfmw) - flx[ty][tx + 1] * zrfme) + zdv);
      }
      ppf[ko + co] = out;
    }
    __syncthreads();
  }
}

// ---- advection: cross points -> staggered (:1343-1387) ------------------
// Writes u, v into buffer 0 so every step replays the same pointers.
template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY) k_stag_from_x(View<T> d) {
  int jj = blockIdx.x * kPtBX + threadIdx.x;
  int ii = blockIdx.y * kPtBY + threadIdx.y;
  const int nj = d.nj, ni = d.ni, kz = d.kz, kk = blockIdx.z;
  if (jj >= nj || ii >= ni) return;
  const size_t pl = d.pl;
  const size_t o = (size_t)kk * pl;
  const size_t c = jj + (size_t)nj * ii;
  const size_t rowj = (size_t)nj * ii;
  const T* __restrict__ ux = d.ux;
  const T* __restrict__ vx = d.vx;
  d.ubuf[0][o + c] = T(0.5625) * (ux[o + c] + ux[o + rowj + wm1(jj, nj)]) -
                     T(0.0625) * (ux[o + rowj + wp1(jj, nj)] + ux[o + rowj + wm2(jj, nj)]);
  d.vbuf[0][o + c] = T(0.5625) * (vx[o + c] + vx[o + jj + (size_t)nj * wm1(ii, ni)]) -
                     T(0.0625) * (vx[o + jj + (size_t)nj * wp1(ii, ni)] + vx[o + jj + (size_t)nj * wm2(ii, ni)]);
  // w(k), k = 2..kz (1-based) <- wx ; level index kk = k-1 in 1..kz-1
  if (kk >= 1) {
    const T* __restrict__ wx = d.wx;
    T wv;
    if (kk == 1)
      wv = T(0.5) * (wx[c + pl] + wx[c]);
    else if (kk == kz - 1)
      wv = T(0.5) * (wx[c + (size_t)(kz - 1) * pl] + wx[c + (size_t)(kz - 2) * pl]);
    else
      wv = T(0.5625) * (wx[c + kk * pl] + wx[c + (kk - 1) * pl]) -
           T(0.0625) * (wx[c + (kk + 1) * pl] + wx[c + (kk - 2) * pl]);
    d.w[c + kk * pl] = wv;
  }
}

// ---- post-diagnostics (:355-391), one thread per column ----------------
template <class T>
__global__ void __launch_bounds__(kColBX* kColBY) k_postdiag(View<T> d, const T* __restrict__ zk,
                                                            const T* __restrict__ zkm1) {
  int jj = blockIdx.x * kColBX + threadIdx.x;
  int ii = blockIdx.y * kColBY + threadIdx.y;
  const int nj = d.nj, ni = d.ni, kz = d.kz;
  if (jj >= nj || ii >= ni) return;
  const size_t pl = d.pl;
  const size_t c = jj + (size_t)nj * ii;
  T tv_km1 = T(0), tv_k = T(0), p_k = T(0);
  for (int kk = 0; kk < kz; ++kk) {
    const size_t q = c + (size_t)kk * pl;
    const T pai = d.pai[q];
    const T tv = d.tetav[q] * pai;
    d.tvirt[q] = tv;
    const T qv = d.q[0][q], qc = d.q[1][q], qi = d.q[2][q], qr = d.q[3][q], qs = d.q[4][q];
    const T t = tv / ((((T(1) + T(kEp1) * qv) - qc) - qi) - qr - qs);
    d.t[q] = t;
    const T p = dpow(pai, T(kCpovr)) * T(kP00);
    d.p[q] = p;
    d.rho[q] = p / (T(kRgas) * t);
    d.qsat[q] = pfwsat(t, p);
    tv_km1 = tv_k; tv_k = tv; p_k = p;
  }
  const T z = zk[c], zm = zkm1[c];
  const T zdgz = z * T(kEgrav);
  T lrt = (tv_km1 - tv_k) / (zm - z);
  lrt = T(0.65) * lrt - T(0.35) * T(kLrate);
  const T tv = tv_k - (T(0.5) * z) * lrt;
  d.ps[c] = p_k * dexp(zdgz / (T(kRgas) * tv));
}

// ---- diagnostics: max/min ps, u, v (:395-411) and FP64 column sums ------
// partial record per block: maxps minps maxu minu maxv minv mass energy nonfinite
constexpr int kDiagN = 9;
template <class T>
__global__ void __launch_bounds__(kColBX* kColBY) k_diag_partial(View<T> d) {
  __shared__ double sh[kDiagN][kColBX * kColBY];
  const int tid = threadIdx.x + kColBX * threadIdx.y;
  int jj = blockIdx.x * kColBX + threadIdx.x;
  int ii = blockIdx.y * kColBY + threadIdx.y;
  const int nj = d.nj, ni = d.ni, kz = d.kz;
  double r[kDiagN] = {-INFINITY, INFINITY, -INFINITY, INFINITY, -INFINITY, INFINITY, 0.0, 0.0, 0.0};
  if (jj < nj && ii < ni) {
    const size_t pl = d.pl;
    const size_t c = jj + (size_t)nj * ii;
    const double ps = (double)d.ps[c];
    if (!isfinite(ps)) r[8] = 1.0;
    else { r[0] = ps; r[1] = ps; }
    const T* __restrict__ u = d.ubuf[d.cur];
    const T* __restrict__ v = d.vbuf[d.cur];
    double mass = 0.0, en = 0.0;
    for (int kk = 0; kk < kz; ++kk) {
      const size_t q = c + (size_t)kk * pl;
      const double uu = (double)u[q], vv = (double)v[q];
      r[2] = fmax(r[2], uu); r[3] = fmin(r[3], uu);
      r[4] = fmax(r[4], vv); r[5] = fmin(r[5], vv);
      const double rdz = (double)d.rho[q] * (double)d.dz[q];
      const double wm = 0.5 * ((double)d.w[q] + (double)d.w[q + pl]);
      mass += rdz;
      en += rdz * (kCvd * (double)d.t[q] + kEgrav * (double)d.zeta[q] + 0.5 * (uu * uu + vv * vv + wm * wm));
    }
    r[6] = mass; r[7] = en;
  }
  for (int n = 0; n < kDiagN; ++n) sh[n][tid] = r[n];
  __syncthreads();
  for (int st = (kColBX * kColBY) / 2; st > 0; st >>= 1) {
    if (tid < st) {
      sh[0][tid] = fmax(sh[0][tid], sh[0][tid + st]); sh[1][tid] = fmin(sh[1][tid], sh[1][tid + st]);
      sh[2][tid] = fmax(sh[2][tid], sh[2][tid + st]); sh[3][tid] = fmin(sh[3][tid], sh[3][tid + st]);
      sh[4][tid] = fmax(sh[4][tid], sh[4][tid + st]); sh[5][tid] = fmin(sh[5][tid], sh[5][tid + st]);
      sh[6][tid] += sh[6][tid + st]; sh[7][tid] += sh[7][tid + st]; sh[8][tid] += sh[8][tid + st];
    }
    __syncthreads();
  }
  if (tid == 0) {
    const size_t b = blockIdx.x + (size_t)gridDim.x * blockIdx.y;
    for (int n = 0; n < kDiagN; ++n) d.dpart[b * kDiagN + n] = sh[n][0];
  }
}

__global__ void __launch_bounds__(256) k_diag_final(const double* __restrict__ part, int nparts, double* res) {
  __shared__ double sh[kDiagN][256];
  const int tid = threadIdx.x;
  double r[kDiagN] = {-INFINITY, INFINITY, -INFINITY, INFINITY, -INFINITY, INFINITY, 0.0, 0.0, 0.0};
  for (int b = tid; b < nparts; b += 256) {  // fixed assignment: deterministic sums
    const double* p = part + (size_t)b * kDiagN;
    r[0] = fmax(r[0], p[0]); r[1] = fmin(r[1], p[1]); r[2] = fmax(r[2], p[2]); r[3] = fmin(r[3], p[3]);
    r[4] = fmax(r[4], p[4]); r[5] = fmin(r[5], p[5]); r[6] += p[6]; r[7] += p[7]; r[8] += p[8];
  }
  for (int n = 0; n < kDiagN; ++n) sh[n][tid] = r[n];
  __syncthreads();
  for (int st = 128; st > 0; st >>= 1) {
    if (tid < st) {
      sh[0][tid] = fmax(sh[0][tid], sh[0][tid + st]); sh[1][tid] = fmin(sh[1][tid], sh[1][tid + st]);
      sh[2][tid] = fmax(sh[2][tid], sh[2][tid + st]); sh[3][tid] = fmin(sh[3][tid], sh[3][tid + st]);
      sh[4][tid] = fmax(sh[4][tid], sh[4][tid + st]); sh[5][tid] = fmin(sh[5][tid], sh[5][tid + st]);
      sh[6][tid] += sh[6][tid + st]; sh[7][tid] += sh[7][tid + st]; sh[8][tid] += sh[8][tid + st];
    }
    __syncthreads();
  }
  if (tid == 0)
    for (int n = 0; n < kDiagN; ++n) res[n] = sh[n][0];
}

// =========================================================================
// Launchers.  Each returns the number of kernels it started.
// =========================================================================
inline thread_local KernelTimer* g_timer = nullptr;
void set_timer(KernelTimer* t) { g_timer = t; }
#define MOLOCH_LAUNCH(KIND, STREAM, ...)                        \
  do {                                                          \
    if (g_timer) g_timer->mark((KIND), (STREAM), true);         \
    __VA_ARGS__;                                                \
    if (g_timer) g_timer->mark((KIND), (STREAM), false);        \
  } while (0)
template <class T>
inline FieldPtrs<T> advected(const View<T>& d) {
  FieldPtrs<T> fp;
  fp.f[0] = d.tetav; fp.f[1] = d.pai; fp.f[2] = d.ux; fp.f[3] = d.vx; fp.f[4] = d.wx;
  for (int n = 0; n < 5; ++n) fp.f[5 + n] = d.q[n];
  return fp;
}

inline dim3 col_grid(int nj, int ni, int z = 1) {
  return dim3((nj + kColBX - 1) / kColBX, (ni + kColBY - 1) / kColBY, z);
}
inline dim3 pt_grid(int nj, int ni, int nz) {
  return dim3((nj + kPtBX - 1) / kPtBX, (ni + kPtBY - 1) / kPtBY, nz);
}
inline dim3 tile_grid(int nj, int ni, int nz) {
  return dim3((nj + kPtBX - 1) / kPtBX, (ni + kTileBI - 1) / kTileBI, nz);
}

template <class T>
int launch_prediag(const View<T>& d, cudaStream_t st, const PhaseFlags& fl) {
  MOLOCH_LAUNCH(KK_PREDIAG, st, k_prediag<T><<<pt_grid(d.nj, d.ni, d.kz), dim3(kPtBX, kPtBY), 0, st>>>(d, fl.filterpai, fl.filtertheta));
  return 1;
}

// one sound() call: nsound substeps; flips d.cur once per substep
template <class T>
int launch_sound(View<T>& d, cudaStream_t st, const PhaseFlags& fl) {
  int n = 0;
  const dim3 cb(kColBX, kColBY), cg = col_grid(d.nj, d.ni);
  const dim3 pb(kPtBX, kPtBY), pg = pt_grid(d.nj, d.ni, d.kz);
  for (int ns = 1; ns <= fl.nsound; ++ns) {
    const int last = ns == fl.nsound;
    MOLOCH_LAUNCH(KK_SOUND_DIV, st, k_sound_div<T><<<cg, cb, 0, st>>>(d));
    ++n;
    if (fl.divfilter) {
      MOLOCH_LAUNCH(KK_SOUND_COLUMN, st, k_sound_column<T><<<cg, cb, 0, st>>>(d, ns, last, 1));
      MOLOCH_LAUNCH(KK_LAP_FILTER, st, k_lap_filter<T><<<pg, pb, 0, st>>>(d, d.zdiv2b, d.zdiv2a, 1, T(0)));
      MOLOCH_LAUNCH(KK_PAI_UPDATE, st, k_pai_update<T><<<pg, pb, 0, st>>>(d, d.zdiv2a));
      n += 3;
    } else {
      MOLOCH_LAUNCH(KK_SOUND_COLUMN, st, k_sound_column<T><<<cg, cb, 0, st>>>(d, ns, last, 0));
      ++n;
    }
    MOLOCH_LAUNCH(KK_SOUND_MOMENTUM, st, k_sound_momentum<T><<<cg, cb, 0, st>>>(d));
    ++n;
    d.cur ^= 1;
  }
  return n;
}

template <class T>
int launch_advection(View<T>& d, cudaStream_t st) {
  const FieldPtrs<T> fp = advected(d);
  MOLOCH_LAUNCH(KK_STAG_TO_X, st, k_stag_to_x<T><<<pt_grid(d.nj, d.ni, d.kz), dim3(kPtBX, kPtBY), 0, st>>>(d));
  MOLOCH_LAUNCH(KK_WAF_VERTICAL, st, k_waf_vertical<T><<<col_grid(d.nj, d.ni, kNumAdvected), dim3(kColBX, kColBY), 0, st>>>(d, fp));
  MOLOCH_LAUNCH(KK_WAF_MERIDIONAL, st, k_waf_meridional<T><<<tile_grid(d.nj, d.ni, d.kz), dim3(kPtBX, kTileBI), 0, st>>>(d, fp));
  MOLOCH_LAUNCH(KK_WAF_ZONAL, st, k_waf_zonal<T><<<tile_grid(d.nj, d.ni, d.kz), dim3(kPtBX, kTileBI), 0, st>>>(d, fp));
  MOLOCH_LAUNCH(KK_STAG_FROM_X, st, k_stag_from_x<T><<<pt_grid(d.nj, d.ni, d.kz), dim3(kPtBX, kPtBY), 0, st>>>(d));
  d.cur = 0;
  return 5;
}

template <class T>
int launch_postdiag(View<T>& d, cudaStream_t st, const PhaseFlags& fl, const T* zk, const T* zkm1) {
  int n = 0;
  const dim3 pb(kPtBX, kPtBY), pg = pt_grid(d.nj, d.ni, d.kz);
  const size_t bytes = sizeof(T) * (size_t)d.pl * d.kz;
  if (fl.filterpai) {
    MOLOCH_LAUNCH(KK_FILTER_INCREMENT, st, k_filter_increment<T><<<pg, pb, 0, st>>>(d, d.pai, d.pf, d.fscr));
    cudaMemcpyAsync(d.pai, d.fscr, bytes, cudaMemcpyDeviceToDevice, st);
    ++n;
  }
  if (fl.filtertheta) {
    MOLOCH_LAUNCH(KK_FILTER_INCREMENT, st, k_filter_increment<T><<<pg, pb, 0, st>>>(d, d.tetav, d.tf, d.fscr));
    cudaMemcpyAsync(d.tetav, d.fscr, bytes, cudaMemcpyDeviceToDevice, st);
    ++n;
  }
  MOLOCH_LAUNCH(KK_POSTDIAG, st, k_postdiag<T><<<col_grid(d.nj, d.ni), dim3(kColBX, kColBY), 0, st>>>(d, zk, zkm1));
  return n + 1;
}

template <class T>
int launch_diag(const View<T>& d, cudaStream_t st) {
  const dim3 g = col_grid(d.nj, d.ni);
  MOLOCH_LAUNCH(KK_DIAG, st, k_diag_partial<T><<<g, dim3(kColBX, kColBY), 0, st>>>(d));
  MOLOCH_LAUNCH(KK_DIAG, st, k_diag_final<<<1, 256, 0, st>>>(d.dpart, (int)(g.x * g.y), d.dres));
  return 2;
}

int diag_parts(int nj, int ni) {
  const dim3 g = col_grid(nj, ni);
  return (int)(g.x * g.y);
}

}  // namespace MOLOCH_KNS
}  // namespace moloch
