// MOLOCH step kernels for sm_103a.  Included by one .cu file per arithmetic
// build (MOLOCH_KNS names the namespace): the exact FP64 build is compiled
// with --fmad=false so every expression keeps the reference's evaluation
// order; the fast build allows multiply-add contraction and also carries the
// FP32-storage instantiation.
//
// Kernel map (reference: nompi/mod_moloch.F90):
//   k_prediag          :289-323  p, qsat, tvirt, qwltot, qwitot, tetav
//   k_sound_div        :514-597  u/v halo + surface w + s (Eq. 10) + zdiv2 (Eq. 16)
//   k_sound_damp       :853-895 + :627-630  divdamp and the vertical s term
//   k_sound_column     :634-728  implicit w (Thomas, one thread per column),
//                      Exner/theta update, nompi pai halo order, s completion (:843-849)
//   k_lap_filter       :423-440 divergence_filter (mo_divfilter)
//   k_pai_update       :716-728 (split form used when the filter is on)
//   k_sound_momentum   :730-837  Equations 17, 18
//   k_waf_vertical     :966-1073  both vertical WAF passes in registers, all 10 fields,
//                      with (u,v,w) -> (ux,vx,wx) of :1327-1341, :1389-1417 formed on the fly
//   k_waf_horizontal   :1075-1187 meridional + zonal WAF of one level, p0 in shared memory
//   k_stag_from_x      :1343-1387  (ux,vx,wx) -> (u,v,w)
//   k_filter_increment :442-481 + :333-353 filtpai / filttheta
//   k_postdiag         :355-391  tvirt, t, p, rho, ps, qsat
//   k_diag_*           :395-411  max/min of ps, u, v; NaN/Inf check; FP64 column sums
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <cstdint>
#include <type_traits>

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

template <class T>
struct FieldPtrs {
  T* f[kNumAdvected];
};

// block-cooperative copy of a member's view into shared memory (batched kernels)
template <class V>
__device__ __forceinline__ void copy_view(V* dst, const V* __restrict__ src) {
  static_assert(sizeof(V) % 4 == 0, "view size");
  const int n = (int)(sizeof(V) / 4);
  const int nt = blockDim.x * blockDim.y;
  for (int q = threadIdx.x + blockDim.x * threadIdx.y; q < n; q += nt)
    reinterpret_cast<int*>(dst)[q] = reinterpret_cast<const int*>(src)[q];
}

// ---- small device helpers ---------------------------------------------
__device__ __forceinline__ int wm1(int x, int n) { return x == 0 ? n - 1 : x - 1; }
__device__ __forceinline__ int wp1(int x, int n) { return x == n - 1 ? 0 : x + 1; }
__device__ __forceinline__ int wm2(int x, int n) { int y = x - 2; return y < 0 ? y + n : y; }
__device__ __forceinline__ int wp2(int x, int n) { int y = x + 2; return y >= n ? y - n : y; }

// a*b - c*d and a*b + c*d with the multiply-add contraction fixed in FP32
// storage: left to the compiler either product may be fused, and which one
// it fuses depends on the code around the expression, so the same body in
// two kernels (k_sound_column and k_sound_column_tm; a batched kernel and
// the persistent ensemble kernel) could round differently.  FP64 keeps the
// expression as written (the exact build contracts nothing).
__device__ __forceinline__ float prod_sub(float a, float b, float c, float d) { return __fmaf_rn(a, b, -__fmul_rn(c, d)); }
__device__ __forceinline__ double prod_sub(double a, double b, double c, double d) { return a * b - c * d; }
__device__ __forceinline__ float prod_add(float a, float b, float c, float d) { return __fmaf_rn(c, d, __fmul_rn(a, b)); }
__device__ __forceinline__ double prod_add(double a, double b, double c, double d) { return a * b + c * d; }
__device__ __forceinline__ int wrapn(int x, int n) { int y = x % n; return y < 0 ? y + n : y; }
// periodic index for -n <= x < 2n (no integer division)
__device__ __forceinline__ int wrap2(int x, int n) { return x < 0 ? x + n : (x >= n ? x - n : x); }

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
// Quotient of the WAF limiter ratio.  FP64 builds: the IEEE quotient, as
// the reference.  FP32 storage: the fast approximate quotient (2 ulp); the
// ratio only selects and scales the limiter, and the FP32 error is measured
// against the FP64 step anyway.
__device__ __forceinline__ float qdiv(float a, float b) { return __fdividef(a, b); }

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
__device__ __forceinline__ void b_prediag(const View<T>& d, const int bx, const int by, const int bz, int filterpai, int filtertheta) {
  int jj = bx * kPtBX + threadIdx.x;
  int ii = by * kPtBY + threadIdx.y;
  if (jj >= d.nj || ii >= d.ni) return;
  size_t c = (size_t)jj + (size_t)d.nj * ii + (size_t)bz * d.pl;
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

template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY) k_prediag(View<T> d, int filterpai, int filtertheta) {
  b_prediag<T>(d, blockIdx.x, blockIdx.y, blockIdx.z, filterpai, filtertheta);
}

template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY)
    kb_prediag(const View<T>* __restrict__ views, const int4* __restrict__ tiles, int filterpai, int filtertheta) {
  __shared__ View<T> sv;
  const int4 t = tiles[blockIdx.x];
  copy_view(&sv, views + t.x);
  __syncthreads();
  b_prediag<T>(sv, t.y, t.z, t.w, filterpai, filtertheta);
}


// ---- sound: halo, surface w, s (Eq. 10), horizontal divergence (Eq. 16) ---
// One thread per point.  Boundary threads also store the pre-divdamp u/v
// edge values that the momentum step reads as the stale ud/vd halo ring
// (:730-735); the bottom level computes w(kz+1) and s(kz+1) (:536-549).
template <class T>
__device__ __forceinline__ void b_sound_div(const View<T>& d, const int bx, const int by, const int bz) {
  if (d.sur_skip && *d.sur_skip) return;  // the surrogate took this cycle
  const int jj = bx * kPtBX + threadIdx.x;
  const int ii = by * kPtBY + threadIdx.y;
  const int kk = bz;
  const int nj = d.nj, ni = d.ni, kz = d.kz;
  if (jj >= nj || ii >= ni) return;
  const size_t pl = d.pl;
  const int jp = wp1(jj, nj), ip = wp1(ii, ni);
  const T* __restrict__ u = d.ubuf[d.cur];
  const T* __restrict__ v = d.vbuf[d.cur];
  const size_t c = (size_t)jj + (size_t)nj * ii;
  const size_t ce = (size_t)jp + (size_t)nj * ii;  // (j+1, i)
  const size_t cn = (size_t)jj + (size_t)nj * ip;  // (j, i+1)
  const size_t o = (size_t)kk * pl;
  const T u0 = u[c + o], u1 = u[ce + o], v0 = v[c + o], v1 = v[cn + o];
  const T hx0 = d.hx[c], hx1 = d.hx[ce], hy0 = d.hy[c], hy1 = d.hy[cn];
  if (kk > 0) {  // s(k), k = 2..kz  (:557-570)
    const T u0p = u[c + o - pl], u1p = u[ce + o - pl], v0p = v[c + o - pl], v1p = v[cn + o - pl];
    T zuh = prod_add(u0 + u0p, hx0, u1 + u1p, hx1);
    T zvh = prod_add(v0 + v0p, hy0, v1 + v1p, hy1);
    d.s[c + o] = -((T(0.25) * (zuh + zvh)) * d.gzitak[kk]);
  }
  const T dtrdx = d.dtrdx, dtrdy = d.dtrdy;
  const T f = d.fmz[c + o];
  const T zrfmzum = d.rfw[c + o], zrfmzup = d.rfw[ce + o];
  const T zrfmzvm = d.rfs[c + o], zrfmzvp = d.rfs[cn + o];
  const T rmv0 = d.rmv[c], rmv1 = d.rmv[cn];
  // zum = (dtrdx u0) zrfmzum etc.; zup - zum and zvp - zvm with the
  // contraction fixed
  if (d.rotllr) {
    const T du = prod_sub(dtrdx * u1, zrfmzup, dtrdx * u0, zrfmzum);
    const T dv = prod_sub((dtrdy * v1) * zrfmzvp, rmv1, (dtrdy * v0) * zrfmzvm, rmv0);
    d.zdiv2a[c + o] = (f * d.mx[c]) * (du + dv);
  } else {
    const T rmu0 = d.rmu[c], rmu1 = d.rmu[ce];
    const T du = prod_sub((dtrdx * u1) * rmu1, zrfmzup, (dtrdx * u0) * rmu0, zrfmzum);
    const T dv = prod_sub((dtrdy * v1) * rmv1, zrfmzvp, (dtrdy * v0) * rmv0, zrfmzvm);
    d.zdiv2a[c + o] = (d.mx2[c] * f) * (du + dv);
  }
  if (jj == 0) d.eu_j[ii + (size_t)ni * kk] = u0;
  if (ii == ni - 1) d.eu_i[jj + (size_t)nj * kk] = u0;
  if (jj == nj - 1) d.ev_j[ii + (size_t)ni * kk] = v0;
  if (ii == 0) d.ev_i[jj + (size_t)nj * kk] = v0;
  if (kk == kz - 1) {  // surface w(kz+1), s(kz+1)
    T zuh = prod_add(u0, hx0, u1, hx1);
    T zvh = prod_add(v0, hy0, v1, hy1);
    T ws = T(0.5) * (zuh + zvh);
    d.w[c + (size_t)kz * pl] = ws;
    d.s[c + (size_t)kz * pl] = -ws;
  }
}

template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY) k_sound_div(View<T> d) {
  b_sound_div<T>(d, blockIdx.x, blockIdx.y, blockIdx.z);
}

template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY)
    kb_sound_div(const View<T>* __restrict__ views, const int4* __restrict__ tiles) {
  __shared__ View<T> sv;
  const int4 t = tiles[blockIdx.x];
  copy_view(&sv, views + t.x);
  __syncthreads();
  b_sound_div<T>(sv, t.y, t.z, t.w);
}


// ---- sound: divdamp (:853-895) and the vertical s term (:627-630) -------
// One thread per point: damps u and v in place (their halo edges already
// hold the pre-damping values) and writes the divergence the implicit
// solve starts from into zdiv2b.
template <class T>
__device__ __forceinline__ void b_sound_damp(const View<T>& d, const int bx, const int by, const int bz) {
  if (d.sur_skip && *d.sur_skip) return;  // the surrogate took this cycle
  const int jj = bx * kPtBX + threadIdx.x;
  const int ii = by * kPtBY + threadIdx.y;
  const int kk = bz;
  const int nj = d.nj, ni = d.ni;
  if (jj >= nj || ii >= ni) return;
  const size_t pl = d.pl;
  const size_t o = (size_t)kk * pl;
  const size_t c = (size_t)jj + (size_t)nj * ii;
  T* __restrict__ u = d.ubuf[d.cur];
  T* __restrict__ v = d.vbuf[d.cur];
  const T zc = d.zdiv2a[c + o];
  const T zw = d.zdiv2a[o + wm1(jj, nj) + (size_t)nj * ii];
  const T ze = d.zdiv2a[o + wp1(jj, nj) + (size_t)nj * ii];
  const T zs = d.zdiv2a[o + jj + (size_t)nj * wm1(ii, ni)];
  const T zn = d.zdiv2a[o + jj + (size_t)nj * wp1(ii, ni)];
  const T cd = d.cdamp[kk];
  u[c + o] = u[c + o] + ((cd * d.mu[c]) * (zc - zw));
  if (d.rotllr)
    v[c + o] = v[c + o] + cd * (zc - zs);
  else
    v[c + o] = v[c + o] + ((cd * d.mv[c]) * (zc - zs));
  const T p2d = prod_sub(T(0.125), ((zw + ze) + zs) + zn, T(0.5), zc);
  T zd = zc + d.ddamp2 * p2d;
  zd = zd + (d.fmz[c + o] * d.dtrdz) * (d.s[c + o] - d.s[c + o + pl]);
  d.zdiv2b[c + o] = zd;
}

template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY) k_sound_damp(View<T> d) {
  b_sound_damp<T>(d, blockIdx.x, blockIdx.y, blockIdx.z);
}

template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY)
    kb_sound_damp(const View<T>* __restrict__ views, const int4* __restrict__ tiles) {
  __shared__ View<T> sv;
  const int4 t = tiles[blockIdx.x];
  copy_view(&sv, views + t.x);
  __syncthreads();
  b_sound_damp<T>(sv, t.y, t.z, t.w);
}


// Exact FP32 -> FP64 widening on the integer pipe.  GB300 executes F2F
// conversions on its FP64 pipe (1/64 of the FP32 rate); these few integer
// operations do not touch it.  Zeros, normal values of either sign,
// infinities and NaNs convert exactly; FP32 subnormals become zero of the
// same sign.
__device__ __forceinline__ double widen_f32(float x) {
  const unsigned b = __float_as_uint(x);
  const unsigned ex = b & 0x7f800000u, sg = b & 0x80000000u;
  unsigned hi = (((b & 0x7fffffffu) >> 3) + 0x38000000u) | sg;  // exponent rebiased by 1023 - 127
  unsigned lo = b << 29;
  if (ex == 0u) { hi = sg; lo = 0u; }
  if (ex == 0x7f800000u) hi |= 0x7ff00000u;
  return __hiloint2double((int)hi, (int)lo);
}

// FP64 -> FP32 by truncation on the integer pipe: sign and exponent exact,
// mantissa cut to 23 bits (relative error < 2^-23).  Magnitudes below the
// FP32 normal range become zero, above it infinity; NaNs stay NaN.
__device__ __forceinline__ float narrow_trunc(double x) {
  const unsigned hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  const unsigned ax = hi & 0x7fffffffu;
  unsigned m = (__funnelshift_l(lo, hi, 3) - (896u << 23)) & 0x7fffffffu;  // exponent rebiased by 127 - 1023
  if (ax < 0x38100000u) m = 0u;
  if (ax >= 0x47f00000u) m = (ax > 0x7ff00000u || (ax == 0x7ff00000u && lo != 0u)) ? 0x7fc00000u : 0x7f800000u;
  return __uint_as_float(m | (hi & 0x80000000u));
}


// Quotient of the Exner/theta update in FP32 storage: the reciprocal
// estimate q = a * rcp(b) with one residual correction q + (a - b q) rcp(b)
// (Markstein's quotient correction, P. Markstein, "IA-64 and Elementary
// Functions", 2000): within one ulp of the IEEE quotient for the normal,
// well-scaled values it sees here (b = 1 + 0.96 qv + 4.8 qc), with no slow
// path or branch.  FP64 keeps the IEEE quotient.
__device__ __forceinline__ float div_corr(float a, float b) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));
  const float q = a * r;
  return fmaf(fmaf(-b, q, a), r, q);
}
__device__ __forceinline__ double div_corr(double a, double b) { return a / b; }

// FP64 quotient of the WAF limiter's slope ratio.  The exact build divides
// as the reference does (IEEE).  The contracting build (MOLOCH_NR_DDIV)
// refines an FP32 estimate of 1/b by two Newton-Raphson steps,
// x <- x + x (1 - b x), each of which doubles the correct bits (about 2^-22,
// 2^-44, then the FP64 precision), forms q = a x and applies one residual
// correction q + (a - b q) x (Markstein's quotient correction, as div_corr
// above): within one ulp of the IEEE quotient, with seven FP64 operations
// and no slow path, for |b| in the FP32 normal range, where the limiter's
// denominators lie (|b| >= kMinden = 1e-30); other b divide as IEEE.  The
// conversions run on the integer pipe (widen_f32, narrow_trunc).
__device__ __forceinline__ double div_nr(double a, double b) {
  const double ab = fabs(b);
  if (!(ab >= 1.2e-38 && ab <= 3.0e38)) return a / b;
  float rf;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(rf) : "f"(narrow_trunc(b)));
  double x = widen_f32(rf);
  x = fma(x, fma(-b, x, 1.0), x);
  x = fma(x, fma(-b, x, 1.0), x);
  const double q = a * x;
  return fma(fma(-b, q, a), x, q);
}
#if defined(MOLOCH_NR_DDIV)
__device__ __forceinline__ double qdiv(double a, double b) { return div_nr(a, b); }
#else
__device__ __forceinline__ double qdiv(double a, double b) { return a / b; }
#endif

// zrom1w of the implicit w with the latent-heat term of saturated rising
// air (:641-652).  FP32 storage: the term is evaluated on every level (fast
// divide) and selected, so the level loop has no data-dependent branch;
// FP64: the reference's branch and IEEE divide.
template <class T>
__device__ __forceinline__ T zrom1w_moist(T zrom1w, T qvk, T qsk, T qskm, T wk, T fz, T pkm, T tm, T ns1, T dts) {
  if constexpr (sizeof(T) == 4) {
    const T zqs = T(0.5) * (qsk + qskm);
    const T zdth = __fdividef((((((T(kEgrav) * wk) * ns1) * dts) * T(kWlhv)) * T(kWlhv)) * zqs,
                              (((T(kCpd) * pkm) * T(kRwat)) * tm) * tm);
    const T zl = zrom1w + zdth * fz;
    return (qvk > T(0.96) * qsk && wk > T(0.1)) ? zl : zrom1w;
  } else {
    if (qvk > T(0.96) * qsk && wk > T(0.1)) {
      const T zqs = T(0.5) * (qsk + qskm);
      const T zdth = ((((((T(kEgrav) * wk) * ns1) * dts) * T(kWlhv)) * T(kWlhv)) * zqs) /
                     ((((T(kCpd) * pkm) * T(kRwat)) * tm) * tm);
      zrom1w = zrom1w + zdth * fz;
    }
    return zrom1w;
  }
}

// ---- sound: implicit w (Thomas, :634-686) + Exner/theta (:690-728) -----
// One thread per column.  Down-sweep k = kz..2 with FP64 pivots in every
// mode, stash of the FP64 down-sweep values, then back-substitution fused
// with the Exner/theta/pai update of the level above it.
// defer_pai: leave zdiv2b final and pai to k_pai_update (divergence filter on).
// PD: levels loaded ahead of the level computed, in both sweeps (a register
// ring of PD level records).  The kernels use PD = 1.  A ring of 3 levels at 4 blocks per SM (so
// that the back-substitution finds more of the down-sweep's levels in L2)
// measured 13 % slower at 512 x 512 x 60: fewer columns in flight cost more
// bandwidth than the extra L2 hits saved.
template <class T, int PD>
__device__ __forceinline__ void b_sound_column(const View<T>& d, const int bx, const int by, const int bz, int nsound, int last, int defer_pai) {
  if (d.sur_skip && *d.sur_skip) return;  // the surrogate took this cycle
  const int jj = bx * kColBX + threadIdx.x;
  const int ii = by * kColBY + threadIdx.y;
  const int nj = d.nj, ni = d.ni, kz = d.kz;
  if (jj >= nj || ii >= ni) return;
  const size_t pl = d.pl;
  const size_t c = (size_t)jj + (size_t)nj * ii;
  // one restrict-qualified pointer per array, offset to this column, so the
  // loads of the next level can be issued ahead of the current level's
  // stores and FP64 work
  T* __restrict__ W = d.w + c;
  const T* __restrict__ FMZF = d.fmzf + c;
  const T* __restrict__ QV = d.q[0] + c;
  const T* __restrict__ QC = d.q[1] + c;
  T* __restrict__ TET = d.tetav + c;
  T* __restrict__ PAI = d.pai + c;
  const T* __restrict__ QSAT = d.qsat + c;
  const T* __restrict__ TT = d.t + c;
  T* __restrict__ ZD = d.zdiv2b + c;
  const T* __restrict__ FMZ = d.fmz + c;
  const T* __restrict__ QWL = d.qwltot + c;
  const T* __restrict__ QWI = d.qwitot + c;
  T* __restrict__ S = d.s + c;
  T* __restrict__ DW = d.deltaw + c;
  const T* __restrict__ FF = d.ffilt;
  const T ns = T(nsound), ns1 = T(nsound - 1);
  const T zcs2 = d.zcs2, dts = d.dts, egdts = d.egdts, dtrdz = d.dtrdz;

  // (b) down-sweep k = kz .. 2, loads of the next level issued one level ahead.
  // The pivots (den, its reciprocal zrapp and the ratio wwkw) are FP64 in
  // every mode.  FP64 storage: the right-hand-side sweep and the stash are
  // FP64 too (the reference's arithmetic).  FP32 storage: the right-hand
  // side and the stash are FP32, which keeps the FP64 pipe -- 1/64 of the
  // FP32 rate on GB300 -- to the pivot recurrence.
  constexpr bool kF32 = sizeof(T) == 4;
  using ST = typename std::conditional<kF32, float, double>::type;  // stash / RHS type
  ST* __restrict__ WPs = reinterpret_cast<ST*>(d.wp) + c;
  ST* __restrict__ WWs = reinterpret_cast<ST*>(d.wwkw) + c;
  const T wsurf = W[(size_t)kz * pl];  // w(kz+1) from k_sound_div
  ST wkp1 = (ST)wsurf;
  double wwp1 = 0.0;  // wwkw(kz+1) = 0 (FP64 storage)
  double cwp1 = 1.0;  // 1 - wwkw(kz+1) (FP32 storage)
  // level kk of the down-sweep reads w, fmzf, qv, ffilt at kk and tetav,
  // pai, qsat, zdiv2b, fmz, t at kk-1 (carried as the next level's kk values)
  struct Dn { T wk, fz, qv, ff, tkm, pkm, qskm, zdkm, fkm, tm; };
  auto load_dn = [&](int kk, Dn& x) {
    const size_t on = (size_t)kk * pl, onm = on - pl;
    x.wk = W[on]; x.fz = FMZF[on]; x.qv = QV[on]; x.ff = FF[kk];
    x.tkm = TET[onm]; x.pkm = PAI[onm]; x.qskm = QSAT[onm]; x.zdkm = ZD[onm];
    x.fkm = FMZ[onm]; x.tm = TT[onm];
  };
  size_t o = (size_t)(kz - 1) * pl;
  T zd_k = ZD[o], tk = TET[o], pk = PAI[o], fk = FMZ[o], qsk = QSAT[o];
  Dn dring[PD];
#pragma unroll
  for (int u = 0; u < PD; ++u)
    if (kz - 1 - u >= 1) load_dn(kz - 1 - u, dring[u]);
  for (int base = kz - 1; base >= 1; base -= PD) {
#pragma unroll
  for (int u = 0; u < PD; ++u) {
    const int kk = base - u;
    if (kk < 1) break;
    o = (size_t)kk * pl;
    const Dn cur = dring[u];
    if (kk - PD >= 1) load_dn(kk - PD, dring[u]);
    const T wk = cur.wk, fz = cur.fz, qvk = cur.qv, ff = cur.ff, tkm = cur.tkm, pkm = cur.pkm;
    const T qskm = cur.qskm, zd_km = cur.zdkm, fkm = cur.fkm, tm = cur.tm;
    T zrom1w = ((T(0.5) * T(kCpd)) * fz) * (tkm + tk);
    zrom1w = zrom1w - (((((T(kCpd) * wk) * fz) * fz) * ns) * dtrdz) * (tkm - tk);
    zrom1w = zrom1w_moist(zrom1w, qvk, qsk, qskm, wk, fz, pkm, tm, ns1, dts);
    T zwexpl = (wk - (zrom1w * dtrdz) * (pkm - pk)) - egdts;
    zwexpl = zwexpl + ((T(kRdrcv) * zrom1w) * dtrdz) * prod_sub(pkm, zd_km, pk, zd_k);
    const T zu_t = ((zcs2 * fkm) * zrom1w) * pkm + ff;
    const T zd_t = ((zcs2 * fk) * zrom1w) * pk + ff;
    ST wpk;
    double wwk;
    if constexpr (kF32) {
      // The pivot recurrence in FP64, written for the complement
      // c = 1 - wwkw: den = (1 + zd c(k+1)) + zu, c(k) = (1 + zd c(k+1)) / den
      // -- the reference's den = ((1 + zd) + zu) - zd wwkw(k+1) and
      // wwkw(k) = zu / den without the cancellation of zd against
      // zd wwkw(k+1).  Four FP64 operations a level: the quotient starts
      // from the FP32 estimate q0 = tt r (r the FP32 estimate of 1/den) and
      // takes one correction, r times the FP64 residual tt - den q0
      // (relative error ~2e-13); the widenings and narrowings run on the
      // integer pipe.  The FP32 right-hand side and the stash use r itself.
      const double zu = widen_f32(zu_t), zdd = widen_f32(zd_t);
      const double tt = fma(zdd, cwp1, 1.0);
      const double den = tt + zu;
      float r;
      asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(narrow_trunc(den)));
      const double q0 = widen_f32(narrow_trunc(tt) * r);
      const double rem = fma(-den, q0, tt);
      cwp1 = q0 + widen_f32(r * narrow_trunc(rem));
      wwk = 0.0;
      wpk = r * (zwexpl + zd_t * wkp1);
      WWs[o] = r * zu_t;
    } else {
      const double zu = (double)zu_t;
      const double zdd = (double)zd_t;
      const double den = ((1.0 + zdd) + zu) - zdd * wwp1;
      const double zrapp = 1.0 / den;
      wwk = zrapp * zu;
      wpk = zrapp * ((double)zwexpl + zdd * wkp1);
      WWs[o] = (ST)wwk;
    }
    WPs[o] = wpk;
    wkp1 = wpk; wwp1 = wwk;
    zd_k = zd_km; tk = tkm; pk = pkm; fk = fkm; qsk = qskm;
  }
  }

  // (c) back-substitution (:681-686) fused with the Exner/theta update of
  // the level above (:690-728); w(1) = 0 always (init_moloch :260-262).
  // Level kk is solved while level kk-1 is finalized; loads run PD ahead.
  const T rdrcv = T(kRdrcv);
  ST wlo_d = 0;
  T wlo = T(0);
  // finalize inputs of level m
  struct Fin { T zd, fmz, qv, qc, tet, qwl, qwi, pai, s, fmzf; };
  auto load_fin = [&](int m) {
    const size_t q = (size_t)m * pl;
    Fin f;
    f.zd = ZD[q]; f.fmz = FMZ[q]; f.qv = QV[q]; f.qc = QC[q]; f.tet = TET[q];
    f.qwl = QWL[q]; f.qwi = QWI[q]; f.pai = PAI[q];
    f.s = last ? S[q] : T(0);
    f.fmzf = last ? FMZF[q] : T(0);
    return f;
  };
  auto finalize = [&](int m, const Fin& f, T wl, T wh) {
    const size_t q = (size_t)m * pl;
    T zd = f.zd;
    zd = zd + (dtrdz * f.fmz) * (wl - wh);
    zd = div_corr(zd * ((T(1) + T(0.86) * f.qv) + T(3.2) * f.qc), (T(1) + T(0.96) * f.qv) + T(4.8) * f.qc);
    TET[q] = f.tet * (T(1) + (rdrcv * zd) * (prod_add(T(0.25), f.qv, T(4.2), f.qwl) + T(2.1) * f.qwi));
    if (defer_pai) {
      ZD[q] = zd;
    } else {
      if (jj == nj - 1) d.ep_j[ii + (size_t)ni * m] = f.pai;
      if (ii == ni - 1) d.ep_i[jj + (size_t)nj * m] = f.pai;
      PAI[q] = f.pai * (T(1) - rdrcv * zd);
    }
    if (last) S[q] = m == 0 ? T(0) : (wl + f.s) * f.fmzf;  // complete Equation 10 (:843-849)
  };
  // record m = 1 .. kz: the stash and old w of level m (m < kz) and the
  // finalize inputs of level m-1
  struct Bk { ST wp, ww; T wold; Fin f; };
  auto load_bk = [&](int m, Bk& x) {
    x.f = load_fin(m - 1);
    if (m < kz) {
      const size_t q = (size_t)m * pl;
      x.wp = WPs[q]; x.ww = WWs[q]; x.wold = W[q];
    }
  };
  Bk bring[PD];
#pragma unroll
  for (int u = 0; u < PD; ++u)
    if (1 + u <= kz) load_bk(1 + u, bring[u]);
  for (int base = 1; base <= kz; base += PD) {
#pragma unroll
  for (int u = 0; u < PD; ++u) {
    const int kk = base + u;
    if (kk > kz) break;
    const Bk cur = bring[u];
    if (kk + PD <= kz) load_bk(kk + PD, bring[u]);
    if (kk < kz) {
      const size_t q = (size_t)kk * pl;
      wlo_d = cur.wp + cur.ww * wlo_d;
      const T wn = (T)wlo_d;
      DW[q] = (-cur.wold) + wn;
      W[q] = wn;
      finalize(kk - 1, cur.f, wlo, wn);
      wlo = wn;
    } else {
      finalize(kz - 1, cur.f, wlo, wsurf);
    }
  }
  }
  if (last) S[(size_t)kz * pl] = T(0);
}

// FP32: 9 blocks of 128 threads per SM (56 registers, 24 bytes spilled):
// 1.5 waves at 512 x 512 instead of 1.68 with 8 blocks (4.51 against
// 4.61 ms per step; 10 blocks, 48 registers, 4.84 ms)
template <class T>
__global__ void __launch_bounds__(kColBX* kColBY, sizeof(T) == 4 ? 9 : 4) k_sound_column(View<T> d, int nsound, int last, int defer_pai) {
  b_sound_column<T, 1>(d, blockIdx.x, blockIdx.y, blockIdx.z, nsound, last, defer_pai);
}

template <class T>
__global__ void __launch_bounds__(kColBX* kColBY, sizeof(T) == 4 ? 8 : 4)
    kb_sound_column(const View<T>* __restrict__ views, const int4* __restrict__ tiles, int nsound, int last, int defer_pai) {
  __shared__ View<T> sv;
  const int4 t = tiles[blockIdx.x];
  copy_view(&sv, views + t.x);
  __syncthreads();
  b_sound_column<T, 1>(sv, t.y, t.z, t.w, nsound, last, defer_pai);
}



}  // namespace MOLOCH_KNS
}  // namespace moloch
#include "moloch_column_tm.cuh"
namespace moloch {
namespace MOLOCH_KNS {

// ---- 5-point Laplacian filter of one field, out of place ----------------
// out = a + coef(k) * (0.125*(aW+aE+aS+aN) - 0.5*a)   (:423-481)
// coef(k) = anu2 * xknu(k) when use_xknu, else the constant c0.
template <class T>
__device__ __forceinline__ void b_lap_filter(const View<T>& d, const int bx, const int by, const int bz) {
  if (d.sur_skip && *d.sur_skip) return;  // the surrogate took this cycle
  const T* __restrict__ a = d.zdiv2b;
  T* __restrict__ out = d.zdiv2a;

  int jj = bx * kPtBX + threadIdx.x;
  int ii = by * kPtBY + threadIdx.y;
  const int nj = d.nj, ni = d.ni;
  if (jj >= nj || ii >= ni) return;
  const size_t o = (size_t)bz * d.pl;
  const size_t c = jj + (size_t)nj * ii;
  T aw = a[o + wm1(jj, nj) + (size_t)nj * ii], ae = a[o + wp1(jj, nj) + (size_t)nj * ii];
  T as = a[o + jj + (size_t)nj * wm1(ii, ni)], an = a[o + jj + (size_t)nj * wp1(ii, ni)];
  T ac = a[o + c];
  T p2d = prod_sub(T(0.125), ((aw + ae) + as) + an, T(0.5), ac);
  const T coef = d.anu2 * d.xknu[bz];
  out[o + c] = ac + coef * p2d;
}

template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY) k_lap_filter(View<T> d) {
  b_lap_filter<T>(d, blockIdx.x, blockIdx.y, blockIdx.z);
}

template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY)
    kb_lap_filter(const View<T>* __restrict__ views, const int4* __restrict__ tiles) {
  __shared__ View<T> sv;
  const int4 t = tiles[blockIdx.x];
  copy_view(&sv, views + t.x);
  __syncthreads();
  b_lap_filter<T>(sv, t.y, t.z, t.w);
}


// pai update with the nompi halo order (:716-728), split form
template <class T>
__device__ __forceinline__ void b_pai_update(const View<T>& d, const int bx, const int by, const int bz) {
  if (d.sur_skip && *d.sur_skip) return;  // the surrogate took this cycle
  const T* __restrict__ zd = d.zdiv2a;

  int jj = bx * kPtBX + threadIdx.x;
  int ii = by * kPtBY + threadIdx.y;
  const int nj = d.nj, ni = d.ni, kk = bz;
  if (jj >= nj || ii >= ni) return;
  const size_t c = jj + (size_t)nj * ii + (size_t)kk * d.pl;
  const T pold = d.pai[c];
  if (jj == nj - 1) d.ep_j[ii + (size_t)ni * kk] = pold;
  if (ii == ni - 1) d.ep_i[jj + (size_t)nj * kk] = pold;
  d.pai[c] = pold * (T(1) - T(kRdrcv) * zd[c]);
}

template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY) k_pai_update(View<T> d) {
  b_pai_update<T>(d, blockIdx.x, blockIdx.y, blockIdx.z);
}

template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY)
    kb_pai_update(const View<T>* __restrict__ views, const int4* __restrict__ tiles) {
  __shared__ View<T> sv;
  const int4 t = tiles[blockIdx.x];
  copy_view(&sv, views + t.x);
  __syncthreads();
  b_pai_update<T>(sv, t.y, t.z, t.w);
}


// filtpai / filttheta on the step increment (:333-353, :442-481):
// x = a - ref; a = ((x + nupaitq * lap(x)) + ref), written to out
template <class T>
__device__ __forceinline__ void b_filter_increment(const View<T>& d, const int bx, const int by, const int bz, int which) {  const T* __restrict__ a = which ? d.tetav : d.pai;
  const T* __restrict__ ref = which ? d.tf : d.pf;
  T* __restrict__ out = d.fscr;

  int jj = bx * kPtBX + threadIdx.x;
  int ii = by * kPtBY + threadIdx.y;
  const int nj = d.nj, ni = d.ni;
  if (jj >= nj || ii >= ni) return;
  const size_t o = (size_t)bz * d.pl;
  auto X = [&](int j, int i) {
    size_t q = o + j + (size_t)nj * i;
    return a[q] - ref[q];
  };
  T xw = X(wm1(jj, nj), ii), xe = X(wp1(jj, nj), ii), xs = X(jj, wm1(ii, ni)), xn = X(jj, wp1(ii, ni));
  T xc = X(jj, ii);
  T p2d = prod_sub(T(0.125), ((xw + xe) + xs) + xn, T(0.5), xc);
  const size_t c = o + jj + (size_t)nj * ii;
  out[c] = (xc + T(kNupaitq) * p2d) + ref[c];
}

template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY) k_filter_increment(View<T> d, int which) {
  b_filter_increment<T>(d, blockIdx.x, blockIdx.y, blockIdx.z, which);
}

template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY)
    kb_filter_increment(const View<T>* __restrict__ views, const int4* __restrict__ tiles, int which) {
  __shared__ View<T> sv;
  const int4 t = tiles[blockIdx.x];
  copy_view(&sv, views + t.x);
  __syncthreads();
  b_filter_increment<T>(sv, t.y, t.z, t.w, which);
}


// ---- sound: momentum, Equations 17 and 18 (:737-837) --------------------
// One thread per point; reads u, v (current buffer, damped interior + the
// pre-damping edges) and writes the other buffer of the pair.
template <class T>
__device__ __forceinline__ void b_sound_momentum(const View<T>& d, const int bx, const int by, const int bz) {
  if (d.sur_skip && *d.sur_skip) return;  // the surrogate took this cycle
  const int jj = bx * kPtBX + threadIdx.x;
  const int ii = by * kPtBY + threadIdx.y;
  const int kk = bz;
  const int nj = d.nj, ni = d.ni;
  if (jj >= nj || ii >= ni) return;
  const size_t pl = d.pl;
  const int jm = wm1(jj, nj), jp = wp1(jj, nj), im = wm1(ii, ni), ip = wp1(ii, ni);
  const T* __restrict__ u = d.ubuf[d.cur];
  const T* __restrict__ v = d.vbuf[d.cur];
  T* __restrict__ uo = d.ubuf[d.cur ^ 1];
  T* __restrict__ vo = d.vbuf[d.cur ^ 1];
  const size_t c = (size_t)jj + (size_t)nj * ii;
  const size_t cw = (size_t)jm + (size_t)nj * ii, ce = (size_t)jp + (size_t)nj * ii;
  const size_t cs = (size_t)jj + (size_t)nj * im, cn = (size_t)jj + (size_t)nj * ip;
  const size_t cwn = (size_t)jm + (size_t)nj * ip, ces = (size_t)jp + (size_t)nj * im;
  const size_t o = (size_t)kk * pl, o1 = o + pl;
  const T dts = d.dts, egdts = d.egdts;
  const T dw_c = d.deltaw[c + o], dw_c1 = d.deltaw[c + o1];
  const T tc = d.tetav[c + o];
  const T pc = d.pai[c + o];
  const T gzh = d.gzitakh[kk];
  const T hcpd = T(0.5) * T(kCpd);
  // Equation 17
  {
    const T zcx = d.dtrdx * d.mu[c];
    const T zfz = egdts + T(0.25) * (((d.deltaw[cw + o] + d.deltaw[cw + o1]) + dw_c) + dw_c1);
    const T zrom1u = hcpd * (d.tetav[cw + o] + tc);
    const T vdc = v[c + o];
    const T vdw = jj == 0 ? d.ev_j[ii + (size_t)ni * kk] : v[cw + o];
    const T vdwn = jj == 0 ? d.ev_j[ip + (size_t)ni * kk] : (ii == ni - 1 ? d.ev_i[jm + (size_t)nj * kk] : v[cwn + o]);
    const T vdn = ii == ni - 1 ? d.ev_i[jj + (size_t)nj * kk] : v[cn + o];
    const T zcor1u = ((d.coru[c] * dts) * T(0.25)) * (((vdc + vdw) + vdwn) + vdn);
    const T paw = jj == 0 ? d.ep_j[ii + (size_t)ni * kk] : d.pai[cw + o];
    uo[c + o] = ((u[c + o] + zcor1u) - (zfz * d.hx[c]) * gzh) - (zcx * zrom1u) * (pc - paw);
  }
  // Equation 18
  {
    const T zcy = d.rotllr ? d.dtrdy : d.dtrdy * d.mv[c];
    const T zfz = egdts + T(0.25) * (((d.deltaw[cs + o] + d.deltaw[cs + o1]) + dw_c) + dw_c1);
    const T zrom1v = hcpd * (d.tetav[cs + o] + tc);
    const T udc = u[c + o];
    const T uds = ii == 0 ? d.eu_i[jj + (size_t)nj * kk] : u[cs + o];
    const T ude = jj == nj - 1 ? d.eu_j[ii + (size_t)ni * kk] : u[ce + o];
    const T udes = jj == nj - 1 ? d.eu_j[im + (size_t)ni * kk] : (ii == 0 ? d.eu_i[jp + (size_t)nj * kk] : u[ces + o]);
    const T zcor1v = ((d.corv[c] * dts) * T(0.25)) * (((udc + uds) + ude) + udes);
    const T pas = ii == 0 ? d.ep_i[jj + (size_t)nj * kk] : d.pai[cs + o];
    vo[c + o] = ((v[c + o] - zcor1v) - (zfz * d.hy[c]) * gzh) - (zcy * zrom1v) * (pc - pas);
  }
}

template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY) k_sound_momentum(View<T> d) {
  b_sound_momentum<T>(d, blockIdx.x, blockIdx.y, blockIdx.z);
}

template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY)
    kb_sound_momentum(const View<T>* __restrict__ views, const int4* __restrict__ tiles) {
  __shared__ View<T> sv;
  const int4 t = tiles[blockIdx.x];
  copy_view(&sv, views + t.x);
  __syncthreads();
  b_sound_momentum<T>(sv, t.y, t.z, t.w);
}

// ---- k-marching variants of the point kernels of the sound loop ---------
// One thread per (j, i) and chunk of kKC levels; the inputs of level k+1
// are loaded into registers before level k is computed and stored, so each
// thread keeps a level of loads in flight (the one-level-per-thread
// versions above leave that to the warp scheduler and stall on latency).
// Same arithmetic, expression by expression.
template <class T>
__device__ __forceinline__ void b_sound_div_km(const View<T>& d, const int bx, const int by, const int bz) {
  if (d.sur_skip && *d.sur_skip) return;  // the surrogate took this cycle
  const int jj = bx * kPtBX + threadIdx.x;
  const int ii = by * kPtBY + threadIdx.y;
  const int nj = d.nj, ni = d.ni, kz = d.kz;
  if (jj >= nj || ii >= ni) return;
  const int k0 = bz * kKC, k1 = min(kz, k0 + kKC);
  const size_t pl = d.pl;
  const int jp = wp1(jj, nj), ip = wp1(ii, ni);
  const T* __restrict__ u = d.ubuf[d.cur];
  const T* __restrict__ v = d.vbuf[d.cur];
  const size_t c = (size_t)jj + (size_t)nj * ii;
  const size_t ce = (size_t)jp + (size_t)nj * ii;  // (j+1, i)
  const size_t cn = (size_t)jj + (size_t)nj * ip;  // (j, i+1)
  const T hx0 = d.hx[c], hx1 = d.hx[ce], hy0 = d.hy[c], hy1 = d.hy[cn];
  const T dtrdx = d.dtrdx, dtrdy = d.dtrdy;
  const T rmv0 = d.rmv[c], rmv1 = d.rmv[cn];
  const bool rot = d.rotllr;
  const T mxc = rot ? d.mx[c] : d.mx2[c];
  const T rmu0 = rot ? T(0) : d.rmu[c], rmu1 = rot ? T(0) : d.rmu[ce];
  struct L { T u0, u1, v0, v1, f, rfw0, rfw1, rfs0, rfs1, gz; };
  auto load = [&](int k, L& x) {
    const size_t o = (size_t)k * pl;
    x.u0 = u[c + o]; x.u1 = u[ce + o]; x.v0 = v[c + o]; x.v1 = v[cn + o];
    x.f = d.fmz[c + o];
    x.rfw0 = d.rfw[c + o]; x.rfw1 = d.rfw[ce + o]; x.rfs0 = d.rfs[c + o]; x.rfs1 = d.rfs[cn + o];
    x.gz = d.gzitak[k];
  };
  T u0p = T(0), u1p = T(0), v0p = T(0), v1p = T(0);  // level k-1
  if (k0 > 0) {
    const size_t q = (size_t)(k0 - 1) * pl;
    u0p = u[c + q]; u1p = u[ce + q]; v0p = v[c + q]; v1p = v[cn + q];
  }
  L cur, nxt;
  load(k0, nxt);
  for (int kk = k0; kk < k1; ++kk) {
    cur = nxt;
    if (kk + 1 < k1) load(kk + 1, nxt);
    const size_t o = (size_t)kk * pl;
    const T u0 = cur.u0, u1 = cur.u1, v0 = cur.v0, v1 = cur.v1;
    if (kk > 0) {  // s(k), k = 2..kz  (:557-570)
      T zuh = prod_add(u0 + u0p, hx0, u1 + u1p, hx1);
      T zvh = prod_add(v0 + v0p, hy0, v1 + v1p, hy1);
      d.s[c + o] = -((T(0.25) * (zuh + zvh)) * cur.gz);
    }
    const T f = cur.f;
    if (rot) {
      const T du = prod_sub(dtrdx * u1, cur.rfw1, dtrdx * u0, cur.rfw0);
      const T dv = prod_sub((dtrdy * v1) * cur.rfs1, rmv1, (dtrdy * v0) * cur.rfs0, rmv0);
      d.zdiv2a[c + o] = (f * mxc) * (du + dv);
    } else {
      const T du = prod_sub((dtrdx * u1) * rmu1, cur.rfw1, (dtrdx * u0) * rmu0, cur.rfw0);
      const T dv = prod_sub((dtrdy * v1) * rmv1, cur.rfs1, (dtrdy * v0) * rmv0, cur.rfs0);
      d.zdiv2a[c + o] = (mxc * f) * (du + dv);
    }
    if (jj == 0) d.eu_j[ii + (size_t)ni * kk] = u0;
    if (ii == ni - 1) d.eu_i[jj + (size_t)nj * kk] = u0;
    if (jj == nj - 1) d.ev_j[ii + (size_t)ni * kk] = v0;
    if (ii == 0) d.ev_i[jj + (size_t)nj * kk] = v0;
    if (kk == kz - 1) {  // surface w(kz+1), s(kz+1)
      T zuh = prod_add(u0, hx0, u1, hx1);
      T zvh = prod_add(v0, hy0, v1, hy1);
      T ws = T(0.5) * (zuh + zvh);
      d.w[c + (size_t)kz * pl] = ws;
      d.s[c + (size_t)kz * pl] = -ws;
    }
    u0p = u0; u1p = u1; v0p = v0; v1p = v1;
  }
}

template <class T>
__device__ __forceinline__ void b_sound_damp_km(const View<T>& d, const int bx, const int by, const int bz) {
  if (d.sur_skip && *d.sur_skip) return;  // the surrogate took this cycle
  const int jj = bx * kPtBX + threadIdx.x;
  const int ii = by * kPtBY + threadIdx.y;
  const int nj = d.nj, ni = d.ni;
  if (jj >= nj || ii >= ni) return;
  const int k0 = bz * kKC, k1 = min(d.kz, k0 + kKC);
  const size_t pl = d.pl;
  const size_t c = (size_t)jj + (size_t)nj * ii;
  const size_t cw = (size_t)wm1(jj, nj) + (size_t)nj * ii, ce = (size_t)wp1(jj, nj) + (size_t)nj * ii;
  const size_t cs = (size_t)jj + (size_t)nj * wm1(ii, ni), cn = (size_t)jj + (size_t)nj * wp1(ii, ni);
  T* __restrict__ u = d.ubuf[d.cur];
  T* __restrict__ v = d.vbuf[d.cur];
  const T muc = d.mu[c];
  const T mvc = d.rotllr ? T(0) : d.mv[c];
  const T ddamp2 = d.ddamp2, dtrdz = d.dtrdz;
  struct L { T zc, zw, ze, zs, zn, s1, uc, vc, fz, cd; };
  auto load = [&](int k, L& x) {
    const size_t o = (size_t)k * pl;
    x.zc = d.zdiv2a[c + o]; x.zw = d.zdiv2a[cw + o]; x.ze = d.zdiv2a[ce + o];
    x.zs = d.zdiv2a[cs + o]; x.zn = d.zdiv2a[cn + o];
    x.s1 = d.s[c + o + pl];
    x.uc = u[c + o]; x.vc = v[c + o];
    x.fz = d.fmz[c + o];
    x.cd = d.cdamp[k];
  };
  T s_k = d.s[c + (size_t)k0 * pl];  // s(k); s(k+1) is carried to the next level
  L cur, nxt;
  load(k0, nxt);
  for (int kk = k0; kk < k1; ++kk) {
    cur = nxt;
    if (kk + 1 < k1) load(kk + 1, nxt);
    const size_t o = (size_t)kk * pl;
    const T zc = cur.zc, zw = cur.zw, ze = cur.ze, zs = cur.zs, zn = cur.zn, cd = cur.cd;
    u[c + o] = cur.uc + ((cd * muc) * (zc - zw));
    if (d.rotllr)
      v[c + o] = cur.vc + cd * (zc - zs);
    else
      v[c + o] = cur.vc + ((cd * mvc) * (zc - zs));
    const T p2d = prod_sub(T(0.125), ((zw + ze) + zs) + zn, T(0.5), zc);
    T zd = zc + ddamp2 * p2d;
    zd = zd + (cur.fz * dtrdz) * (s_k - cur.s1);
    d.zdiv2b[c + o] = zd;
    s_k = cur.s1;
  }
}

template <class T>
__device__ __forceinline__ void b_sound_momentum_km(const View<T>& d, const int bx, const int by, const int bz) {
  if (d.sur_skip && *d.sur_skip) return;  // the surrogate took this cycle
  const int jj = bx * kPtBX + threadIdx.x;
  const int ii = by * kPtBY + threadIdx.y;
  const int nj = d.nj, ni = d.ni;
  if (jj >= nj || ii >= ni) return;
  const int k0 = bz * kKC, k1 = min(d.kz, k0 + kKC);
  const size_t pl = d.pl;
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
  const T hcpd = T(0.5) * T(kCpd);
  const T zcx = d.dtrdx * d.mu[c];
  const T zcy = d.rotllr ? d.dtrdy : d.dtrdy * d.mv[c];
  const T corx = (d.coru[c] * dts) * T(0.25), cory = (d.corv[c] * dts) * T(0.25);
  const T hxc = d.hx[c], hyc = d.hy[c];
  struct L { T dwc1, dww1, dws1, tc, tw, ts, pc, pw, ps, uc, us, ue, ues, vc, vw, vwn, vn, gzh; };
  auto load = [&](int k, L& x) {
    const size_t o = (size_t)k * pl, o1 = o + pl;
    x.dwc1 = d.deltaw[c + o1]; x.dww1 = d.deltaw[cw + o1]; x.dws1 = d.deltaw[cs + o1];
    x.tc = d.tetav[c + o]; x.tw = d.tetav[cw + o]; x.ts = d.tetav[cs + o];
    x.pc = d.pai[c + o];
    x.pw = jj == 0 ? d.ep_j[ii + (size_t)ni * k] : d.pai[cw + o];
    x.ps = ii == 0 ? d.ep_i[jj + (size_t)nj * k] : d.pai[cs + o];
    x.vc = v[c + o];
    x.vw = jj == 0 ? d.ev_j[ii + (size_t)ni * k] : v[cw + o];
    x.vwn = jj == 0 ? d.ev_j[ip + (size_t)ni * k] : (ii == ni - 1 ? d.ev_i[jm + (size_t)nj * k] : v[cwn + o]);
    x.vn = ii == ni - 1 ? d.ev_i[jj + (size_t)nj * k] : v[cn + o];
    x.uc = u[c + o];
    x.us = ii == 0 ? d.eu_i[jj + (size_t)nj * k] : u[cs + o];
    x.ue = jj == nj - 1 ? d.eu_j[ii + (size_t)ni * k] : u[ce + o];
    x.ues = jj == nj - 1 ? d.eu_j[im + (size_t)ni * k] : (ii == 0 ? d.eu_i[jp + (size_t)nj * k] : u[ces + o]);
    x.gzh = d.gzitakh[k];
  };
  // deltaw at level k of (c, w, s); level k+1 is carried to the next level
  T dw_c = d.deltaw[c + (size_t)k0 * pl], dw_w = d.deltaw[cw + (size_t)k0 * pl];
  T dw_s = d.deltaw[cs + (size_t)k0 * pl];
  L cur, nxt;
  load(k0, nxt);
  for (int kk = k0; kk < k1; ++kk) {
    cur = nxt;
    if (kk + 1 < k1) load(kk + 1, nxt);
    const size_t o = (size_t)kk * pl;
    const T tc = cur.tc, pc = cur.pc, gzh = cur.gzh;
    // Equation 17
    {
      const T zfz = egdts + T(0.25) * (((dw_w + cur.dww1) + dw_c) + cur.dwc1);
      const T zrom1u = hcpd * (cur.tw + tc);
      const T zcor1u = corx * (((cur.vc + cur.vw) + cur.vwn) + cur.vn);
      uo[c + o] = ((cur.uc + zcor1u) - (zfz * hxc) * gzh) - (zcx * zrom1u) * (pc - cur.pw);
    }
    // Equation 18
    {
      const T zfz = egdts + T(0.25) * (((dw_s + cur.dws1) + dw_c) + cur.dwc1);
      const T zrom1v = hcpd * (cur.ts + tc);
      const T zcor1v = cory * (((cur.uc + cur.us) + cur.ue) + cur.ues);
      vo[c + o] = ((cur.vc - zcor1v) - (zfz * hyc) * gzh) - (zcy * zrom1v) * (pc - cur.ps);
    }
    dw_c = cur.dwc1; dw_w = cur.dww1; dw_s = cur.dws1;
  }
}

#define MOLOCH_KM_KERNELS(NAME)                                                                      \
  template <class T>                                                                                 \
  __global__ void __launch_bounds__(kPtBX* kPtBY) k_##NAME##_km(View<T> d) {                          \
    b_##NAME##_km<T>(d, blockIdx.x, blockIdx.y, blockIdx.z);                                         \
  }                                                                                                  \
  template <class T>                                                                                 \
  __global__ void __launch_bounds__(kPtBX* kPtBY)                                                    \
      kb_##NAME##_km(const View<T>* __restrict__ views, const int4* __restrict__ tiles) {            \
    __shared__ View<T> sv;                                                                           \
    const int4 t = tiles[blockIdx.x];                                                                \
    copy_view(&sv, views + t.x);                                                                     \
    __syncthreads();                                                                                 \
    b_##NAME##_km<T>(sv, t.y, t.z, t.w);                                                             \
  }
MOLOCH_KM_KERNELS(sound_div)
MOLOCH_KM_KERNELS(sound_damp)
MOLOCH_KM_KERNELS(sound_momentum)
#undef MOLOCH_KM_KERNELS


// ---- momentum as warp strips (:730-837) -------------------------------------
// asynchronous global -> shared copies (cp.async, one element per lane)
template <class T>
__device__ __forceinline__ void cp_async_elem(T* dst_smem, const T* src) {
  const uint32_t dst = static_cast<uint32_t>(__cvta_generic_to_shared(dst_smem));
  if constexpr (sizeof(T) == 4)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// One warp per strip of 30 output columns x R rows of one level, lanes on
// columns j0-1 .. j0+30.  West and east neighbours come from the lanes
// beside (shuffles), the row below and the row above (v at i+1) from a ring
// of kMomS row slots in shared memory: the six state arrays of a row (u, v,
// tetav, pai, deltaw at k and k+1) are copied there with cp.async
// kMomS - 3 rows ahead of the row computed, each lane copying and later
// reading only its own column, so the pipeline needs no warp barrier and
// holds no registers; the 2-D metric fields come one row ahead in
// registers.  The stale-halo reads of the reference (edge buffers at
// j = 1, j = nj, i = 1, i = ni) replace the neighbour values on those lanes
// and rows, as in k_sound_momentum.
constexpr int kMomS = 6;  // row slots: rows i-1, i, i+1 and three in flight
template <class T>
using MomSlots = T[kMomS][6][32];  // one warp's ring: [slot][array][lane]
template <class T>
using MomRing = MomSlots<T>[4];    // [warp] of a 128-thread block

// bx: block of nw strips, wid: this warp's strip in it, rg: its ring
template <class T>
__device__ __forceinline__ void b_momentum_strip(const View<T>& d, const int bx, const int k, const int R,
                                                 MomSlots<T>& rg, const int wid, const int nw) {
  if (d.sur_skip && *d.sur_skip) return;  // the surrogate took this cycle
  const int lane = threadIdx.x & 31;
  const int nj = d.nj, ni = d.ni, pl = d.pl;
  const int nsj = (nj + kMomJ - 1) / kMomJ, nsi = (ni + R - 1) / R;
  const int w = bx * nw + wid;
  if (w >= nsj * nsi) return;  // whole warp
  const int sj = w % nsj, si = w / nsj;
  const int jl = sj * kMomJ - 1 + lane;
  const int jj = wrapn(jl, nj);
  const bool out_lane = lane >= 1 && lane <= kMomJ && jl < nj;
  const int i_s = si * R, i_e = min(i_s + R, ni);
  const size_t o = (size_t)k * pl, o1 = o + pl;
  const T* __restrict__ u = d.ubuf[d.cur] + o;
  const T* __restrict__ v = d.vbuf[d.cur] + o;
  T* __restrict__ uo = d.ubuf[d.cur ^ 1] + o;
  T* __restrict__ vo = d.vbuf[d.cur ^ 1] + o;
  const T* __restrict__ tet = d.tetav + o;
  const T* __restrict__ pai = d.pai + o;
  const T* __restrict__ dw0 = d.deltaw + o;
  const T* __restrict__ dw1 = d.deltaw + o1;
  const T dts = d.dts, egdts = d.egdts, dtrdx = d.dtrdx, dtrdy = d.dtrdy;
  const T hcpd = T(0.5) * T(kCpd);
  const T gzh = d.gzitakh[k];
  const bool rot = d.rotllr;
  const int jm = wm1(jj, nj), jp = wp1(jj, nj);
  // rows i_s-1 .. i_e stream through the slots in order; the slot indices
  // rotate by one per row
  auto nxt = [](int q) { return q + 1 == kMomS ? 0 : q + 1; };
  auto issue = [&](int r, int q) {  // copies of row r into slot q (nothing past i_e); one group either way
    if (r <= i_e) {
      const size_t c = (size_t)jj + (size_t)nj * wrap2(r, ni);
      T(*const sl)[32] = rg[q];
      cp_async_elem(&sl[0][lane], u + c);
      cp_async_elem(&sl[1][lane], v + c);
      cp_async_elem(&sl[2][lane], tet + c);
      cp_async_elem(&sl[3][lane], pai + c);
      cp_async_elem(&sl[4][lane], dw0 + c);
      cp_async_elem(&sl[5][lane], dw1 + c);
    }
    cp_async_commit();
  };
  // 2-D fields of a row, one row ahead in registers
  struct Row2 { T coru, corv, hx, hy, mu, mv; };
  auto load2 = [&](int i, Row2& x) {
    const size_t c = (size_t)jj + (size_t)nj * wrap2(i, ni);
    x.coru = d.coru[c]; x.corv = d.corv[c]; x.hx = d.hx[c]; x.hy = d.hy[c]; x.mu = d.mu[c];
    x.mv = rot ? T(0) : d.mv[c];
  };
  for (int r = i_s - 1, q = 0; r <= i_s + kMomS - 3; ++r, ++q) issue(r, q);
  Row2 c2, n2;
  load2(i_s, n2);
  // slots of rows i-1, i, i+1 and of the row issued next (i + kMomS - 2)
  int qb = 0, qc = 1, qn = 2, qi = kMomS - 1;
  // a strip that touches none of the domain edges (j = 1, nj; i = 1, ni)
  // never reads the stale-halo edge buffers: its rows run a copy of the
  // step without those tests
  const bool interior = sj != 0 && sj != nsj - 1 && i_s != 0 && i_e != ni;
  auto row = [&](const int i, auto edge) {
    constexpr bool EDGE = decltype(edge)::value;
    issue(i + kMomS - 2, qi);        // into the slot of row i-2
    cp_async_wait<kMomS - 3>();      // rows up to i+1 have landed
    c2 = n2;
    if (i + 1 < i_e) load2(i + 1, n2);
    const T(*const sb)[32] = rg[qb];
    const T(*const sc)[32] = rg[qc];
    const T(*const sn)[32] = rg[qn];
    const T cu = sc[0][lane], cv = sc[1][lane], ct = sc[2][lane], cp = sc[3][lane];
    const T cd0 = sc[4][lane], cd1 = sc[5][lane];
    const T us = sb[0][lane], ts = sb[2][lane], ps = sb[3][lane], ds0 = sb[4][lane], ds1 = sb[5][lane];
    const T vn = sn[1][lane];
    const int ii = i;
    // neighbours from the lanes beside
    const T ue = __shfl_down_sync(0xffffffffu, cu, 1);
    const T ues = __shfl_down_sync(0xffffffffu, us, 1);
    const T vw = __shfl_up_sync(0xffffffffu, cv, 1);
    const T vwn = __shfl_up_sync(0xffffffffu, vn, 1);
    const T tw = __shfl_up_sync(0xffffffffu, ct, 1);
    const T pw = __shfl_up_sync(0xffffffffu, cp, 1);
    const T dw0w = __shfl_up_sync(0xffffffffu, cd0, 1);
    const T dw1w = __shfl_up_sync(0xffffffffu, cd1, 1);
    if (out_lane) {
      const T dw_c = cd0, dw_c1 = cd1;
      const T tc = ct, pc = cp;
      // Equation 17
      {
        const T zcx = dtrdx * c2.mu;
        const T zfz = egdts + T(0.25) * (((dw0w + dw1w) + dw_c) + dw_c1);
        const T zrom1u = hcpd * (tw + tc);
        const T vdc = cv;
        T vdw = vw, vdwn = vwn, vdn = vn, paw = pw;
        if (EDGE) {
          const int ip = wp1(ii, ni);
          vdw = jj == 0 ? d.ev_j[ii + (size_t)ni * k] : vw;
          vdwn = jj == 0 ? d.ev_j[ip + (size_t)ni * k] : (ii == ni - 1 ? d.ev_i[jm + (size_t)nj * k] : vwn);
          vdn = ii == ni - 1 ? d.ev_i[jj + (size_t)nj * k] : vn;
          paw = jj == 0 ? d.ep_j[ii + (size_t)ni * k] : pw;
        }
        const T zcor1u = ((c2.coru * dts) * T(0.25)) * (((vdc + vdw) + vdwn) + vdn);
        uo[(size_t)jj + (size_t)nj * ii] = ((cu + zcor1u) - (zfz * c2.hx) * gzh) - (zcx * zrom1u) * (pc - paw);
      }
      // Equation 18
      {
        const T zcy = rot ? dtrdy : dtrdy * c2.mv;
        const T zfz = egdts + T(0.25) * (((ds0 + ds1) + dw_c) + dw_c1);
        const T zrom1v = hcpd * (ts + tc);
        const T udc = cu;
        T uds = us, ude = ue, udes = ues, pas = ps;
        if (EDGE) {
          const int im = wm1(ii, ni);
          uds = ii == 0 ? d.eu_i[jj + (size_t)nj * k] : us;
          ude = jj == nj - 1 ? d.eu_j[ii + (size_t)ni * k] : ue;
          udes = jj == nj - 1 ? d.eu_j[im + (size_t)ni * k] : (ii == 0 ? d.eu_i[jp + (size_t)nj * k] : ues);
          pas = ii == 0 ? d.ep_i[jj + (size_t)nj * k] : ps;
        }
        const T zcor1v = ((c2.corv * dts) * T(0.25)) * (((udc + uds) + ude) + udes);
        vo[(size_t)jj + (size_t)nj * ii] = ((cv - zcor1v) - (zfz * c2.hy) * gzh) - (zcy * zrom1v) * (pc - pas);
      }
    }
    qb = qc; qc = qn; qn = nxt(qn); qi = nxt(qi);
  };
  if (interior)
    for (int i = i_s; i < i_e; ++i) row(i, std::false_type());
  else
    for (int i = i_s; i < i_e; ++i) row(i, std::true_type());
  cp_async_wait<0>();  // no copy outlives the kernel
}

template <class T>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 8 : 4) k_momentum_strip(View<T> d, int R) {
  __shared__ __align__(16) MomRing<T> ring;
  b_momentum_strip<T>(d, blockIdx.x, blockIdx.y, R, ring[threadIdx.x >> 5], threadIdx.x >> 5, 4);
}

template <class T>
__global__ void __launch_bounds__(128)
    kb_momentum_strip(const View<T>* __restrict__ views, const int4* __restrict__ tiles, int R) {
  __shared__ View<T> sv;
  __shared__ __align__(16) MomRing<T> ring;
  const int4 t = tiles[blockIdx.x];
  copy_view(&sv, views + t.x);
  __syncthreads();
  b_momentum_strip<T>(sv, t.y, t.z, R, ring[threadIdx.x >> 5], threadIdx.x >> 5, 4);
}

// ---- momentum as warp strips, two columns per lane (FP32, jx even) --------
// b_momentum_strip with each lane on a pair of adjacent columns: strip s
// computes columns 62 s - 1 .. 62 s + 60 (inside the domain), lane l holds
// columns 62 s - 2 + 2 l and the next one, so a warp covers 62 output
// columns with 64 loaded.  The six state arrays of a row arrive as one
// 8-byte cp.async copy per array and lane, the metric fields as 8-byte
// loads; a west or east neighbour is the lane's own other column or one
// shuffle of the lane beside (half the copies, shared loads, shuffles and
// address arithmetic per point of the one-column strips).  Pairs start at
// even columns, and with jx even a pair never straddles the periodic seam,
// so every copy and load is 8-byte aligned.  The same expressions in the
// same order as b_momentum_strip: the results are bit-identical.
constexpr int kMom2J = 62;
constexpr int kMom2S = 6;  // row slots: rows i-1, i, i+1 and three in flight
using Mom2Slots = float[kMom2S][6][64];  // one warp's ring: [slot][array][column]

__device__ __forceinline__ void cp_async_8(void* dst_smem, const void* src) {
  const uint32_t dst = static_cast<uint32_t>(__cvta_generic_to_shared(dst_smem));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
}

__device__ __forceinline__ void b_momentum_strip2(const View<float>& d, const int bx, const int k, const int R,
                                                  Mom2Slots& rg, const int wid, const int nw) {
  if (d.sur_skip && *d.sur_skip) return;  // the surrogate took this cycle
  const int lane = threadIdx.x & 31;
  const int nj = d.nj, ni = d.ni, pl = d.pl;
  const int nsj = (nj + 1 + kMom2J - 1) / kMom2J, nsi = (ni + R - 1) / R;
  const int w = bx * nw + wid;
  if (w >= nsj * nsi) return;  // whole warp
  const int sj = w % nsj, si = w / nsj;
  const int cl = kMom2J * sj - 2 + 2 * lane;  // first column of the pair, before wrapping
  const int ja = wrapn(cl, nj), jb = ja + 1;  // ja even, so jb < nj
  const bool out0 = lane >= 1 && cl >= 0 && cl < nj;
  const bool out1 = lane <= 30 && cl + 1 >= 0 && cl + 1 < nj;
  const int i_s = si * R, i_e = min(i_s + R, ni);
  const size_t o = (size_t)k * pl, o1 = o + pl;
  const float* __restrict__ u = d.ubuf[d.cur] + o;
  const float* __restrict__ v = d.vbuf[d.cur] + o;
  float* __restrict__ uo = d.ubuf[d.cur ^ 1] + o;
  float* __restrict__ vo = d.vbuf[d.cur ^ 1] + o;
  const float* __restrict__ tet = d.tetav + o;
  const float* __restrict__ pai = d.pai + o;
  const float* __restrict__ dw0 = d.deltaw + o;
  const float* __restrict__ dw1 = d.deltaw + o1;
  const float dts = d.dts, egdts = d.egdts, dtrdx = d.dtrdx, dtrdy = d.dtrdy;
  const float hcpd = 0.5f * float(kCpd);
  const float gzh = d.gzitakh[k];
  const bool rot = d.rotllr;
  auto nxt = [](int q) { return q + 1 == kMom2S ? 0 : q + 1; };
  auto issue = [&](int r, int q) {  // copies of row r into slot q (nothing past i_e); one group either way
    if (r <= i_e) {
      const size_t c = (size_t)ja + (size_t)nj * wrap2(r, ni);
      float(*const sl)[64] = rg[q];
      cp_async_8(&sl[0][2 * lane], u + c);
      cp_async_8(&sl[1][2 * lane], v + c);
      cp_async_8(&sl[2][2 * lane], tet + c);
      cp_async_8(&sl[3][2 * lane], pai + c);
      cp_async_8(&sl[4][2 * lane], dw0 + c);
      cp_async_8(&sl[5][2 * lane], dw1 + c);
    }
    cp_async_commit();
  };
  struct Row2 { float2 coru, corv, hx, hy, mu, mv; };
  auto ld2 = [](const float* p) { return *reinterpret_cast<const float2*>(p); };
  auto load2 = [&](int i, Row2& x) {
    const size_t c = (size_t)ja + (size_t)nj * wrap2(i, ni);
    x.coru = ld2(d.coru + c); x.corv = ld2(d.corv + c); x.hx = ld2(d.hx + c); x.hy = ld2(d.hy + c);
    x.mu = ld2(d.mu + c);
    x.mv = rot ? make_float2(0.f, 0.f) : ld2(d.mv + c);
  };
  for (int r = i_s - 1, q = 0; r <= i_s + kMom2S - 3; ++r, ++q) issue(r, q);
  Row2 c2, n2;
  load2(i_s, n2);
  int qb = 0, qc = 1, qn = 2, qi = kMom2S - 1;
  const bool interior = sj != 0 && sj != nsj - 1 && i_s != 0 && i_e != ni;
  // one column: its values, its west / east neighbours and metric terms
  struct Col { float cu, cv, ct, cp, cd0, cd1, us, ts, ps, ds0, ds1, vn; };
  auto point = [&](const int jj, const int ii, const Col& x, const float vw, const float vwn, const float tw,
                   const float pw, const float dw0w, const float dw1w, const float ue, const float ues,
                   const float coru, const float corv, const float hx, const float hy, const float mu,
                   const float mv, auto edge, float& un, float& vnew) {
    constexpr bool EDGE = decltype(edge)::value;
    // Equation 17
    {
      const float zcx = dtrdx * mu;
      const float zfz = egdts + 0.25f * (((dw0w + dw1w) + x.cd0) + x.cd1);
      const float zrom1u = hcpd * (tw + x.ct);
      float vdw = vw, vdwn = vwn, vdn = x.vn, paw = pw;
      if (EDGE) {
        const int ip = wp1(ii, ni), jm = wm1(jj, nj);
        vdw = jj == 0 ? d.ev_j[ii + (size_t)ni * k] : vw;
        vdwn = jj == 0 ? d.ev_j[ip + (size_t)ni * k] : (ii == ni - 1 ? d.ev_i[jm + (size_t)nj * k] : vwn);
        vdn = ii == ni - 1 ? d.ev_i[jj + (size_t)nj * k] : x.vn;
        paw = jj == 0 ? d.ep_j[ii + (size_t)ni * k] : pw;
      }
      const float zcor1u = ((coru * dts) * 0.25f) * (((x.cv + vdw) + vdwn) + vdn);
      un = ((x.cu + zcor1u) - (zfz * hx) * gzh) - (zcx * zrom1u) * (x.cp - paw);
    }
    // Equation 18
    {
      const float zcy = rot ? dtrdy : dtrdy * mv;
      const float zfz = egdts + 0.25f * (((x.ds0 + x.ds1) + x.cd0) + x.cd1);
      const float zrom1v = hcpd * (x.ts + x.ct);
      float uds = x.us, ude = ue, udes = ues, pas = x.ps;
      if (EDGE) {
        const int im = wm1(ii, ni), jp = wp1(jj, nj);
        uds = ii == 0 ? d.eu_i[jj + (size_t)nj * k] : x.us;
        ude = jj == nj - 1 ? d.eu_j[ii + (size_t)ni * k] : ue;
        udes = jj == nj - 1 ? d.eu_j[im + (size_t)ni * k] : (ii == 0 ? d.eu_i[jp + (size_t)nj * k] : ues);
        pas = ii == 0 ? d.ep_i[jj + (size_t)nj * k] : x.ps;
      }
      const float zcor1v = ((corv * dts) * 0.25f) * (((x.cu + uds) + ude) + udes);
      vnew = ((x.cv - zcor1v) - (zfz * hy) * gzh) - (zcy * zrom1v) * (x.cp - pas);
    }
  };
  auto row = [&](const int i, auto edge) {
    issue(i + kMom2S - 2, qi);   // into the slot of row i-2
    cp_async_wait<kMom2S - 3>();  // rows up to i+1 have landed
    c2 = n2;
    if (i + 1 < i_e) load2(i + 1, n2);
    auto lds2 = [&](int q, int a) { return *reinterpret_cast<const float2*>(&rg[q][a][2 * lane]); };
    const float2 cu = lds2(qc, 0), cv = lds2(qc, 1), ct = lds2(qc, 2), cp = lds2(qc, 3);
    const float2 cd0 = lds2(qc, 4), cd1 = lds2(qc, 5);
    const float2 us = lds2(qb, 0), ts = lds2(qb, 2), ps = lds2(qb, 3), ds0 = lds2(qb, 4), ds1 = lds2(qb, 5);
    const float2 vn = lds2(qn, 1);
    // east neighbours of the second column: the next lane's first
    const float ue1 = __shfl_down_sync(0xffffffffu, cu.x, 1);
    const float ues1 = __shfl_down_sync(0xffffffffu, us.x, 1);
    // west neighbours of the first column: the previous lane's second
    const float vw0 = __shfl_up_sync(0xffffffffu, cv.y, 1);
    const float vwn0 = __shfl_up_sync(0xffffffffu, vn.y, 1);
    const float tw0 = __shfl_up_sync(0xffffffffu, ct.y, 1);
    const float pw0 = __shfl_up_sync(0xffffffffu, cp.y, 1);
    const float dw0w0 = __shfl_up_sync(0xffffffffu, cd0.y, 1);
    const float dw1w0 = __shfl_up_sync(0xffffffffu, cd1.y, 1);
    const Col xa{cu.x, cv.x, ct.x, cp.x, cd0.x, cd1.x, us.x, ts.x, ps.x, ds0.x, ds1.x, vn.x};
    const Col xb{cu.y, cv.y, ct.y, cp.y, cd0.y, cd1.y, us.y, ts.y, ps.y, ds0.y, ds1.y, vn.y};
    float ua = 0.f, va = 0.f, ub = 0.f, vb = 0.f;
    if (out0)
      point(ja, i, xa, vw0, vwn0, tw0, pw0, dw0w0, dw1w0, cu.y, us.y, c2.coru.x, c2.corv.x, c2.hx.x, c2.hy.x,
            c2.mu.x, c2.mv.x, edge, ua, va);
    if (out1)
      point(jb, i, xb, cv.x, vn.x, ct.x, cp.x, cd0.x, cd1.x, ue1, ues1, c2.coru.y, c2.corv.y, c2.hx.y, c2.hy.y,
            c2.mu.y, c2.mv.y, edge, ub, vb);
    const size_t c = (size_t)ja + (size_t)nj * i;
    if (out0 && out1) {
      *reinterpret_cast<float2*>(uo + c) = make_float2(ua, ub);
      *reinterpret_cast<float2*>(vo + c) = make_float2(va, vb);
    } else if (out0) {
      uo[c] = ua;
      vo[c] = va;
    } else if (out1) {
      uo[c + 1] = ub;
      vo[c + 1] = vb;
    }
    qb = qc; qc = qn; qn = nxt(qn); qi = nxt(qi);
  };
  if (interior)
    for (int i = i_s; i < i_e; ++i) row(i, std::false_type());
  else
    for (int i = i_s; i < i_e; ++i) row(i, std::true_type());
  cp_async_wait<0>();  // no copy outlives the kernel
}

__global__ void __launch_bounds__(128, 5) k_momentum_strip2(View<float> d, int R) {
  __shared__ __align__(16) Mom2Slots ring[4];
  b_momentum_strip2(d, blockIdx.x, blockIdx.y, R, ring[threadIdx.x >> 5], threadIdx.x >> 5, 4);
}

// ---- divergence + divdamp as warp strips (:514-597, :853-895, :627-630) ---
// The work of k_sound_div and k_sound_damp in one pass.  One warp per strip
// of kDDJ output columns x R rows of one level k, lanes on columns
// j0-1 .. j0+30.  For each row the lane's point gets s(k) and s(k+1)
// (Equation 10, or the surface values when k is the lowest level) and the
// horizontal divergence zdiv2a (Equation 16) from the pre-damping u, v of
// the current buffer: east neighbours from the lane beside (shuffles),
// north neighbours from the next row, whose v-part is loaded two rows
// ahead.  The damping of row i then takes zdiv2a of the lanes beside and of
// rows i-1, i+1 from registers.  Damped u, v go to the other buffer
// (ubuf[cur^1]) -- the caller flips cur -- so no strip ever reads a value
// another strip has damped; zdiv2a never goes to memory.  The boundary
// lanes and rows store the pre-damping edge values the momentum step reads
// as the stale ud/vd halo (:730-735), as k_sound_div does.
template <class T>
__device__ __forceinline__ void b_divdamp_strip(const View<T>& d, const int bx, const int k, const int R,
                                                const int wid, const int nw) {
  if (d.sur_skip && *d.sur_skip) return;  // the surrogate took this cycle
  const int lane = threadIdx.x & 31;
  const int nj = d.nj, ni = d.ni, kz = d.kz;
  const size_t pl = d.pl;
  const int nsj = (nj + kDDJ - 1) / kDDJ, nsi = (ni + R - 1) / R;
  const int w = bx * nw + wid;
  if (w >= nsj * nsi) return;  // whole warp
  const int sj = w % nsj, si = w / nsj;
  const int jl = sj * kDDJ - 1 + lane;
  const int jj = wrapn(jl, nj);
  const bool out_lane = lane >= 1 && lane <= kDDJ && jl < nj;
  const int i_s = si * R, i_e = min(i_s + R, ni);
  const size_t o = (size_t)k * pl;
  const bool has_up = k > 0, has_dn = k < kz - 1;  // levels k-1 and k+1 exist
  const T* __restrict__ u = d.ubuf[d.cur] + o;
  const T* __restrict__ v = d.vbuf[d.cur] + o;
  T* __restrict__ uo = d.ubuf[d.cur ^ 1] + o;
  T* __restrict__ vo = d.vbuf[d.cur ^ 1] + o;
  const T* __restrict__ rfw = d.rfw + o;
  const T* __restrict__ rfs = d.rfs + o;
  const T* __restrict__ fmz = d.fmz + o;
  const bool rot = d.rotllr;
  const T dtrdx = d.dtrdx, dtrdy = d.dtrdy, dtrdz = d.dtrdz, ddamp2 = d.ddamp2;
  const T cd = d.cdamp[k];
  const T gzk = has_up ? d.gzitak[k] : T(0), gzk1 = has_dn ? d.gzitak[k + 1] : T(0);
  // u-part and v-part of a row of this lane's column
  struct Ur { T uk, um, up, rfw, fmz, hx, mx, rmu, mu, mv, s0; };
  struct Vr { T vk, vm, vp, rfs, rmv, hy; };
  auto load_u = [&](int i, Ur& x) {
    const size_t c = (size_t)jj + (size_t)nj * wrap2(i, ni);
    x.uk = u[c];
    x.um = has_up ? u[c - pl] : T(0);
    x.up = has_dn ? u[c + pl] : T(0);
    x.rfw = rfw[c]; x.fmz = fmz[c]; x.hx = d.hx[c]; x.mu = d.mu[c];
    x.mx = rot ? d.mx[c] : d.mx2[c];
    x.rmu = rot ? T(0) : d.rmu[c];
    x.mv = rot ? T(0) : d.mv[c];
    x.s0 = has_up ? T(0) : d.s[c];  // s at the top level is never computed here
  };
  auto load_v = [&](int i, Vr& x) {
    const size_t c = (size_t)jj + (size_t)nj * wrap2(i, ni);
    x.vk = v[c];
    x.vm = has_up ? v[c - pl] : T(0);
    x.vp = has_dn ? v[c + pl] : T(0);
    x.rfs = rfs[c]; x.rmv = d.rmv[c]; x.hy = d.hy[c];
  };
  // zdiv2a, s(k), s(k+1) of a row from its u-part and the v-parts of the
  // row and the row after (expressions of k_sound_div)
  struct Zr { T z, sk, sk1, ws; };
  auto row_terms = [&](const Ur& a, const Vr& b, const Vr& bn) {
    const T uk_e = __shfl_down_sync(0xffffffffu, a.uk, 1);
    const T um_e = __shfl_down_sync(0xffffffffu, a.um, 1);
    const T up_e = __shfl_down_sync(0xffffffffu, a.up, 1);
    const T rfw_e = __shfl_down_sync(0xffffffffu, a.rfw, 1);
    const T hx_e = __shfl_down_sync(0xffffffffu, a.hx, 1);
    const T rmu_e = __shfl_down_sync(0xffffffffu, a.rmu, 1);
    Zr r;
    if (has_up) {
      const T zuh = prod_add(a.uk + a.um, a.hx, uk_e + um_e, hx_e);
      const T zvh = prod_add(b.vk + b.vm, b.hy, bn.vk + bn.vm, bn.hy);
      r.sk = -((T(0.25) * (zuh + zvh)) * gzk);
    } else {
      r.sk = a.s0;
    }
    if (has_dn) {
      const T zuh = prod_add(a.up + a.uk, a.hx, up_e + uk_e, hx_e);
      const T zvh = prod_add(b.vp + b.vk, b.hy, bn.vp + bn.vk, bn.hy);
      r.sk1 = -((T(0.25) * (zuh + zvh)) * gzk1);
      r.ws = T(0);
    } else {  // surface w(kz+1) and s(kz+1) (:536-549)
      const T zuh = prod_add(a.uk, a.hx, uk_e, hx_e);
      const T zvh = prod_add(b.vk, b.hy, bn.vk, bn.hy);
      r.ws = T(0.5) * (zuh + zvh);
      r.sk1 = -r.ws;
    }
    if (rot) {
      const T du = prod_sub(dtrdx * uk_e, rfw_e, dtrdx * a.uk, a.rfw);
      const T dv = prod_sub((dtrdy * bn.vk) * bn.rfs, bn.rmv, (dtrdy * b.vk) * b.rfs, b.rmv);
      r.z = (a.fmz * a.mx) * (du + dv);
    } else {
      const T du = prod_sub((dtrdx * uk_e) * rmu_e, rfw_e, (dtrdx * a.uk) * a.rmu, a.rfw);
      const T dv = prod_sub((dtrdy * bn.vk) * bn.rmv, bn.rfs, (dtrdy * b.vk) * b.rmv, b.rfs);
      r.z = (a.mx * a.fmz) * (du + dv);
    }
    return r;
  };
  // prologue: zdiv2a of row i_s-1, all terms of row i_s
  Ur ua, ub, un;
  Vr va, vb, vc, vn;
  load_u(i_s - 1, ua); load_v(i_s - 1, va); load_v(i_s, vb);
  load_u(i_s, ub); load_v(i_s + 1, vc);
  const T z_first = row_terms(ua, va, vb).z;
  T z_prev = z_first;
  Zr zcur = row_terms(ub, vb, vc);
  Ur ucur = ub;
  Vr vcur = vb;
  if (i_s + 1 <= i_e) { load_u(i_s + 1, un); load_v(i_s + 2, vn); }
  for (int i = i_s; i < i_e; ++i) {
    // in registers: z(i-1); row i (ucur, vcur, zcur); v-part of row i+1 (vc);
    // in flight: u-part of row i+1 (un), v-part of row i+2 (vn)
    const Ur unext = un;
    const Vr vnext = vn;
    if (i + 2 <= i_e) { load_u(i + 2, un); load_v(i + 3, vn); }
    const Zr znext = row_terms(unext, vc, vnext);  // row i+1
    const T zc = zcur.z;
    const T zw = __shfl_up_sync(0xffffffffu, zc, 1);
    const T ze = __shfl_down_sync(0xffffffffu, zc, 1);
    const T zs = z_prev, zn = znext.z;
    if (out_lane) {
      const int ii = i;
      const size_t c = (size_t)jj + (size_t)nj * ii;
      const T u0 = ucur.uk, v0 = vcur.vk;
      if (has_up) d.s[o + c] = zcur.sk;
      if (!has_dn) {
        d.w[c + (size_t)kz * pl] = zcur.ws;
        d.s[c + (size_t)kz * pl] = -zcur.ws;
      }
      if (jj == 0) d.eu_j[ii + (size_t)ni * k] = u0;
      if (ii == ni - 1) d.eu_i[jj + (size_t)nj * k] = u0;
      if (jj == nj - 1) d.ev_j[ii + (size_t)ni * k] = v0;
      if (ii == 0) d.ev_i[jj + (size_t)nj * k] = v0;
      uo[c] = u0 + ((cd * ucur.mu) * (zc - zw));
      if (rot)
        vo[c] = v0 + cd * (zc - zs);
      else
        vo[c] = v0 + ((cd * ucur.mv) * (zc - zs));
      const T p2d = prod_sub(T(0.125), ((zw + ze) + zs) + zn, T(0.5), zc);
      T zd = zc + ddamp2 * p2d;
      zd = zd + (ucur.fmz * dtrdz) * (zcur.sk - zcur.sk1);
      d.zdiv2b[o + c] = zd;
    }
    z_prev = zc;
    zcur = znext;
    ucur = unext;
    vcur = vc;
    vc = vnext;
  }
}

// (8 blocks per SM with 64 registers measured slower in the full step:
// 2.74 against 2.56 ms per step)
template <class T>
__global__ void __launch_bounds__(128) k_divdamp_strip(View<T> d, int R) {
  b_divdamp_strip<T>(d, blockIdx.x, blockIdx.y, R, threadIdx.x >> 5, 4);
}

template <class T>
__global__ void __launch_bounds__(128, sizeof(T) == 4 ? 8 : 3)
    kb_divdamp_strip(const View<T>* __restrict__ views, const int4* __restrict__ tiles, int R) {
  __shared__ View<T> sv;
  const int4 t = tiles[blockIdx.x];
  copy_view(&sv, views + t.x);
  __syncthreads();
  b_divdamp_strip<T>(sv, t.y, t.z, R, threadIdx.x >> 5, 4);
}

// The same strips over NL consecutive levels k0 .. k0+NL-1 per warp
// (kmarch bit 512, with 16).  The levels of a strip share each row's loads
// of u and v at the levels between them (NL+2 levels instead of 3 NL), its
// 2-D metric fields, the east shuffles of those values and the address
// arithmetic, and s(k) at each inner level is formed once instead of
// twice (as s(k+1) of the level above and s(k) of the level below: the
// same sums in the same order, so the same bits).  Per level the
// arithmetic is that of b_divdamp_strip.
template <class T, int NL>
__device__ __forceinline__ void b_divdamp_strip_nl(const View<T>& d, const int bx, const int kp, const int R,
                                                   const int wid, const int nw) {
  if (d.sur_skip && *d.sur_skip) return;  // the surrogate took this cycle
  const int lane = threadIdx.x & 31;
  const int nj = d.nj, ni = d.ni, kz = d.kz;
  const unsigned pl = (unsigned)d.pl;  // 32-bit element offsets: a field holds at most 2^31 points
  const int nsj = (nj + kDDJ - 1) / kDDJ, nsi = (ni + R - 1) / R;
  const int w = bx * nw + wid;
  if (w >= nsj * nsi) return;  // whole warp
  const int sj = w % nsj, si = w / nsj;
  const int jl = sj * kDDJ - 1 + lane;
  const int jj = wrapn(jl, nj);
  const bool out_lane = lane >= 1 && lane <= kDDJ && jl < nj;
  const int i_s = si * R, i_e = min(i_s + R, ni);
  const int k0 = kp * NL;
  const T* __restrict__ u = d.ubuf[d.cur];
  const T* __restrict__ v = d.vbuf[d.cur];
  T* __restrict__ uo = d.ubuf[d.cur ^ 1];
  T* __restrict__ vo = d.vbuf[d.cur ^ 1];
  const bool rot = d.rotllr;
  const T dtrdx = d.dtrdx, dtrdy = d.dtrdy, dtrdz = d.dtrdz, ddamp2 = d.ddamp2;
  // level k0-1+l, l = 0 .. NL+1, inside the domain; level k0+l, l < NL
  bool lin[NL + 2];
#pragma unroll
  for (int l = 0; l < NL + 2; ++l) lin[l] = k0 - 1 + l >= 0 && k0 - 1 + l < kz;
  T cd[NL], gz[NL + 1];
#pragma unroll
  for (int l = 0; l < NL; ++l) cd[l] = lin[l + 1] ? d.cdamp[k0 + l] : T(0);
#pragma unroll
  for (int l = 0; l <= NL; ++l) gz[l] = (k0 + l >= 1 && k0 + l <= kz - 1) ? d.gzitak[k0 + l] : T(0);
  // u-part and v-part of a row of this lane's column: u, v at the levels
  // k0-1 .. k0+NL, rfw, fmz, rfs at k0 .. k0+NL-1
  struct Ur { T u[NL + 2], rfw[NL], fmz[NL]; T hx, mx, rmu, mu, mv, s0; };
  struct Vr { T v[NL + 2], rfs[NL]; T rmv, hy; };
  auto load_u = [&](int i, Ur& x) {
    const unsigned c = (unsigned)jj + (unsigned)nj * (unsigned)wrap2(i, ni);
#pragma unroll
    for (int l = 0; l < NL + 2; ++l) x.u[l] = lin[l] ? u[c + (unsigned)(k0 - 1 + l) * pl] : T(0);
#pragma unroll
    for (int l = 0; l < NL; ++l) {
      x.rfw[l] = lin[l + 1] ? d.rfw[c + (unsigned)(k0 + l) * pl] : T(0);
      x.fmz[l] = lin[l + 1] ? d.fmz[c + (unsigned)(k0 + l) * pl] : T(0);
    }
    x.hx = d.hx[c]; x.mu = d.mu[c];
    x.mx = rot ? d.mx[c] : d.mx2[c];
    x.rmu = rot ? T(0) : d.rmu[c];
    x.mv = rot ? T(0) : d.mv[c];
    x.s0 = k0 == 0 ? d.s[c] : T(0);  // s at the top level is never computed here
  };
  auto load_v = [&](int i, Vr& x) {
    const unsigned c = (unsigned)jj + (unsigned)nj * (unsigned)wrap2(i, ni);
#pragma unroll
    for (int l = 0; l < NL + 2; ++l) x.v[l] = lin[l] ? v[c + (unsigned)(k0 - 1 + l) * pl] : T(0);
#pragma unroll
    for (int l = 0; l < NL; ++l) x.rfs[l] = lin[l + 1] ? d.rfs[c + (unsigned)(k0 + l) * pl] : T(0);
    x.rmv = d.rmv[c]; x.hy = d.hy[c];
  };
  // zdiv2a of the levels, s at k0 .. k0+NL (the surface value -ws at kz),
  // ws when the lowest level is kz-1 (expressions of k_sound_div)
  struct Zr { T z[NL], s[NL + 1], ws; };
  auto row_terms = [&](const Ur& a, const Vr& b, const Vr& bn) {
    T ue[NL + 2];
#pragma unroll
    for (int l = 0; l < NL + 2; ++l) ue[l] = __shfl_down_sync(0xffffffffu, a.u[l], 1);
    T rfw_e[NL];
#pragma unroll
    for (int l = 0; l < NL; ++l) rfw_e[l] = __shfl_down_sync(0xffffffffu, a.rfw[l], 1);
    const T hx_e = __shfl_down_sync(0xffffffffu, a.hx, 1);
    const T rmu_e = __shfl_down_sync(0xffffffffu, a.rmu, 1);
    Zr r;
    r.ws = T(0);
#pragma unroll
    for (int l = 0; l <= NL; ++l) {
      const int kk = k0 + l;  // s(kk) from the levels kk-1 (index l) and kk (index l+1)
      if (kk == 0) {
        r.s[l] = a.s0;
      } else if (kk <= kz - 1) {
        const T zuh = prod_add(a.u[l + 1] + a.u[l], a.hx, ue[l + 1] + ue[l], hx_e);
        const T zvh = prod_add(b.v[l + 1] + b.v[l], b.hy, bn.v[l + 1] + bn.v[l], bn.hy);
        r.s[l] = -((T(0.25) * (zuh + zvh)) * gz[l]);
      } else if (kk == kz) {  // surface w(kz+1) and s(kz+1) (:536-549)
        const T zuh = prod_add(a.u[l], a.hx, ue[l], hx_e);
        const T zvh = prod_add(b.v[l], b.hy, bn.v[l], bn.hy);
        r.ws = T(0.5) * (zuh + zvh);
        r.s[l] = -r.ws;
      } else {
        r.s[l] = T(0);
      }
    }
#pragma unroll
    for (int l = 0; l < NL; ++l) {
      const T uk = a.u[l + 1], uk_e = ue[l + 1];
      if (rot) {
        const T du = prod_sub(dtrdx * uk_e, rfw_e[l], dtrdx * uk, a.rfw[l]);
        const T dv = prod_sub((dtrdy * bn.v[l + 1]) * bn.rfs[l], bn.rmv, (dtrdy * b.v[l + 1]) * b.rfs[l], b.rmv);
        r.z[l] = (a.fmz[l] * a.mx) * (du + dv);
      } else {
        const T du = prod_sub((dtrdx * uk_e) * rmu_e, rfw_e[l], (dtrdx * uk) * a.rmu, a.rfw[l]);
        const T dv = prod_sub((dtrdy * bn.v[l + 1]) * bn.rmv, bn.rfs[l], (dtrdy * b.v[l + 1]) * b.rmv, b.rfs[l]);
        r.z[l] = (a.mx * a.fmz[l]) * (du + dv);
      }
    }
    return r;
  };
  // prologue: zdiv2a of row i_s-1, all terms of row i_s
  Ur ua, ub, un;
  Vr va, vb, vc, vn;
  load_u(i_s - 1, ua); load_v(i_s - 1, va); load_v(i_s, vb);
  load_u(i_s, ub); load_v(i_s + 1, vc);
  const Zr zfirst = row_terms(ua, va, vb);
  T z_prev[NL];
#pragma unroll
  for (int l = 0; l < NL; ++l) z_prev[l] = zfirst.z[l];
  Zr zcur = row_terms(ub, vb, vc);
  Ur ucur = ub;
  Vr vcur = vb;
  if (i_s + 1 <= i_e) { load_u(i_s + 1, un); load_v(i_s + 2, vn); }
  for (int i = i_s; i < i_e; ++i) {
    // in registers: z(i-1); row i (ucur, vcur, zcur); v-part of row i+1 (vc);
    // in flight: u-part of row i+1 (un), v-part of row i+2 (vn)
    const Ur unext = un;
    const Vr vnext = vn;
    if (i + 2 <= i_e) { load_u(i + 2, un); load_v(i + 3, vn); }
    const Zr znext = row_terms(unext, vc, vnext);  // row i+1
    const unsigned c = (unsigned)jj + (unsigned)nj * (unsigned)i;
#pragma unroll
    for (int l = 0; l < NL; ++l) {
      const int k = k0 + l;
      const T zc = zcur.z[l];
      const T zw = __shfl_up_sync(0xffffffffu, zc, 1);
      const T ze = __shfl_down_sync(0xffffffffu, zc, 1);
      const T zs = z_prev[l], zn = znext.z[l];
      if (out_lane && k < kz) {
        const unsigned o = (unsigned)k * pl;
        const T u0 = ucur.u[l + 1], v0 = vcur.v[l + 1];
        if (k > 0) d.s[o + c] = zcur.s[l];
        if (k == kz - 1) {
          d.w[c + (unsigned)kz * pl] = zcur.ws;
          d.s[c + (unsigned)kz * pl] = -zcur.ws;
        }
        if (jj == 0) d.eu_j[i + (size_t)ni * k] = u0;
        if (i == ni - 1) d.eu_i[jj + (size_t)nj * k] = u0;
        if (jj == nj - 1) d.ev_j[i + (size_t)ni * k] = v0;
        if (i == 0) d.ev_i[jj + (size_t)nj * k] = v0;
        uo[o + c] = u0 + ((cd[l] * ucur.mu) * (zc - zw));
        if (rot)
          vo[o + c] = v0 + cd[l] * (zc - zs);
        else
          vo[o + c] = v0 + ((cd[l] * ucur.mv) * (zc - zs));
        const T p2d = prod_sub(T(0.125), ((zw + ze) + zs) + zn, T(0.5), zc);
        T zd = zc + ddamp2 * p2d;
        zd = zd + (ucur.fmz[l] * dtrdz) * (zcur.s[l] - zcur.s[l + 1]);
        d.zdiv2b[o + c] = zd;
      }
      z_prev[l] = zc;
    }
    zcur = znext;
    ucur = unext;
    vcur = vc;
    vc = vnext;
  }
}

// 4 blocks per SM (FP32: 122 registers): 0.167 ms per launch at
// 512 x 512 x 60 against 0.171 for the one-level strips; 5 blocks (96
// registers, spills) 0.180
template <class T>
__global__ void __launch_bounds__(128, 4) k_divdamp_strip_nl(View<T> d, int R) {
  b_divdamp_strip_nl<T, kDDLevels>(d, blockIdx.x, blockIdx.y, R, threadIdx.x >> 5, 4);
}
template <class T>
__global__ void __launch_bounds__(128, 4)
    kb_divdamp_strip_nl(const View<T>* __restrict__ views, const int4* __restrict__ tiles, int R) {
  __shared__ View<T> sv;
  const int4 t = tiles[blockIdx.x];
  copy_view(&sv, views + t.x);
  __syncthreads();
  b_divdamp_strip_nl<T, kDDLevels>(sv, t.y, t.z, R, threadIdx.x >> 5, 4);
}

// ---- advection: vertical WAF, two passes at dt/2 (:966-1073) ------------
// wfw(k+1) of one pass from x(max(k-1,1)), x(k), x(k+1), x(min(k+2,kz))
template <class T>
__device__ __forceinline__ T waf_vflux(T s_k1, T dtrdz, T xm, T x0, T x1, T x2) {
  const T zamu = s_k1 * dtrdz;
  T is, num;
  if (zamu >= T(0)) {
    is = T(1); num = x1 - x2;  // k1 = k+1, k1p1 = min(k+2, kz)
  } else {
    is = T(-1); num = xm - x0;  // k1 = max(k-1, 1), k1p1 = k
  }
  const T r = qdiv(num, safeden(x0 - x1));
  const T bb = superbee(r);
  const T zphi = (is + zamu * bb) - is * bb;
  return (T(0.5) * s_k1) * ((T(1) + zphi) * x1 + (T(1) - zphi) * x0);
}
// FP32 storage: the same flux, rearranged for fewer instructions (these
// kernels are bound by the ALU pipe, not HBM): superbee as
// max(sat(2r), min(r, 2)), phi = is + bb (zamu - is), and
// (1+phi) x1 + (1-phi) x0 = (x1 + x0) - phi (x0 - x1)
template <>
__device__ __forceinline__ float waf_vflux<float>(float s_k1, float dtrdz, float xm, float x0, float x1, float x2) {
  const float zamu = s_k1 * dtrdz;
  const bool pos = zamu >= 0.f;
  const float d = x0 - x1;
  const float den = copysignf(fmaxf(fabsf(d), (float)kMinden), d);
  const float r = __fdividef(pos ? x1 - x2 : xm - x0, den);
  const float bb = fmaxf(__saturatef(2.f * r), fminf(r, 2.f));
  const float is = pos ? 1.f : -1.f;
  const float zphi = fmaf(bb, zamu - is, is);
  return (0.5f * s_k1) * fmaf(-zphi, d, x1 + x0);
}

// One thread per column and F fields (F = 1, 2, 5 or 10: the tuned
// View::vfields).  Both passes stream k in registers: pass 1 yields wz1(t)
// at step t, pass 2 consumes it two levels later, so the intermediate field
// never leaves the SM.  The fields of a thread share the loads of s, wafu,
// wafd and the velocity-only terms of the fluxes (Courant number, its sign,
// s/2, the metric term of the update), which the compiler computes once.
// The grid puts the field group fastest, so the groups of one column tile
// run together and share the s / metric loads through L2.
// G >= 0: the thread's field group holds some of fields 2, 3, 4 (ux, vx,
// wx), which are formed here from the staggered winds -- the fourth-order
// averages of :1327-1341 and :1389-1417, two-point at the bottom and top
// levels of wx -- and stored for the horizontal pass, which reads them.
// Each level is formed once, in order, with its store; the clamped repeats
// at the bottom reuse the last level.  G = -1: a group of read fields only.
template <class T, int F, int G>
__device__ __forceinline__ void b_waf_vertical_g(const View<T>& d, const int g, const int jj, const int ii) {
  const int nj = d.nj, ni = d.ni, kz = d.kz;
  // element offsets fit in 32 bits (a field holds at most 2^31 points)
  const unsigned pl = (unsigned)d.pl;
  const unsigned c = (unsigned)jj + (unsigned)nj * (unsigned)ii;
  const T* src[F];
  T* wz[F];
#pragma unroll
  for (int u = 0; u < F; ++u) {
    src[u] = d.fset[d.fcur][g * F + u];
    wz[u] = d.wz + (size_t)(g * F + u) * d.pl * kz;
  }
  const T* __restrict__ s = d.s;
  const T* __restrict__ wafu = d.wafu;
  const T* __restrict__ wafd = d.wafd;
  const T dtrdz = d.dtrdz_a;
  auto xval = [&](const int u, const int kk) -> T {
    const unsigned o = (unsigned)kk * pl;
    if constexpr (G < 0) {
      return src[u][c + o];
    } else {
      const int f = G * F + u;
      T x;
      if (f == 2) {
        const T* __restrict__ us = d.ubuf[d.cur] + (o + (unsigned)nj * ii);
        x = T(0.5625) * (us[wp1(jj, nj)] + us[jj]) - T(0.0625) * (us[wp2(jj, nj)] + us[wm1(jj, nj)]);
      } else if (f == 3) {
        const T* __restrict__ vs = d.vbuf[d.cur] + (o + jj);
        x = T(0.5625) * (vs[(unsigned)nj * wp1(ii, ni)] + vs[(unsigned)nj * ii]) -
            T(0.0625) * (vs[(unsigned)nj * wp2(ii, ni)] + vs[(unsigned)nj * wm1(ii, ni)]);
      } else if (f == 4) {
        const T* __restrict__ w = d.w + c;
        if (kk == 0)
          x = T(0.5) * (w[pl] + w[0]);
        else if (kk == kz - 1)
          x = T(0.5) * (w[(unsigned)kz * pl] + w[(unsigned)(kz - 1) * pl]);
        else
          x = T(0.5625) * (w[(kk + 1) * pl] + w[kk * pl]) - T(0.0625) * (w[(kk + 2) * pl] + w[(kk - 1) * pl]);
      } else {
        return src[u][c + o];
      }
      const_cast<T*>(src[u])[c + o] = x;
      return x;
    }
  };
  T xa[F], xb[F], xc[F];               // pass-1 window x(t-1), x(t), x(t+1)
  T wfw1[F], wfw2[F];                  // wfw1(t), wfw2(m)
  T y0[F], y1[F], y2[F], y3[F];        // wz1(t-3 .. t)
#pragma unroll
  for (int u = 0; u < F; ++u) {
    xa[u] = xval(u, 0); xb[u] = xa[u]; xc[u] = kz > 1 ? xval(u, 1) : xa[u];
    wfw1[u] = T(0); wfw2[u] = T(0);
    y0[u] = T(0); y1[u] = T(0); y2[u] = T(0); y3[u] = T(0);
  }
  T sA = T(0), sB = T(0), sC = s[c], sD;    // s(t-2 .. t+1)
  T uA = T(0), uB = T(0), dA = T(0), dB = T(0);  // wafu/wafd at t-2, t-1
  // one step t of both passes; FAST: 4 <= t <= kz-2, where no boundary
  // case applies (t2 = t+2, both fluxes exist, ym = y0), so the tests drop
  auto step = [&](const int t, auto fast) {
    constexpr bool FAST = decltype(fast)::value;
    T uC = T(0), dC = T(0);
    sD = T(0);
    const int m = t - 2;
    if (FAST || t <= kz) {
      sD = s[c + (unsigned)t * pl];
      uC = wafu[c + (unsigned)(t - 1) * pl];
      dC = wafd[c + (unsigned)(t - 1) * pl];
    }
    const int t2 = FAST ? t + 2 : (t + 2 <= kz ? t + 2 : kz);
#pragma unroll
    for (int u = 0; u < F; ++u) {
      T w1 = y3[u];
      if (FAST || t <= kz) {
        const T xd = (FAST || t + 2 <= kz) ? xval(u, t2 - 1) : xc[u];  // x(min(t+2, kz))
        const T wfw1n = (FAST || t <= kz - 1) ? waf_vflux(sD, dtrdz, xa[u], xb[u], xc[u], xd) : T(0);
        w1 = ((xb[u] - wfw1[u] * uC) + wfw1n * dC) + (sC * uC - sD * dC) * xb[u];
        xa[u] = xb[u]; xb[u] = xc[u]; xc[u] = xd; wfw1[u] = wfw1n;
      }
      y0[u] = y1[u]; y1[u] = y2[u]; y2[u] = y3[u]; y3[u] = w1;  // for t > kz, wz1 stays clamped at wz1(kz)
      if (FAST || m >= 1) {
        const T ym = (!FAST && m == 1) ? y1[u] : y0[u];
        const T wfw2n = (FAST || m <= kz - 1) ? waf_vflux(sB, dtrdz, ym, y1[u], y2[u], y3[u]) : T(0);
        wz[u][c + (unsigned)(m - 1) * pl] = ((y1[u] - wfw2[u] * uA) + wfw2n * dA) + (sA * uA - sB * dA) * y1[u];
        wfw2[u] = wfw2n;
      }
    }
    sA = sB; sB = sC; sC = sD;
    uA = uB; uB = uC; dA = dB; dB = dC;
  };
  const int tf = kz - 2 >= 4 ? kz - 2 : 3;  // last step of the fast range
  for (int t = 1; t <= 3; ++t) step(t, std::false_type());
  for (int t = 4; t <= tf; ++t) step(t, std::true_type());
  for (int t = tf + 1; t <= kz + 2; ++t) step(t, std::false_type());
}

template <class T, int F>
__device__ __forceinline__ void b_waf_vertical(const View<T>& d, const int bx, const int by, const int bz) {
  constexpr int NG = kNumAdvected / F;
  const int g = bx % NG;
  const int tj = bx / NG;
  const int jj = tj * kColBX + threadIdx.x;
  const int ii = by * kColBY + threadIdx.y;
  if (jj >= d.nj || ii >= d.ni) return;
  // the groups holding fields 2..4 (block-uniform branch)
  if constexpr (F == 1) {
    if (g == 2) b_waf_vertical_g<T, 1, 2>(d, g, jj, ii);
    else if (g == 3) b_waf_vertical_g<T, 1, 3>(d, g, jj, ii);
    else if (g == 4) b_waf_vertical_g<T, 1, 4>(d, g, jj, ii);
    else b_waf_vertical_g<T, 1, -1>(d, g, jj, ii);
  } else if constexpr (F == 2) {
    if (g == 1) b_waf_vertical_g<T, 2, 1>(d, g, jj, ii);
    else if (g == 2) b_waf_vertical_g<T, 2, 2>(d, g, jj, ii);
    else b_waf_vertical_g<T, 2, -1>(d, g, jj, ii);
  } else if constexpr (F == 5) {
    if (g == 0) b_waf_vertical_g<T, 5, 0>(d, g, jj, ii);
    else b_waf_vertical_g<T, 5, -1>(d, g, jj, ii);
  } else {
    b_waf_vertical_g<T, F, 0>(d, g, jj, ii);
  }
}

// Blocks per SM by bulk type and fields per thread.  FP32, one field per
// thread: 12 (40 registers; with 32-bit element offsets about 50 bytes
// spilled, 128 with 64-bit ones): 1.69 ms per step at 512 x 512 x 60
// (1.88 with 64-bit offsets), against 1.75 at 13 to 16 blocks, 1.76 at 10
// (48 registers) and 2.00 at 9 (56 registers, no spills); the other
// variants keep the occupancy of their unconstrained register counts.
template <class T, int F>
constexpr int vert_min_blocks() {
  if (sizeof(T) == 4) return F == 1 ? 12 : F == 2 ? 9 : F == 5 ? 5 : 3;
  return F == 1 ? 6 : F == 2 ? 4 : F == 5 ? 2 : 1;
}

template <class T, int F>
__global__ void __launch_bounds__(kColBX* kColBY, vert_min_blocks<T, F>()) k_waf_vertical(View<T> d) {
  b_waf_vertical<T, F>(d, blockIdx.x, blockIdx.y, blockIdx.z);
}

template <class T, int F>
__global__ void __launch_bounds__(kColBX* kColBY, vert_min_blocks<T, F>())
    kb_waf_vertical(const View<T>* __restrict__ views, const int4* __restrict__ tiles) {
  __shared__ View<T> sv;
  const int4 t = tiles[blockIdx.x];
  copy_view(&sv, views + t.x);
  __syncthreads();
  b_waf_vertical<T, F>(sv, t.y, t.z, t.w);
}

// ---- advection: meridional + zonal WAF (:1075-1187) ----------------------
// Block = 32 (j) x 8 (i) output points of kHzLevels consecutive levels, ten
// fields per level.  Per field: the wz tile with a 2-point halo in both
// directions and the pp tile go to shared memory; the meridional fluxes and
// p0 are formed for the 36-wide strip the zonal step needs, then the zonal
// fluxes and the new pp.  p0 never leaves the SM.  The next field's tiles
// travel in registers while the current one is computed.  The result goes to
// the other field buffer (dst): neighbouring blocks still read the old pp at
// their halo columns.  The wrapped (periodic) tile offsets are computed once
// per block and reused for every level and field; d.hz_levels (levels per
// block) is picked by the autotuner (moloch_gpu_autotune).

// WAF flux between cells m1 and x0 (limiter from m2, p1), the reference's
// expression (:1091-1106, :1148-1163)
template <class T>
__device__ __forceinline__ T waf_hflux(T zamu, T m2, T m1, T x0, T p1) {
  T is, num;
  if (zamu > T(0)) {
    is = T(1); num = m1 - m2;   // ih = i-1, ihm1 = i-2
  } else {
    is = T(-1); num = p1 - x0;  // ih = i+1, ihm1 = i
  }
  const T rr = qdiv(num, safeden(x0 - m1));
  const T bb = superbee(rr);
  const T zphi = (is + zamu * bb) - is * bb;
  return (T(1) + zphi) * m1 + (T(1) - zphi) * x0;
}
// FP32 storage: rearranged as waf_vflux<float>
template <>
__device__ __forceinline__ float waf_hflux<float>(float zamu, float m2, float m1, float x0, float p1) {
  const bool pos = zamu > 0.f;
  const float d = x0 - m1;
  const float den = copysignf(fmaxf(fabsf(d), (float)kMinden), d);
  const float r = __fdividef(pos ? m1 - m2 : p1 - x0, den);
  const float bb = fmaxf(__saturatef(2.f * r), fminf(r, 2.f));
  const float is = pos ? 1.f : -1.f;
  const float zphi = fmaf(bb, zamu - is, is);
  return fmaf(zphi, -d, m1 + x0);
}

template <class T>
__device__ __forceinline__ void b_waf_horizontal(const View<T>& d, const int bx, const int by, const int bz) {
  constexpr int TJ = 32, TI = 8, HJ = TJ + 4, HI = TI + 4;
  constexpr int NW = HI * HJ, NP = TI * HJ, NM = (TI + 1) * HJ, NZ = TI * (TJ + 1);
  // flat row-major tiles: a work item's linear number q is its own index
  __shared__ T sw[2][NW];  // wz, rows i0-2 .. i0+TI+1, cols j0-2 .. j0+TJ+1
  __shared__ T sp[2][NP];  // pp (old), rows i0 .., cols j0-2 ..
  __shared__ T smf[NM];    // meridional fluxes at rows i0 .. i0+TI
  __shared__ T sp0[NP];    // p0
  __shared__ T szf[NZ];    // zonal fluxes at cols j0 .. j0+TJ
  const int tx = threadIdx.x, ty = threadIdx.y, tid = tx + 32 * ty;
  const int nj = d.nj, ni = d.ni, kz = d.kz, pl = d.pl;
  const int j0 = bx * TJ, i0 = by * TI;
  const int k0 = bz * d.hz_levels;
  const int k1 = min(k0 + d.hz_levels, kz);
  const T* __restrict__ u = d.ubuf[d.cur];
  const T* __restrict__ v = d.vbuf[d.cur];
  const T dtrdx = d.dtrdx_a, dtrdy = d.dtrdy_a;
  const int rot = d.rotllr;

  // ---- per block: wrapped offsets (valid for every level) and map factors
  int woff[2], poff[2], pnoff[2], zoffg[2], zoff[2];
  T mrm[2], prs[2], prn[2], pmx[2], zm[2];
  for (int n = 0; n < 2; ++n) {
    const int q = tid + 256 * n;
    const int jq = wrapn(j0 - 2 + q % HJ, nj);
    woff[n] = q < NW ? jq + nj * wrapn(i0 - 2 + q / HJ, ni) : 0;
    const int iq = wrapn(i0 + q / HJ, ni);  // meridional flux rows and p0 rows
    poff[n] = q < NM ? jq + nj * iq : 0;
    pnoff[n] = q < NP ? jq + nj * wp1(iq, ni) : 0;
    const int r = q / (TJ + 1), x = q % (TJ + 1);
    zoff[n] = q < NZ ? r * HJ + x : 0;
    zoffg[n] = q < NZ ? wrapn(j0 + x, nj) + nj * wrapn(i0 + r, ni) : 0;
  }
  const int jo = j0 + tx, io = i0 + ty;
  const bool ook = jo < nj && io < ni;
  const int co = ook ? jo + nj * io : 0;
  const int coe = ook ? wp1(jo, nj) + nj * io : 0;
  const int op0 = ty * HJ + tx + 2, ozf = ty * (TJ + 1) + tx;

  // raw per-level inputs (velocities, metric factors), loaded one level ahead
  T rv[2], rwn[2], rws[2], rvn[2], ru[2], rwe = T(0), rww = T(0), ruw = T(0), rue = T(0);
  auto fetch_level = [&](int k) {
    const size_t ko = (size_t)k * pl;
    for (int n = 0; n < 2; ++n) {
      const int q = tid + 256 * n;
      rv[n] = q < NM ? v[ko + poff[n]] : T(0);
      rwn[n] = q < NP ? d.wafn[ko + poff[n]] : T(0);
      rws[n] = q < NP ? d.wafs[ko + poff[n]] : T(0);
      rvn[n] = q < NP ? v[ko + pnoff[n]] : T(0);
      ru[n] = q < NZ ? u[ko + zoffg[n]] : T(0);
    }
    rwe = d.wafe[ko + co]; rww = d.wafw[ko + co];
    ruw = u[ko + co]; rue = u[ko + coe];
  };
  T rw[2], rp[2];
  auto fetch = [&](int k, int f) {
    const T* __restrict__ wzf = d.wz + ((size_t)f * kz + k) * pl;
    const T* __restrict__ ppf = d.fset[d.fcur][f] + (size_t)k * pl;
    for (int n = 0; n < 2; ++n) {
      const int q = tid + 256 * n;
      rw[n] = q < NW ? wzf[woff[n]] : T(0);
      rp[n] = q < NP ? ppf[poff[n]] : T(0);
    }
  };
  auto stash = [&](int b) {
    for (int n = 0; n < 2; ++n) {
      const int q = tid + 256 * n;
      if (q < NW) sw[b][q] = rw[n];
      if (q < NP) sp[b][q] = rp[n];
    }
  };
  fetch_level(k0);
  fetch(k0, 0);
  for (int n = 0; n < 2; ++n) {
    const int q = tid + 256 * n;
    mrm[n] = q < NM ? d.rmv[poff[n]] : T(1);
    prs[n] = q < NP ? d.rmv[poff[n]] : T(1);
    prn[n] = q < NP ? d.rmv[pnoff[n]] : T(1);
    pmx[n] = q < NP ? d.mx2[poff[n]] : T(0);
    zm[n] = q < NZ ? (rot ? d.mu[zoffg[n]] : d.rmu[zoffg[n]]) : T(0);
  }
  const T ormw = d.rmu[co], orme = d.rmu[coe], omx = d.mx2[co];
  stash(0);
  __syncthreads();
  int b = 0;
  for (int k = k0; k < k1; ++k) {
    const size_t ko = (size_t)k * pl;
    T mz[2], mfac[2], pn[2], ps_[2], pdv[2], zz[2], zfac[2];
    for (int n = 0; n < 2; ++n) {
      const T vv = rv[n];
      mz[n] = rot ? vv * dtrdy : (vv * mrm[n]) * dtrdy;
      mfac[n] = rot ? T(0.5) * vv : (T(0.5) * vv) * mrm[n];
      const T zrfmn = rwn[n], zrfms = rws[n], vs = rv[n], vn = rvn[n];
      pn[n] = zrfmn; ps_[n] = zrfms;
      pdv[n] = rot ? (vn * zrfmn - vs * zrfms) : ((vn * prn[n]) * zrfmn - (vs * prs[n]) * zrfms);
      const T uu = ru[n];
      zz[n] = (uu * zm[n]) * dtrdx;
      zfac[n] = rot ? T(0.5) * uu : (T(0.5) * uu) * zm[n];
    }
    const T oe = rwe, ow = rww;
    const T odv = rot ? (rue * oe - ruw * ow) : ((rue * orme) * oe - (ruw * ormw) * ow);
    for (int f = 0; f < kNumAdvected; ++f) {
      const T* __restrict__ W = sw[b];
      const T* __restrict__ P = sp[b];
      const bool next_field = f + 1 < kNumAdvected;
      const bool next_level = !next_field && k + 1 < k1;
      if (next_field) fetch(k, f + 1);
      if (next_level) {
        fetch(k + 1, 0);
        fetch_level(k + 1);
      }
      for (int n = 0; n < 2; ++n) {  // zpby between tile rows r+1 and r+2 (flat: q+HJ, q+2HJ)
        const int q = tid + 256 * n;
        if (q < NM)
          smf[q] = mfac[n] * waf_hflux(mz[n], W[q], W[q + HJ], W[q + 2 * HJ], W[q + 3 * HJ]);
      }
      __syncthreads();
      for (int n = 0; n < 2; ++n) {  // p0 (:1113-1131, :1222-1240)
        const int q = tid + 256 * n;
        if (q < NP) {
          const T zdv = pdv[n] * P[q];
          const T wc = W[q + 2 * HJ];
          sp0[q] = rot ? ((wc + smf[q] * ps_[n]) - smf[q + HJ] * pn[n]) + zdv
                       : wc + pmx[n] * (((smf[q] * ps_[n]) - smf[q + HJ] * pn[n]) + zdv);
        }
      }
      __syncthreads();
      for (int n = 0; n < 2; ++n) {  // zpbw between sp0 cols x+1 and x+2
        const int q = tid + 256 * n;
        if (q < NZ) {
          const int z0 = zoff[n];
          szf[q] = zfac[n] * waf_hflux(zz[n], sp0[z0], sp0[z0 + 1], sp0[z0 + 2], sp0[z0 + 3]);
        }
      }
      __syncthreads();
      if (ook) {  // new pp (:1173-1187, :1283-1297)
        const T p0 = sp0[op0];
        const T zdv = odv * P[op0];
        const T out = rot ? ((p0 + szf[ozf] * ow) - szf[ozf + 1] * oe) + zdv
                          : p0 + omx * (((szf[ozf] * ow) - szf[ozf + 1] * oe) + zdv);
        d.fset[d.fcur ^ 1][f][ko + co] = out;
      }
      if (next_field || next_level) stash(b ^ 1);  // the other buffer was last read two fields ago
      b ^= 1;
      __syncthreads();
    }
  }
}

template <class T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 2) k_waf_horizontal(View<T> d) {
  b_waf_horizontal<T>(d, blockIdx.x, blockIdx.y, blockIdx.z);
}

template <class T>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 3 : 2)
    kb_waf_horizontal(const View<T>* __restrict__ views, const int4* __restrict__ tiles) {
  __shared__ View<T> sv;
  const int4 t = tiles[blockIdx.x];
  copy_view(&sv, views + t.x);
  __syncthreads();
  b_waf_horizontal<T>(sv, t.y, t.z, t.w);
}

// ---- advection: horizontal WAF as warp strips (:1075-1187) ---------------
// One warp per strip of 28 output columns x R rows of one level (R =
// d.hz_levels, 16..64), 32 lanes on columns j0-2 .. j0+29.  Each lane marches
// down its own column: the wz values of rows i-1 .. i+2 and the meridional
// flux of the face above the row stay in registers, p0 of the row is formed
// in the lane, and the zonal fluxes take their p0 neighbours from the lanes
// beside it (warp shuffles).  No shared memory and no barriers.  Fields are
// processed G at a time so the per-row velocities and metric factors are
// loaded once per group.  The result goes to the other field buffer.
constexpr int kStripJ = 28;
template <class T> struct StripG { static constexpr int G = 10; };
template <> struct StripG<double> { static constexpr int G = 5; };

template <class T>
__device__ __forceinline__ void b_waf_hstrip(const View<T>& d, const int bx, const int k) {
  constexpr int G = StripG<T>::G;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nj = d.nj, ni = d.ni, pl = d.pl, kz = d.kz;
  const int R = d.hz_levels;
  const int nsj = (nj + kStripJ - 1) / kStripJ, nsi = (ni + R - 1) / R;
  const int w = bx * (blockDim.x >> 5) + wid;
  if (w >= nsj * nsi) return;  // whole warp
  const int sj = w % nsj, si = w / nsj;
  const int j0 = sj * kStripJ;
  const int jl = j0 - 2 + lane;  // this lane's column before wrapping
  const int j = wrapn(jl, nj);
  const bool out_lane = lane >= 2 && lane < 2 + kStripJ && jl < nj;
  const int i_s = si * R, i_e = min(i_s + R, ni);
  const T* __restrict__ u = d.ubuf[d.cur] + (size_t)k * pl;
  const T* __restrict__ v = d.vbuf[d.cur] + (size_t)k * pl;
  const T* __restrict__ wn_ = d.wafn + (size_t)k * pl;
  const T* __restrict__ ws_ = d.wafs + (size_t)k * pl;
  const T* __restrict__ we_ = d.wafe + (size_t)k * pl;
  const T* __restrict__ ww_ = d.wafw + (size_t)k * pl;
  const T dtrdx = d.dtrdx_a, dtrdy = d.dtrdy_a;
  const bool rot = d.rotllr;
  auto row = [&](int i) { return (size_t)j + (size_t)nj * wrap2(i, ni); };

  for (int g0 = 0; g0 < kNumAdvected; g0 += G) {
    const int ng = min(G, kNumAdvected - g0);
    const T* wz[G];
    const T* pp[G];
    T* out[G];
    T wm1_[G], w0_[G], wp1_[G], fl_[G];  // wz(i-1), wz(i), wz(i+1), flux of face i
#pragma unroll
    for (int g = 0; g < G; ++g) {
      if (g < ng) {
        wz[g] = d.wz + ((size_t)(g0 + g) * kz + k) * pl;
        pp[g] = d.fset[d.fcur][g0 + g] + (size_t)k * pl;
        out[g] = d.fset[d.fcur ^ 1][g0 + g] + (size_t)k * pl;
      }
    }
    // warm-up: the flux of face i_s (between rows i_s-1 and i_s)
    T v_i, rmv_i = T(1);
    {
      const size_t r = row(i_s);
      v_i = v[r];
      if (!rot) rmv_i = d.rmv[r];
      const T mz = rot ? v_i * dtrdy : (v_i * rmv_i) * dtrdy;
      const T mfac = rot ? T(0.5) * v_i : (T(0.5) * v_i) * rmv_i;
      const size_t r2 = row(i_s - 2), r1 = row(i_s - 1), rp = row(i_s + 1);
#pragma unroll
      for (int g = 0; g < G; ++g) {
        if (g < ng) {
          const T a = wz[g][r2], b = wz[g][r1], c = wz[g][r], e = wz[g][rp];
          fl_[g] = mfac * waf_hflux(mz, a, b, c, e);
          wm1_[g] = b; w0_[g] = c; wp1_[g] = e;
        }
      }
    }
    // the loads of row i+1 are issued while row i is computed
    T n_wp2[G], n_pold[G];
    T n_vn, n_rmvn, n_pn, n_ps, n_uu, n_oe, n_ow, n_zm, n_mx2;
    auto fetch_row = [&](int i) {
      const size_t r = row(i), rn = row(i + 1), r2 = row(i + 2);
#pragma unroll
      for (int g = 0; g < G; ++g) {
        if (g < ng) {
          n_wp2[g] = wz[g][r2];
          n_pold[g] = pp[g][r];
        }
      }
      n_vn = v[rn];
      n_rmvn = rot ? T(1) : d.rmv[rn];
      n_pn = wn_[r]; n_ps = ws_[r];
      n_uu = u[r];
      n_oe = we_[r]; n_ow = ww_[r];
      n_zm = rot ? d.mu[r] : d.rmu[r];
      n_mx2 = rot ? T(0) : d.mx2[r];
    };
    fetch_row(i_s);
    for (int i = i_s; i < i_e; ++i) {
      const size_t r = row(i);
      // per-row values shared by the fields of the group
      const T v_n = n_vn, rmv_n = n_rmvn, pn = n_pn, ps = n_ps, uu = n_uu, oe = n_oe, ow = n_ow;
      const T zm = n_zm, mx2 = n_mx2;
      T wp2v[G], poldv[G];
#pragma unroll
      for (int g = 0; g < G; ++g) { wp2v[g] = n_wp2[g]; poldv[g] = n_pold[g]; }
      if (i + 1 < i_e) fetch_row(i + 1);
      const T mz = rot ? v_n * dtrdy : (v_n * rmv_n) * dtrdy;
      const T mfac = rot ? T(0.5) * v_n : (T(0.5) * v_n) * rmv_n;
      const T pdv = rot ? (v_n * pn - v_i * ps) : ((v_n * rmv_n) * pn - (v_i * rmv_i) * ps);
      const T zz = (uu * zm) * dtrdx;
      const T zfac = rot ? T(0.5) * uu : (T(0.5) * uu) * zm;
      const T ue = __shfl_down_sync(0xffffffffu, uu, 1);  // u(j+1)
      const T zme = __shfl_down_sync(0xffffffffu, zm, 1);
      const T odv = rot ? (ue * oe - uu * ow) : ((ue * zme) * oe - (uu * zm) * ow);
#pragma unroll
      for (int g = 0; g < G; ++g) {
        if (g < ng) {
          const T wp2 = wp2v[g];
          const T fl_n = mfac * waf_hflux(mz, wm1_[g], w0_[g], wp1_[g], wp2);  // face i+1
          const T pold = poldv[g];
          const T zdv = pdv * pold;
          const T p0 = rot ? ((w0_[g] + fl_[g] * ps) - fl_n * pn) + zdv
                           : w0_[g] + mx2 * (((fl_[g] * ps) - fl_n * pn) + zdv);
          const T pm2 = __shfl_up_sync(0xffffffffu, p0, 2);
          const T pm1 = __shfl_up_sync(0xffffffffu, p0, 1);
          const T pp1 = __shfl_down_sync(0xffffffffu, p0, 1);
          const T zf = zfac * waf_hflux(zz, pm2, pm1, p0, pp1);  // face between j-1 and j
          const T zfe = __shfl_down_sync(0xffffffffu, zf, 1);    // face between j and j+1
          if (out_lane) {
            const T zdv2 = odv * pold;
            out[g][r] = rot ? ((p0 + zf * ow) - zfe * oe) + zdv2 : p0 + mx2 * (((zf * ow) - zfe * oe) + zdv2);
          }
          wm1_[g] = w0_[g]; w0_[g] = wp1_[g]; wp1_[g] = wp2; fl_[g] = fl_n;
        }
      }
      v_i = v_n; rmv_i = rmv_n;
    }
  }
}

template <class T>
__global__ void __launch_bounds__(128) k_waf_hstrip(View<T> d) {
  b_waf_hstrip<T>(d, blockIdx.x, blockIdx.y);
}

template <class T>
__global__ void __launch_bounds__(128)
    kb_waf_hstrip(const View<T>* __restrict__ views, const int4* __restrict__ tiles) {
  __shared__ View<T> sv;
  const int4 t = tiles[blockIdx.x];
  copy_view(&sv, views + t.x);
  __syncthreads();
  b_waf_hstrip<T>(sv, t.y, t.z);
}


// ---- advection: cross points -> staggered (:1343-1387) ------------------
// Writes u, v into buffer 0 so every step replays the same pointers.
template <class T>
__device__ __forceinline__ void b_stag_from_x(const View<T>& d, const int bx, const int by, const int bz) {
  int jj = bx * kPtBX + threadIdx.x;
  int ii = by * kPtBY + threadIdx.y;
  const int nj = d.nj, ni = d.ni, kz = d.kz, kk = bz;
  if (jj >= nj || ii >= ni) return;
  // 32-bit element offsets: a field holds at most 2^31 points
  const unsigned pl = (unsigned)d.pl;
  const unsigned o = (unsigned)kk * pl;
  const unsigned c = (unsigned)jj + (unsigned)nj * (unsigned)ii;
  const unsigned rowj = (unsigned)nj * (unsigned)ii;
  const T* __restrict__ ux = d.ux;
  const T* __restrict__ vx = d.vx;
  d.ubuf[0][o + c] = T(0.5625) * (ux[o + c] + ux[o + rowj + wm1(jj, nj)]) -
                     T(0.0625) * (ux[o + rowj + wp1(jj, nj)] + ux[o + rowj + wm2(jj, nj)]);
  d.vbuf[0][o + c] = T(0.5625) * (vx[o + c] + vx[o + jj + (unsigned)nj * wm1(ii, ni)]) -
                     T(0.0625) * (vx[o + jj + (unsigned)nj * wp1(ii, ni)] + vx[o + jj + (unsigned)nj * wm2(ii, ni)]);
  // w(k), k = 2..kz (1-based) <- wx ; level index kk = k-1 in 1..kz-1
  if (kk >= 1) {
    const T* __restrict__ wx = d.wx;
    T wv;
    if (kk == 1)
      wv = T(0.5) * (wx[c + pl] + wx[c]);
    else if (kk == kz - 1)
      wv = T(0.5) * (wx[c + (unsigned)(kz - 1) * pl] + wx[c + (unsigned)(kz - 2) * pl]);
    else
      wv = T(0.5625) * (wx[c + kk * pl] + wx[c + (kk - 1) * pl]) -
           T(0.0625) * (wx[c + (kk + 1) * pl] + wx[c + (kk - 2) * pl]);
    d.w[c + kk * pl] = wv;
  }
}

template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY) k_stag_from_x(View<T> d) {
  b_stag_from_x<T>(d, blockIdx.x, blockIdx.y, blockIdx.z);
}

// The same for FP32 storage with jx a multiple of 4 (View::stag4): each
// thread takes four consecutive columns j0 .. j0+3 of one row and level,
// with 16-byte loads and stores -- ux of columns j0-4 .. j0+7 (periodic:
// the neighbouring quads wrap whole, since jx is a multiple of 4), vx of
// rows i-2 .. i+1 and wx of levels k-2 .. k+1 -- and the expressions of
// b_stag_from_x per column: 14 vector memory instructions per four points
// instead of 60 scalar ones.
__global__ void __launch_bounds__(kPtBX* kPtBY) k_stag_from_x4(View<float> d) {
  const int nj = d.nj, ni = d.ni, kz = d.kz, kk = blockIdx.z;
  const int nq = nj >> 2;
  const int qj = blockIdx.x * kPtBX + threadIdx.x, ii = blockIdx.y * kPtBY + threadIdx.y;
  if (qj >= nq || ii >= ni) return;
  const unsigned pl = (unsigned)d.pl, o = (unsigned)kk * pl;
  const int j0 = 4 * qj;
  const unsigned row = (unsigned)nj * (unsigned)ii;
  const unsigned c = (unsigned)j0 + row;
  auto ld4 = [](const float* p) { return *reinterpret_cast<const float4*>(p); };
  auto st4 = [](float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; };
  auto f = [](float a, float b, float cc, float dd) { return 0.5625f * (a + b) - 0.0625f * (cc + dd); };
  {  // u(j) <- ux(j-2 .. j+1)
    const float* ux = d.ux + o + row;
    const float4 A = ld4(ux + (j0 == 0 ? nj - 4 : j0 - 4)), B = ld4(ux + j0), C = ld4(ux + (j0 + 4 == nj ? 0 : j0 + 4));
    st4(d.ubuf[0] + o + c, make_float4(f(B.x, A.w, B.y, A.z), f(B.y, B.x, B.z, A.w), f(B.z, B.y, B.w, B.x),
                                       f(B.w, B.z, C.x, B.y)));
  }
  {  // v(i) <- vx(i-2 .. i+1)
    const float* vx = d.vx + o + j0;
    const float4 P = ld4(vx + row), M1 = ld4(vx + (unsigned)nj * wm1(ii, ni)), P1 = ld4(vx + (unsigned)nj * wp1(ii, ni)),
                 M2 = ld4(vx + (unsigned)nj * wm2(ii, ni));
    st4(d.vbuf[0] + o + c, make_float4(f(P.x, M1.x, P1.x, M2.x), f(P.y, M1.y, P1.y, M2.y), f(P.z, M1.z, P1.z, M2.z),
                                       f(P.w, M1.w, P1.w, M2.w)));
  }
  if (kk >= 1) {  // w(k), k = 2..kz (1-based) <- wx; level index kk = k-1 in 1..kz-1
    const float* wx = d.wx + c;
    float4 wv;
    if (kk == 1 || kk == kz - 1) {
      const float4 a = ld4(wx + (unsigned)kk * pl), b = ld4(wx + (unsigned)(kk - 1) * pl);
      wv = make_float4(0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z), 0.5f * (a.w + b.w));
    } else {
      const float4 a = ld4(wx + (unsigned)kk * pl), b = ld4(wx + (unsigned)(kk - 1) * pl);
      const float4 e = ld4(wx + (unsigned)(kk + 1) * pl), g = ld4(wx + (unsigned)(kk - 2) * pl);
      wv = make_float4(f(a.x, b.x, e.x, g.x), f(a.y, b.y, e.y, g.y), f(a.z, b.z, e.z, g.z), f(a.w, b.w, e.w, g.w));
    }
    st4(d.w + c + (unsigned)kk * pl, wv);
  }
}

template <class T>
__global__ void __launch_bounds__(kPtBX* kPtBY)
    kb_stag_from_x(const View<T>* __restrict__ views, const int4* __restrict__ tiles) {
  __shared__ View<T> sv;
  const int4 t = tiles[blockIdx.x];
  copy_view(&sv, views + t.x);
  __syncthreads();
  b_stag_from_x<T>(sv, t.y, t.z, t.w);
}


// ---- post-diagnostics (:355-391), one thread per column ----------------
template <class T>
__device__ __forceinline__ void b_postdiag(const View<T>& d, const int bx, const int by, const int bz) {  const T* __restrict__ zk = d.zeta + (size_t)d.pl * (d.kz - 1);
  const T* __restrict__ zkm1 = d.zeta + (size_t)d.pl * (d.kz - 2);

  int jj = bx * kColBX + threadIdx.x;
  int ii = by * kColBY + threadIdx.y;
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

template <class T>
__global__ void __launch_bounds__(kColBX* kColBY) k_postdiag(View<T> d) {
  b_postdiag<T>(d, blockIdx.x, blockIdx.y, blockIdx.z);
}

template <class T>
__global__ void __launch_bounds__(kColBX* kColBY)
    kb_postdiag(const View<T>* __restrict__ views, const int4* __restrict__ tiles) {
  __shared__ View<T> sv;
  const int4 t = tiles[blockIdx.x];
  copy_view(&sv, views + t.x);
  __syncthreads();
  b_postdiag<T>(sv, t.y, t.z, t.w);
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
inline FieldPtrs<T> field_set(const View<T>& d, int set) {
  FieldPtrs<T> fp;
  for (int n = 0; n < kNumAdvected; ++n) fp.f[n] = d.fset[set][n];
  return fp;
}

inline dim3 col_grid(int nj, int ni, int z = 1) {
  return dim3((nj + kColBX - 1) / kColBX, (ni + kColBY - 1) / kColBY, z);
}
inline dim3 pt_grid(int nj, int ni, int nz) {
  return dim3((nj + kPtBX - 1) / kPtBX, (ni + kPtBY - 1) / kPtBY, nz);
}

template <class T>
int launch_prediag(const View<T>& d, cudaStream_t st, const PhaseFlags& fl) {
  MOLOCH_LAUNCH(KK_PREDIAG, st, k_prediag<T><<<pt_grid(d.nj, d.ni, d.kz), dim3(kPtBX, kPtBY), 0, st>>>(d, fl.filterpai, fl.filtertheta));
  return 1;
}

// the staged column kernel runs when asked for (kmarch bit 32) on an FP32
// domain whose tensor maps were built
template <class T>
inline bool column_tm_ok(const View<T>& d) {
  return sizeof(T) == 4 && (d.kmarch & 32) && d.cmaps != nullptr;
}
// persistent column kernels: one CTA per SM, at most one per tile
inline int persistent_grid(int ntiles) {
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (nsm <= 0) nsm = 1;
  }
  return ntiles < nsm ? ntiles : nsm;
}
inline int column_tm_grid(int nj, int ni) { return persistent_grid(((nj + 31) / 32) * ((ni + 3) / 4)); }
template <class T>
inline int column_tm_grid(const View<T>& d) { return column_tm_grid(d.nj, d.ni); }

// one sound() call: nsound substeps; flips d.cur once per substep, twice
// with the fused divergence/damping kernel (kmarch bit 16)
template <class T>
int launch_sound(View<T>& d, cudaStream_t st, const PhaseFlags& fl) {
  int n = 0;
  const dim3 cb(kColBX, kColBY), cg = col_grid(d.nj, d.ni);
  const dim3 pb(kPtBX, kPtBY), pg = pt_grid(d.nj, d.ni, d.kz);
  const dim3 kg = pt_grid(d.nj, d.ni, (d.kz + kKC - 1) / kKC);  // k-marching: chunks of kKC levels
  for (int ns = 1; ns <= fl.nsound; ++ns) {
    const int last = ns == fl.nsound;
    if (d.kmarch & 16) {
      const int nstrips = ((d.nj + kDDJ - 1) / kDDJ) * ((d.ni + kDDR - 1) / kDDR);
      const dim3 g2((nstrips + 3) / 4, (d.kz + kDDLevels - 1) / kDDLevels);
      if (d.kmarch & 512)  // kDDLevels levels per warp
        MOLOCH_LAUNCH(KK_SOUND_DIVDAMP, st, k_divdamp_strip_nl<T><<<g2, 128, 0, st>>>(d, kDDR));
      else
        MOLOCH_LAUNCH(KK_SOUND_DIVDAMP, st, k_divdamp_strip<T><<<dim3((nstrips + 3) / 4, d.kz), 128, 0, st>>>(d, kDDR));
      d.cur ^= 1;  // the damped u, v are in the other buffer
      ++n;
    } else {
      if (d.kmarch & 1)
        MOLOCH_LAUNCH(KK_SOUND_DIV, st, k_sound_div_km<T><<<kg, pb, 0, st>>>(d));
      else
        MOLOCH_LAUNCH(KK_SOUND_DIV, st, k_sound_div<T><<<pg, pb, 0, st>>>(d));
      if (d.kmarch & 2)
        MOLOCH_LAUNCH(KK_SOUND_DAMP, st, k_sound_damp_km<T><<<kg, pb, 0, st>>>(d));
      else
        MOLOCH_LAUNCH(KK_SOUND_DAMP, st, k_sound_damp<T><<<pg, pb, 0, st>>>(d));
      n += 2;
    }
    if (fl.divfilter) {
      MOLOCH_LAUNCH(KK_SOUND_COLUMN, st, k_sound_column<T><<<cg, cb, 0, st>>>(d, ns, last, 1));
      MOLOCH_LAUNCH(KK_LAP_FILTER, st, k_lap_filter<T><<<pg, pb, 0, st>>>(d));
      MOLOCH_LAUNCH(KK_PAI_UPDATE, st, k_pai_update<T><<<pg, pb, 0, st>>>(d));
      n += 3;
    } else {
      bool staged = false;
      if constexpr (sizeof(T) == 4) {
        if (column_tm_ok(d)) {
          // bits 128 / 256: two words of column state a level, 12 / 16 rows
          const int cfg = (d.kmarch & 256) ? 2 : (d.kmarch & 128) ? 1 : 0;
          const ColumnMaps& cm = static_cast<const ColumnMaps*>(d.cmaps)[2 * cfg + d.fcur];
          const int grid = column_tm_grid(d);
          if (cfg == 2) {
            if (last)
              MOLOCH_LAUNCH(KK_SOUND_COLUMN_TM, st,
                            k_sound_column_tw<T, 1, 16><<<grid, TwCfg<16>::threads, TwCfg<16>::smem, st>>>(d, cm, ns));
            else
              MOLOCH_LAUNCH(KK_SOUND_COLUMN_TM, st,
                            k_sound_column_tw<T, 0, 16><<<grid, TwCfg<16>::threads, TwCfg<16>::smem, st>>>(d, cm, ns));
          } else if (cfg == 1) {
            if (last)
              MOLOCH_LAUNCH(KK_SOUND_COLUMN_TM, st,
                            k_sound_column_tw<T, 1, 12><<<grid, TwCfg<12>::threads, TwCfg<12>::smem, st>>>(d, cm, ns));
            else
              MOLOCH_LAUNCH(KK_SOUND_COLUMN_TM, st,
                            k_sound_column_tw<T, 0, 12><<<grid, TwCfg<12>::threads, TwCfg<12>::smem, st>>>(d, cm, ns));
          } else if (last) {
            MOLOCH_LAUNCH(KK_SOUND_COLUMN_TM, st, k_sound_column_tm<T, 1><<<grid, kTmThreads, kTmSmem, st>>>(d, cm, ns));
          } else {
            MOLOCH_LAUNCH(KK_SOUND_COLUMN_TM, st, k_sound_column_tm<T, 0><<<grid, kTmThreads, kTmSmem, st>>>(d, cm, ns));
          }
          staged = true;
        }
      }
      if (!staged) MOLOCH_LAUNCH(KK_SOUND_COLUMN, st, k_sound_column<T><<<cg, cb, 0, st>>>(d, ns, last, 0));
      ++n;
    }
    bool pairs = false;
    if constexpr (sizeof(T) == 4) {
      if ((d.kmarch & 8) && (d.kmarch & 64) && d.nj % 2 == 0) {  // two columns per lane
        const int nstrips = ((d.nj + 1 + kMom2J - 1) / kMom2J) * ((d.ni + d.srows - 1) / d.srows);
        MOLOCH_LAUNCH(KK_SOUND_MOMENTUM, st,
                      k_momentum_strip2<<<dim3((nstrips + 3) / 4, d.kz), 128, 0, st>>>(d, d.srows));
        pairs = true;
      }
    }
    if (pairs) {
    } else if (d.kmarch & 8) {
      const int nstrips = ((d.nj + kMomJ - 1) / kMomJ) * ((d.ni + d.srows - 1) / d.srows);
      MOLOCH_LAUNCH(KK_SOUND_MOMENTUM, st, k_momentum_strip<T><<<dim3((nstrips + 3) / 4, d.kz), 128, 0, st>>>(d, d.srows));
    } else if (d.kmarch & 4)
      MOLOCH_LAUNCH(KK_SOUND_MOMENTUM, st, k_sound_momentum_km<T><<<kg, pb, 0, st>>>(d));
    else
      MOLOCH_LAUNCH(KK_SOUND_MOMENTUM, st, k_sound_momentum<T><<<pg, pb, 0, st>>>(d));
    ++n;
    d.cur ^= 1;
  }
  return n;
}

// launch of the vertical WAF with the View's fields per thread
template <class T>
void launch_waf_vertical(const View<T>& d, cudaStream_t st) {
  const int ng = kNumAdvected / d.vfields;
  const dim3 vg(((d.nj + kColBX - 1) / kColBX) * ng, (d.ni + kColBY - 1) / kColBY), vb(kColBX, kColBY);
  switch (d.vfields) {
    case 2: MOLOCH_LAUNCH(KK_WAF_VERTICAL, st, k_waf_vertical<T, 2><<<vg, vb, 0, st>>>(d)); break;
    case 5: MOLOCH_LAUNCH(KK_WAF_VERTICAL, st, k_waf_vertical<T, 5><<<vg, vb, 0, st>>>(d)); break;
    case 10: MOLOCH_LAUNCH(KK_WAF_VERTICAL, st, k_waf_vertical<T, 10><<<vg, vb, 0, st>>>(d)); break;
    default: MOLOCH_LAUNCH(KK_WAF_VERTICAL, st, k_waf_vertical<T, 1><<<vg, vb, 0, st>>>(d)); break;
  }
}

template <class T>
void blaunch_waf_vertical(const Batch<T>& b, const View<T>* views, cudaStream_t st) {
  const int n = b.ntiles[TK_VERTICAL];
  const int4* tl = b.tiles[TK_VERTICAL];
  const dim3 vb(kColBX, kColBY);
  switch (b.vfields) {
    case 2: MOLOCH_LAUNCH(KK_WAF_VERTICAL, st, kb_waf_vertical<T, 2><<<n, vb, 0, st>>>(views, tl)); break;
    case 5: MOLOCH_LAUNCH(KK_WAF_VERTICAL, st, kb_waf_vertical<T, 5><<<n, vb, 0, st>>>(views, tl)); break;
    case 10: MOLOCH_LAUNCH(KK_WAF_VERTICAL, st, kb_waf_vertical<T, 10><<<n, vb, 0, st>>>(views, tl)); break;
    default: MOLOCH_LAUNCH(KK_WAF_VERTICAL, st, kb_waf_vertical<T, 1><<<n, vb, 0, st>>>(views, tl)); break;
  }
}


// one advection() call; the advected fields move to the other buffer set
template <class T>
int launch_advection(View<T>& d, cudaStream_t st) {
  const dim3 pb(kPtBX, kPtBY), pg = pt_grid(d.nj, d.ni, d.kz);
  const dim3 hg((d.nj + 31) / 32, (d.ni + 7) / 8, (d.kz + d.hz_levels - 1) / d.hz_levels);
  launch_waf_vertical<T>(d, st);  // forms ux, vx, wx from u, v, w as well
  if (d.hz_levels >= 16) {  // warp strips of hz_levels rows
    const int nstrips = ((d.nj + kStripJ - 1) / kStripJ) * ((d.ni + d.hz_levels - 1) / d.hz_levels);
    MOLOCH_LAUNCH(KK_WAF_HORIZONTAL, st, k_waf_hstrip<T><<<dim3((nstrips + 3) / 4, d.kz), 128, 0, st>>>(d));
  } else {
    MOLOCH_LAUNCH(KK_WAF_HORIZONTAL, st, k_waf_horizontal<T><<<hg, dim3(32, 8), 0, st>>>(d));
  }
  d.fcur ^= 1;
  d.bind_fields();
  bool vec = false;
  if constexpr (sizeof(T) == 4) {
    if (d.stag4 && d.nj % 4 == 0) {  // four columns per thread
      const dim3 g4((d.nj / 4 + kPtBX - 1) / kPtBX, (d.ni + kPtBY - 1) / kPtBY, d.kz);
      MOLOCH_LAUNCH(KK_STAG_FROM_X, st, k_stag_from_x4<<<g4, pb, 0, st>>>(d));
      vec = true;
    }
  }
  if (!vec) MOLOCH_LAUNCH(KK_STAG_FROM_X, st, k_stag_from_x<T><<<pg, pb, 0, st>>>(d));
  d.cur = 0;
  return 3;
}

template <class T>
int launch_postdiag(View<T>& d, cudaStream_t st, const PhaseFlags& fl, const T* zk, const T* zkm1) {
  int n = 0;
  const dim3 pb(kPtBX, kPtBY), pg = pt_grid(d.nj, d.ni, d.kz);
  const size_t bytes = sizeof(T) * (size_t)d.pl * d.kz;
  if (fl.filterpai) {
    MOLOCH_LAUNCH(KK_FILTER_INCREMENT, st, k_filter_increment<T><<<pg, pb, 0, st>>>(d, 0));
    cudaMemcpyAsync(d.pai, d.fscr, bytes, cudaMemcpyDeviceToDevice, st);
    ++n;
  }
  if (fl.filtertheta) {
    MOLOCH_LAUNCH(KK_FILTER_INCREMENT, st, k_filter_increment<T><<<pg, pb, 0, st>>>(d, 1));
    cudaMemcpyAsync(d.tetav, d.fscr, bytes, cudaMemcpyDeviceToDevice, st);
    ++n;
  }
  MOLOCH_LAUNCH(KK_POSTDIAG, st, k_postdiag<T><<<col_grid(d.nj, d.ni), dim3(kColBX, kColBY), 0, st>>>(d));
  return n + 1;
}

template <class T>
int launch_diag(const View<T>& d, cudaStream_t st) {
  const dim3 g = col_grid(d.nj, d.ni);
  MOLOCH_LAUNCH(KK_DIAG, st, k_diag_partial<T><<<g, dim3(kColBX, kColBY), 0, st>>>(d));
  MOLOCH_LAUNCH(KK_DIAG, st, k_diag_final<<<1, 256, 0, st>>>(d.dpart, (int)(g.x * g.y), d.dres));
  return 2;
}

// ---- batched launchers (ensembles) --------------------------------------
// One launch per phase covers every member; cur / fcur track the u/v buffer
// and field-set parities exactly as the single-domain launchers do.
template <class T>
int blaunch_step(const Batch<T>& b, cudaStream_t st, const PhaseFlags& fl, int& cur, int& fcur) {
  int n = 0;
  const dim3 pb(kPtBX, kPtBY), cb(kColBX, kColBY), hb(32, 8);
  auto V = [&]() { return b.views[cur][fcur]; };
  const int4* PT = b.tiles[TK_POINT];
  const int4* CO = b.tiles[TK_COLUMN];
  const int4* HZ = b.tiles[TK_HORIZONTAL];
  const int4* KC = b.tiles[TK_CHUNK];
  const int nkc = b.ntiles[TK_CHUNK];
  const int npt = b.ntiles[TK_POINT], nco = b.ntiles[TK_COLUMN];
  const int nhz = b.ntiles[TK_HORIZONTAL];
  MOLOCH_LAUNCH(KK_PREDIAG, st, kb_prediag<T><<<npt, pb, 0, st>>>(V(), PT, fl.filterpai, fl.filtertheta));
  ++n;
  for (int a = 0; a < fl.nadv; ++a) {
    for (int ns = 1; ns <= fl.nsound; ++ns) {
      const int last = ns == fl.nsound;
      if (b.kmarch & 16) {
        if (b.kmarch & 512)  // two levels per warp
          MOLOCH_LAUNCH(KK_SOUND_DIVDAMP, st,
                        kb_divdamp_strip_nl<T><<<b.ntiles[TK_DSTRIP2], 128, 0, st>>>(V(), b.tiles[TK_DSTRIP2], kDDR));
        else
          MOLOCH_LAUNCH(KK_SOUND_DIVDAMP, st,
                        kb_divdamp_strip<T><<<b.ntiles[TK_DSTRIP], 128, 0, st>>>(V(), b.tiles[TK_DSTRIP], kDDR));
        cur ^= 1;  // the damped u, v are in the other buffer
        --n;
      } else {
        if (b.kmarch & 1)
          MOLOCH_LAUNCH(KK_SOUND_DIV, st, kb_sound_div_km<T><<<nkc, pb, 0, st>>>(V(), KC));
        else
          MOLOCH_LAUNCH(KK_SOUND_DIV, st, kb_sound_div<T><<<npt, pb, 0, st>>>(V(), PT));
        if (b.kmarch & 2)
          MOLOCH_LAUNCH(KK_SOUND_DAMP, st, kb_sound_damp_km<T><<<nkc, pb, 0, st>>>(V(), KC));
        else
          MOLOCH_LAUNCH(KK_SOUND_DAMP, st, kb_sound_damp<T><<<npt, pb, 0, st>>>(V(), PT));
      }
      if (fl.divfilter) {
        MOLOCH_LAUNCH(KK_SOUND_COLUMN, st, kb_sound_column<T><<<nco, cb, 0, st>>>(V(), CO, ns, last, 1));
        MOLOCH_LAUNCH(KK_LAP_FILTER, st, kb_lap_filter<T><<<npt, pb, 0, st>>>(V(), PT));
        MOLOCH_LAUNCH(KK_PAI_UPDATE, st, kb_pai_update<T><<<npt, pb, 0, st>>>(V(), PT));
        n += 2;
      } else {
        bool staged = false;
        if constexpr (sizeof(T) == 4) {
          if ((b.kmarch & 32) && b.cmaps) {
            // the staged column solve over the tiles of the members with
            // tensor maps, the one-thread kernel over the others
            using TC = TwCfg<kTwRows>;
            const int ntw = b.ntiles[TK_COLTW], nrest = b.ntiles[TK_COLREST];
            const ColumnMaps* cms = static_cast<const ColumnMaps*>(b.cmaps);
            if (ntw > 0) {
              const int grid = persistent_grid(ntw);
              if (last)
                MOLOCH_LAUNCH(KK_SOUND_COLUMN, st,
                              kb_sound_column_tw<T, 1, kTwRows><<<grid, TC::threads, TC::smem, st>>>(
                                  V(), cms, b.tiles[TK_COLTW], ntw, fcur, ns, b.kerr, b.spin));
              else
                MOLOCH_LAUNCH(KK_SOUND_COLUMN, st,
                              kb_sound_column_tw<T, 0, kTwRows><<<grid, TC::threads, TC::smem, st>>>(
                                  V(), cms, b.tiles[TK_COLTW], ntw, fcur, ns, b.kerr, b.spin));
            }
            if (nrest > 0) {
              MOLOCH_LAUNCH(KK_SOUND_COLUMN, st,
                            kb_sound_column<T><<<nrest, cb, 0, st>>>(V(), b.tiles[TK_COLREST], ns, last, 0));
              if (ntw > 0) ++n;
            }
            staged = true;
          }
        }
        if (!staged) MOLOCH_LAUNCH(KK_SOUND_COLUMN, st, kb_sound_column<T><<<nco, cb, 0, st>>>(V(), CO, ns, last, 0));
      }
      if (b.kmarch & 8)
        MOLOCH_LAUNCH(KK_SOUND_MOMENTUM, st,
                      kb_momentum_strip<T><<<b.ntiles[TK_MSTRIP], 128, 0, st>>>(V(), b.tiles[TK_MSTRIP], b.mrows));
      else if (b.kmarch & 4)
        MOLOCH_LAUNCH(KK_SOUND_MOMENTUM, st, kb_sound_momentum_km<T><<<nkc, pb, 0, st>>>(V(), KC));
      else
        MOLOCH_LAUNCH(KK_SOUND_MOMENTUM, st, kb_sound_momentum<T><<<npt, pb, 0, st>>>(V(), PT));
      n += 4;
      cur ^= 1;
    }
    blaunch_waf_vertical<T>(b, V(), st);
    if (b.hstrip)
      MOLOCH_LAUNCH(KK_WAF_HORIZONTAL, st, kb_waf_hstrip<T><<<nhz, 128, 0, st>>>(V(), HZ));
    else
      MOLOCH_LAUNCH(KK_WAF_HORIZONTAL, st, kb_waf_horizontal<T><<<nhz, hb, 0, st>>>(V(), HZ));
    fcur ^= 1;
    MOLOCH_LAUNCH(KK_STAG_FROM_X, st, kb_stag_from_x<T><<<npt, pb, 0, st>>>(V(), PT));
    cur = 0;
    n += 3;
  }
  MOLOCH_LAUNCH(KK_POSTDIAG, st, kb_postdiag<T><<<nco, cb, 0, st>>>(V(), CO));
  return n + 1;
}

// the advection phase alone, for the ensemble autotuner
template <class T>
int blaunch_advection(const Batch<T>& b, cudaStream_t st, int& cur, int& fcur) {
  const dim3 pb(kPtBX, kPtBY), cb(kColBX, kColBY), hb(32, 8);
  blaunch_waf_vertical<T>(b, b.views[cur][fcur], st);
  if (b.hstrip)
    MOLOCH_LAUNCH(KK_WAF_HORIZONTAL, st, kb_waf_hstrip<T><<<b.ntiles[TK_HORIZONTAL], 128, 0, st>>>(b.views[cur][fcur], b.tiles[TK_HORIZONTAL]));
  else
    MOLOCH_LAUNCH(KK_WAF_HORIZONTAL, st, kb_waf_horizontal<T><<<b.ntiles[TK_HORIZONTAL], hb, 0, st>>>(b.views[cur][fcur], b.tiles[TK_HORIZONTAL]));
  fcur ^= 1;
  MOLOCH_LAUNCH(KK_STAG_FROM_X, st, kb_stag_from_x<T><<<b.ntiles[TK_POINT], pb, 0, st>>>(b.views[cur][fcur], b.tiles[TK_POINT]));
  cur = 0;
  return 3;
}

int diag_parts(int nj, int ni) {
  const dim3 g = col_grid(nj, ni);
  return (int)(g.x * g.y);
}

}  // namespace MOLOCH_KNS
}  // namespace moloch
