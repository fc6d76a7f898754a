// Idealized initial state on the device: the reference driver's param()
// (nompi/regcm_dynamical_core.F90:93-194, with the vertical coordinate of
// nompi/mod_zita.F90:43-179) and fill_atmosphere()
// (nompi/mod_atmosphere.F90:171-235), plus the input generator's hills,
// background wind and seeded theta perturbation -- the same arithmetic as
// the host restatement in moloch_ideal.cpp, one thread per column.
// Compiled without multiply-add contraction, so only the CUDA exp/pow/sqrt
// roundings can differ from the host path.
//
// Outputs: the FP64 static fields a Fortran caller would upload (zeta, fmz,
// fmzf, hx, hy, ulat, vlat: dense interiors, j fastest) and the prognostic
// state t, pai, qv written directly in the bulk type.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "moloch_constants.h"
#include "moloch_launch.h"

namespace moloch {
namespace init {

__device__ double u01(uint64_t seed, uint64_t idx) {  // splitmix64 of the linear index
  uint64_t z = seed + (idx + 1ULL) * 0x9E3779B97F4A7C15ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z = z ^ (z >> 31);
  return (double)(z >> 11) * (1.0 / 9007199254740992.0);
}

__device__ double zfz(double ztop, double zh) { return ztop / (exp(ztop / zh) - 1.0); }
__device__ double bzita(double z, double ztop, double zh) { return zfz(ztop, zh) * (exp(z / zh) - 1.0); }
__device__ double bzitap(double z, double ztop, double zh) { return zfz(ztop, zh) * exp(z / zh) / zh; }
__device__ double gzita(double z, double ztop, double a0) {
  double r = z / ztop, r2 = r * r, r3 = r2 * r;
  return (((0.0 - 1.0 * a0) * r - (3.0 - 2.0 * a0) * r2) + (2.0 - 1.0 * a0) * r3) + 1.0;
}
__device__ double gzitap(double z, double ztop, double a0) {
  double r = z / ztop, r2 = r * r;
  return (((0.0 - 1.0 * a0) * 1.0 - (6.0 - 4.0 * a0) * r) + (6.0 - 3.0 * a0) * r2) / ztop;
}

// ht of an interior point (1-based); the reference never sets the ghosts of
// ht, so ht(0, i) and ht(j, 0) are 0
__device__ double ht_at(const IdealArgs& a, int j, int i) {
  if (j < 1 || i < 1) return 0.0;
  double h = 0.0;
  for (int n = 0; n < a.nhills && n < 4; ++n) {
    double dj = (double)j - a.hill_j[n], di = (double)i - a.hill_i[n];
    double rr = (dj * dj + di * di) / (a.hill_r[n] * a.hill_r[n]);
    h += a.hill_h[n] * kEgrav * exp(-rr);
  }
  return h;
}

template <class T>
__global__ void __launch_bounds__(128) k_ideal(IdealArgs a, const double* __restrict__ zita,
                                                const double* __restrict__ zitah, double* __restrict__ zeta,
                                                double* __restrict__ fmz, double* __restrict__ fmzf,
                                                double* __restrict__ hx, double* __restrict__ hy,
                                                double* __restrict__ ulat, double* __restrict__ vlat,
                                                T* __restrict__ t_out, T* __restrict__ pai_out, T* __restrict__ qv_out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;  // 1-based
  const int i = blockIdx.y + 1;
  const int nj = a.nj, ni = a.ni, kz = a.kz;
  if (j > nj) return;
  const size_t pl = (size_t)nj * ni, c = (size_t)(j - 1) + (size_t)nj * (i - 1);
  const double rdx = 1.0 / a.dx;
  // ---- param(): orography, map terms, latitude, vertical coordinate
  const double ht = ht_at(a, j, i);
  hx[c] = (((ht - ht_at(a, j - 1, i)) * 1.0) * rdx) * kRegrav;
  hy[c] = a.rotllr ? ((ht - ht_at(a, j, i - 1)) * rdx) * kRegrav
                   : (((ht - ht_at(a, j, i - 1)) * 1.0) * rdx) * kRegrav;
  const double dl = kRaddeg * a.dx / kEarthrad;
  ulat[c] = 0.0 + dl * (((double)i - (double)ni * 0.5) - 0.5);
  vlat[c] = 0.0 + dl * ((double)i - (double)ni * 0.5);
  const double orog = ht * kRegrav;
  for (int k = 1; k <= kz; ++k) {
    const double z = zitah[k];
    zeta[c + pl * (k - 1)] = orog * (gzita(z, a.ztop, a.a0) - 1.0) + bzita(z, a.ztop, a.zh);
    fmz[c + pl * (k - 1)] = 1.0 / (gzitap(z, a.ztop, a.a0) * orog + bzitap(z, a.ztop, a.zh));
  }
  for (int k = 1; k <= kz + 1; ++k)
    fmzf[c + pl * (k - 1)] = 1.0 / (gzitap(zita[k], a.ztop, a.a0) * orog + bzitap(zita[k], a.ztop, a.zh));

  // ---- fill_atmosphere(): moisture and temperature profiles
  const double ts = 300.0, qs0 = 0.01865, ps0 = 101480.0, tropoh = 15000.0;
  const double tvs = ts * (1.0 + kEp1 * qs0);
  const double tvt = tvs - kLrate * tropoh;
  auto T3 = [&](int k) { return c + pl * (size_t)(k - 1); };
  auto profile = [&](int k, double& ti, double& qi) {
    const double zi = zeta[T3(k)];
    if (zi < tropoh) {
      const double xq = -(zi / 7500.0);
      qi = (qs0 * exp(-(zi / 4000.0))) * exp(xq * xq);
      ti = (tvs - kLrate * zi) / (1.0 + qi);
    } else {
      qi = 1.0e-8;
      ti = tvt;
    }
  };
  for (int k = 1; k <= kz; ++k) {
    double ti, qi;
    profile(k, ti, qi);
    qv_out[T3(k)] = (T)qi;
  }
  // t and qv of the two lowest levels; the warm bubble on the lowest level,
  // whose radius mixes default-REAL (single) and FP64 arithmetic as written
  // in the reference
  double t_lo, q_lo, t_lo1, q_lo1;
  profile(kz, t_lo, q_lo);
  profile(kz - 1, t_lo1, q_lo1);
  {
    const int mx = nj / 2, my = ni / 2;
    const double aj = (double)(float)nj / 5.0;
    const float bi = (float)ni / 5.0f;
    const float bi2 = bi * bi;
    const double mr = sqrt(aj * aj + (double)bi2) / 2.0;
    const float fj = (float)(j - mx), fi = (float)(i - my);
    const double md = (double)sqrtf(fj * fj + fi * fi);
    if (md < mr) t_lo = t_lo + (mr - md) / mr;
  }
  // ---- hydrostatic pai from the lowest level up (k = kz .. 1), FP64
  double pai_k;
  {
    const double zk = zeta[T3(kz)], zk1 = zeta[T3(kz - 1)];
    const double zdelta = zk * kEgrav;
    const double tv1 = t_lo * (1.0 + kEp1 * q_lo);
    const double tv2 = t_lo1 * (1.0 + kEp1 * q_lo1);
    double lrt = (tv2 - tv1) / (zk1 - zk);
    lrt = 0.65 * lrt - 0.35 * kLrate;
    const double tv = tv1 - (0.5 * zk) * lrt;
    const double zz = 1.0 / (kRgas * tv);
    const double p = ps0 * exp(-(zdelta * zz));
    pai_k = pow(p / kP00, kRovcp);
  }
  const double dzita = zita[kz];
  const int kp0 = a.pert_amp != 0.0 ? (kz - a.pert_levels + 1 < 1 ? 1 : kz - a.pert_levels + 1) : kz + 1;
  auto emit = [&](int k, double ti, double pk) {
    if (k >= kp0) {
      const uint64_t idx = (uint64_t)(j - 1) + (uint64_t)nj * ((uint64_t)(i - 1) + (uint64_t)ni * (uint64_t)(k - 1));
      const double dth = a.pert_amp * (2.0 * u01(a.seed, idx) - 1.0);
      ti = ti + dth * pk;
    }
    t_out[T3(k)] = (T)ti;
    pai_out[T3(k)] = (T)pk;
  };
  emit(kz, t_lo, pai_k);
  double t_up = t_lo, q_up = q_lo;  // level k+1
  for (int k = kz - 1; k >= 1; --k) {
    double tk, qk;
    if (k == kz - 1) { tk = t_lo1; qk = q_lo1; } else { profile(k, tk, qk); }
    const double tv1 = tk * (1.0 + kEp1 * qk);
    const double tv2 = t_up * (1.0 + kEp1 * q_up);
    const double zb = (((2.0 * kEgrav) * dzita) / (fmzf[T3(k + 1)] * kCpd) + tv1) - tv2;
    const double zdelta = sqrt(zb * zb + (4.0 * tv2) * tv1);
    pai_k = -((pai_k / (2.0 * tv2)) * (zb - zdelta));
    emit(k, tk, pai_k);
    t_up = tk; q_up = qk;
  }
}

template <class T>
int launch_ideal(const IdealArgs& a, const double* zita, const double* zitah, double* zeta, double* fmz,
                 double* fmzf, double* hx, double* hy, double* ulat, double* vlat, T* t, T* pai, T* qv,
                 cudaStream_t st) {
  dim3 grid((a.nj + 127) / 128, a.ni);
  k_ideal<T><<<grid, 128, 0, st>>>(a, zita, zitah, zeta, fmz, fmzf, hx, hy, ulat, vlat, t, pai, qv);
  return 1;
}

template <class T>
__global__ void k_fill(T* __restrict__ p, size_t n, T value) {
  for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n; q += (size_t)gridDim.x * blockDim.x)
    p[q] = value;
}

template <class T>
int launch_fill(T* p, size_t n, double value, cudaStream_t st) {
  const int blocks = (int)((n + 255) / 256 < 152 * 8 ? (n + 255) / 256 : 152 * 8);
  k_fill<T><<<blocks > 0 ? blocks : 1, 256, 0, st>>>(p, n, (T)value);
  return 1;
}

// ---- direct host uploads and output layout ------------------------------------
// Row-wise: a block takes whole rows (one (level, i) row of nj values), its
// threads consecutive j, so no per-element division and whole host rows.
// The upload kernel serves two sources: the caller's host array read
// through the host page tables (small grid, one block of 128 threads per
// SM: it runs beside the steps it overlaps, each thread with up to eight
// reads in flight) and a device staging copy of the array (that one by
// k_upload_gather below, at HBM speed).
template <class T>
__global__ void __launch_bounds__(128) k_upload_direct(T* __restrict__ dst, const double* __restrict__ src, long A,
                                                       long P, long Rw, int nj, int ni, int rows) {
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    const int kk = r / ni, i = r - kk * ni;
    const double* __restrict__ in = src + A + kk * P + i * Rw;
    T* __restrict__ out = dst + (size_t)r * nj;
    for (int j0 = threadIdx.x; j0 < nj; j0 += 8 * blockDim.x) {
      double x[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int j = j0 + u * blockDim.x;
        x[u] = j < nj ? in[j] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int j = j0 + u * blockDim.x;
        if (j < nj) out[j] = (T)x[u];
      }
    }
  }
}

// The same gather from a device staging copy: kUpR rows per block, all
// kUpR x kUpV loads of a thread issued before its stores (16 in flight for
// rows of up to 512 points), so the blocks do not end after one round trip.
constexpr int kUpR = 4, kUpV = 4;
template <class T>
__global__ void __launch_bounds__(128) k_upload_gather(T* __restrict__ dst, const double* __restrict__ src, long A,
                                                       long P, long Rw, int nj, int ni, int rows) {
  const int r0 = blockIdx.x * kUpR;
  for (int j0 = threadIdx.x; j0 < nj; j0 += kUpV * 128) {
    double x[kUpR][kUpV];
#pragma unroll
    for (int a = 0; a < kUpR; ++a) {
      const int r = r0 + a;
      const bool rv = r < rows;
      const int kk = rv ? r / ni : 0, i = rv ? r - kk * ni : 0;
      const double* __restrict__ in = src + A + kk * P + i * Rw;
#pragma unroll
      for (int u = 0; u < kUpV; ++u) {
        const int j = j0 + u * 128;
        x[a][u] = (rv && j < nj) ? in[j] : 0.0;
      }
    }
#pragma unroll
    for (int a = 0; a < kUpR; ++a) {
      const int r = r0 + a;
      if (r < rows) {
        T* __restrict__ out = dst + (size_t)r * nj;
#pragma unroll
        for (int u = 0; u < kUpV; ++u) {
          const int j = j0 + u * 128;
          if (j < nj) out[j] = (T)x[a][u];
        }
      }
    }
  }
}

// wide: the source is device memory (a staging copy), gathered by
// k_upload_gather; otherwise the source is host memory read through the
// host page tables by one block per SM
template <class T>
int launch_upload_direct(T* dst, const double* src, long A, long P, long Rw, int nj, int ni, int nk, cudaStream_t st,
                         bool wide) {
  const int rows = ni * nk;
  if (wide) {
    const int blocks = (rows + kUpR - 1) / kUpR;
    k_upload_gather<T><<<blocks > 0 ? blocks : 1, 128, 0, st>>>(dst, src, A, P, Rw, nj, ni, rows);
    return 1;
  }
  const int blocks = std::min(rows, 152);
  k_upload_direct<T><<<blocks > 0 ? blocks : 1, 128, 0, st>>>(dst, src, A, P, Rw, nj, ni, rows);
  return 1;
}

// Fortran layout of an output field: every element of an array with bounds
// (lb0:lb0+n1-1, lb1:lb1+n2-1, 1:nk) from the dense device field, halo
// indices wrapped periodically (they lie within one period of the
// interior), into device memory; a DMA then moves it to the caller's
// registered host array.  One block per row.
__device__ __forceinline__ int wrap1(int x, int n) {  // 1-based index -> 0-based periodic
  int y = x - 1;
  if (y < 0) y += n;
  else if (y >= n) y -= n;
  return y;
}

template <class T>
__global__ void __launch_bounds__(128) k_output_layout(double* __restrict__ dst, const T* __restrict__ src, int lb0,
                                                       int n1, int lb1, int n2, int nj, int ni, int rows) {
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    const int kk = r / n2, i = lb1 + (r - kk * n2);
    const T* __restrict__ in = src + ((size_t)kk * ni + wrap1(i, ni)) * nj;
    double* __restrict__ out = dst + (size_t)r * n1;
    for (int q = threadIdx.x; q < n1; q += blockDim.x) out[q] = (double)in[wrap1(lb0 + q, nj)];
  }
}

template <class T>
int launch_output_layout(double* dst, const T* src, int lb0, int n1, int lb1, int n2, int nk, int nj, int ni,
                         cudaStream_t st) {
  const int rows = n2 * nk;
  k_output_layout<T><<<rows > 0 ? rows : 1, 128, 0, st>>>(dst, src, lb0, n1, lb1, n2, nj, ni, rows);
  return 1;
}

template int launch_output_layout<double>(double*, const double*, int, int, int, int, int, int, int, cudaStream_t);
template int launch_output_layout<float>(double*, const float*, int, int, int, int, int, int, int, cudaStream_t);
template int launch_upload_direct<double>(double*, const double*, long, long, long, int, int, int, cudaStream_t, bool);
template int launch_upload_direct<float>(float*, const double*, long, long, long, int, int, int, cudaStream_t, bool);

template int launch_fill<double>(double*, size_t, double, cudaStream_t);
template int launch_fill<float>(float*, size_t, double, cudaStream_t);
template int launch_ideal<double>(const IdealArgs&, const double*, const double*, double*, double*, double*,
                                  double*, double*, double*, double*, double*, double*, double*, cudaStream_t);
template int launch_ideal<float>(const IdealArgs&, const double*, const double*, double*, double*, double*,
                                 double*, double*, double*, double*, float*, float*, float*, cudaStream_t);

}  // namespace init
}  // namespace moloch
