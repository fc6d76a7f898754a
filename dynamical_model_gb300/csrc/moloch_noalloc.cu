// WAF advection of one field that allocates no device memory
// (moloch_gpu_wafone_noalloc in include/moloch_gb300.h).
//
// Who needs it: callers that own every byte of device memory themselves --
// a Fortran model whose arrays live in its own CUDA/OpenACC data regions, or
// a host framework running its own memory pool -- and therefore cannot let a
// library call cudaMalloc (which can synchronise the device, fragment or
// exceed the caller's pool, or fail in a process that has already reserved
// the GPU's memory).  They pass device pointers for the inputs and the
// output; the two work arrays of wafone (wz, p0) live in a fixed
// file-scope __device__ array instead of being allocated.
//
// The arithmetic is that of wafone (nompi/mod_moloch.F90:929-1311) with the
// metric factors computed inline from fmz, fmzf and the map factors; this
// file is compiled without multiply-add contraction, so its results are the
// same as the advection phase of the exact FP64 build.
#define MOLOCH_KNS knoalloc
#include <cstdio>
#include <mutex>

#include "../../include/moloch_gb300.h"
#include "moloch_kernels.cuh"

extern "C" void moloch_internal_set_error(const char* msg);

namespace moloch {
namespace knoalloc {

// Largest jx*iy*kz a call may pass: 2^21 points.  Scratch = wz + p0 =
// 2 * 2^21 doubles = 32 MiB.  The CUDA runtime reserves it on a device when
// it loads this file's device code there -- with lazy module loading (the
// default), during the first call on that device, which looks the array up
// -- and holds it until the process exits.
constexpr long long kMaxPoints = 1LL << 21;
static __device__ __align__(256) double g_scratch[2 * kMaxPoints];

struct NaArgs {
  double* pp;
  const double* s;
  const double* u;
  const double* v;
  const double* fmz;
  const double* fmzf;
  const double* mu;
  const double* mv;
  const double* mx;
  double* wz;
  double* p0;
  int nj, ni, kz;
  double dtrdx, dtrdy, dtrdz;
  int rotllr;
};

// one vertical pass (:966-1020 / :1022-1072) with inline metric factors
__device__ void na_vpass(const double* src, double* dst, const NaArgs& a, size_t c) {
  const size_t pl = (size_t)a.nj * a.ni;
  const int kz = a.kz;
  double x0 = src[c], x1 = x0, x2 = src[c + pl];
  double wfw_k = 0.0, s_k = a.s[c];
  for (int k = 1; k <= kz; ++k) {
    const size_t o = (size_t)(k - 1) * pl;
    const double s_k1 = a.s[c + (size_t)k * pl];
    const int k2 = k + 2 <= kz ? k + 2 : kz;
    const double x3 = src[c + (size_t)(k2 - 1) * pl];
    double wfw_k1 = 0.0;
    if (k <= kz - 1) {
      const double zamu = s_k1 * a.dtrdz;
      double is, num;
      if (zamu >= 0.0) { is = 1.0; num = x2 - x3; } else { is = -1.0; num = x0 - x1; }
      const double r = num / safeden(x1 - x2);
      const double b = superbee(r);
      const double zphi = (is + zamu * b) - is * b;
      wfw_k1 = (0.5 * s_k1) * ((1.0 + zphi) * x2 + (1.0 - zphi) * x1);
    }
    const double f = a.fmz[c + o];
    const double zrfmu = (a.dtrdz * f) / a.fmzf[c + o];
    const double zrfmd = (a.dtrdz * f) / a.fmzf[c + o + pl];
    const double zdv = (s_k * zrfmu - s_k1 * zrfmd) * x1;
    dst[c + o] = ((x1 - wfw_k * zrfmu) + wfw_k1 * zrfmd) + zdv;
    x0 = x1; x1 = x2; x2 = x3; wfw_k = wfw_k1; s_k = s_k1;
  }
}

__global__ void __launch_bounds__(128) k_na_vertical(NaArgs a) {
  const int jj = blockIdx.x * 32 + threadIdx.x, ii = blockIdx.y * 4 + threadIdx.y;
  if (jj >= a.nj || ii >= a.ni) return;
  const size_t c = jj + (size_t)a.nj * ii;
  na_vpass(a.pp, a.wz, a, c);
  na_vpass(a.wz, a.wz, a, c);
}

// WAF flux between cells m1 and 0 given the neighbours m2 and p1
__device__ __forceinline__ double na_flux(double zamu, double m2, double m1, double x0, double p1) {
  double is, num;
  if (zamu > 0.0) { is = 1.0; num = m1 - m2; } else { is = -1.0; num = p1 - x0; }
  const double r = num / safeden(x0 - m1);
  const double b = superbee(r);
  const double zphi = (is + zamu * b) - is * b;
  return (1.0 + zphi) * m1 + (1.0 - zphi) * x0;
}

// meridional flux + update (:1080-1131); each point evaluates its two fluxes
__global__ void __launch_bounds__(256) k_na_meridional(NaArgs a) {
  const int jj = blockIdx.x * 32 + threadIdx.x, ii = blockIdx.y * 8 + threadIdx.y, kk = blockIdx.z;
  const int nj = a.nj, ni = a.ni;
  if (jj >= nj || ii >= ni) return;
  const size_t ko = (size_t)kk * nj * ni;
  auto W = [&](int i) { return a.wz[ko + jj + (size_t)nj * wrapn(i, ni)]; };
  auto V = [&](int i) { return a.v[ko + jj + (size_t)nj * wrapn(i, ni)]; };
  auto RMV = [&](int i) { return 1.0 / a.mv[jj + (size_t)nj * wrapn(i, ni)]; };
  double zp[2];
  for (int n = 0; n < 2; ++n) {  // zpby at i and i+1
    const int i = ii + n;
    const double vv = V(i);
    const double zamu = a.rotllr ? vv * a.dtrdy : (vv * RMV(i)) * a.dtrdy;
    const double fl = na_flux(zamu, W(i - 2), W(i - 1), W(i), W(i + 1));
    zp[n] = a.rotllr ? (0.5 * vv) * fl : ((0.5 * vv) * RMV(i)) * fl;
  }
  const size_t c = jj + (size_t)nj * ii;
  const double f = a.fmz[ko + c], fn = a.fmz[ko + jj + (size_t)nj * wrapn(ii + 1, ni)];
  const double fs = a.fmz[ko + jj + (size_t)nj * wrapn(ii - 1, ni)];
  const double pp = a.pp[ko + c], vs = V(ii), vn = V(ii + 1);
  double p0;
  if (a.rotllr) {
    const double mxx = a.mx[c];
    const double zhxvtn = (a.dtrdy * RMV(ii + 1)) * mxx, zhxvts = (a.dtrdy * RMV(ii)) * mxx;
    const double zrfmn = ((zhxvtn * 2.0) * f) / (f + fn), zrfms = ((zhxvts * 2.0) * f) / (f + fs);
    const double zdv = (vn * zrfmn - vs * zrfms) * pp;
    p0 = ((W(ii) + zp[0] * zrfms) - zp[1] * zrfmn) + zdv;
  } else {
    const double zrfmn = ((a.dtrdy * 2.0) * f) / (f + fn), zrfms = ((a.dtrdy * 2.0) * f) / (f + fs);
    const double zdv = ((vn * RMV(ii + 1)) * zrfmn - (vs * RMV(ii)) * zrfms) * pp;
    const double mx2 = a.mx[c] * a.mx[c];
    p0 = W(ii) + mx2 * (((zp[0] * zrfms) - zp[1] * zrfmn) + zdv);
  }
  a.p0[ko + c] = p0;
}

// zonal flux + update of pp (:1138-1187)
__global__ void __launch_bounds__(256) k_na_zonal(NaArgs a) {
  const int jj = blockIdx.x * 32 + threadIdx.x, ii = blockIdx.y * 8 + threadIdx.y, kk = blockIdx.z;
  const int nj = a.nj, ni = a.ni;
  if (jj >= nj || ii >= ni) return;
  const size_t ko = (size_t)kk * nj * ni, row = (size_t)nj * ii;
  auto P = [&](int j) { return a.p0[ko + row + wrapn(j, nj)]; };
  auto U = [&](int j) { return a.u[ko + row + wrapn(j, nj)]; };
  auto MU = [&](int j) { return a.mu[row + wrapn(j, nj)]; };
  double zp[2];
  for (int n = 0; n < 2; ++n) {  // zpbw at j and j+1
    const int j = jj + n;
    const double uu = U(j);
    const double m = a.rotllr ? MU(j) : 1.0 / MU(j);
    const double zamu = (uu * m) * a.dtrdx;
    const double fl = na_flux(zamu, P(j - 2), P(j - 1), P(j), P(j + 1));
    zp[n] = a.rotllr ? (0.5 * uu) * fl : ((0.5 * uu) * m) * fl;
  }
  const size_t c = row + jj;
  const double f = a.fmz[ko + c], fe = a.fmz[ko + row + wrapn(jj + 1, nj)], fw = a.fmz[ko + row + wrapn(jj - 1, nj)];
  const double pp = a.pp[ko + c], uw = U(jj), ue = U(jj + 1);
  double out;
  if (a.rotllr) {
    const double zcostx = a.dtrdx * MU(jj);
    const double zrfme = ((zcostx * 2.0) * f) / (f + fe), zrfmw = ((zcostx * 2.0) * f) / (f + fw);
    const double zdv = (ue * zrfme - uw * zrfmw) * pp;
    out = ((P(jj) + zp[0] * zrfmw) - zp[1] * zrfme) + zdv;
  } else {
    const double zrfme = ((a.dtrdx * 2.0) * f) / (f + fe), zrfmw = ((a.dtrdx * 2.0) * f) / (f + fw);
    const double zdv = ((ue * (1.0 / MU(jj + 1))) * zrfme - (uw * (1.0 / MU(jj))) * zrfmw) * pp;
    const double mx2 = a.mx[c] * a.mx[c];
    out = P(jj) + mx2 * (((zp[0] * zrfmw) - zp[1] * zrfme) + zdv);
  }
  a.pp[ko + c] = out;
}

// device address of g_scratch, looked up once per device
constexpr int kMaxDevices = 64;
static double* g_scratch_ptr[kMaxDevices];
static std::mutex g_scratch_mu;

}  // namespace knoalloc
}  // namespace moloch

extern "C" int moloch_gpu_wafone_noalloc(double* pp, const double* s, const double* u, const double* v,
                                         const double* fmz, const double* fmzf, const double* msfu,
                                         const double* msfv, const double* msfx, int jx, int iy, int kz,
                                         double dta, double dx, double dzita, int rotllr, void* stream) {
  using namespace moloch::knoalloc;
  if (!pp || !s || !u || !v || !fmz || !fmzf || !msfu || !msfv || !msfx) {
    moloch_internal_set_error("wafone_noalloc: null pointer");
    return MOLOCH_ERR_ARG;
  }
  if (jx < 4 || iy < 4 || kz < 4) {
    moloch_internal_set_error("wafone_noalloc: jx, iy and kz must be >= 4");
    return MOLOCH_ERR_ARG;
  }
  if (kz > 65535) {  // the meridional and zonal kernels take k as gridDim.z
    moloch_internal_set_error("wafone_noalloc: kz must be <= 65535");
    return MOLOCH_ERR_ARG;
  }
  if ((long long)jx * iy * kz > kMaxPoints) {
    char buf[200];
    snprintf(buf, sizeof buf, "wafone_noalloc: jx*iy*kz = %lld exceeds the fixed scratch of %lld points",
             (long long)jx * iy * kz, kMaxPoints);
    moloch_internal_set_error(buf);
    return MOLOCH_ERR_ARG;
  }
  if (!(dta > 0) || !(dx > 0) || !(dzita > 0)) {
    moloch_internal_set_error("wafone_noalloc: dta, dx and dzita must be positive");
    return MOLOCH_ERR_ARG;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    moloch_internal_set_error("wafone_noalloc: no current CUDA device");
    return MOLOCH_ERR_CUDA;
  }
  double* scratch;
  {
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {  // set-up on the first call on this device
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_scratch);
      if (e != cudaSuccess || !p) {
        moloch_internal_set_error(cudaGetErrorString(e));
        return MOLOCH_ERR_CUDA;
      }
      g_scratch_ptr[dev] = (double*)p;
    }
    scratch = g_scratch_ptr[dev];
  }
  NaArgs a;
  a.pp = pp; a.s = s; a.u = u; a.v = v; a.fmz = fmz; a.fmzf = fmzf;
  a.mu = msfu; a.mv = msfv; a.mx = msfx;
  const size_t n = (size_t)jx * iy * kz;
  a.wz = scratch;      // fully written by k_na_vertical before it is read
  a.p0 = scratch + n;  // fully written by k_na_meridional before it is read
  a.nj = jx; a.ni = iy; a.kz = kz;
  a.dtrdx = dta / dx;  // wafone :951-956
  a.dtrdy = dta / dx;
  a.dtrdz = 0.5 * (dta / dzita);
  a.rotllr = rotllr;
  cudaStream_t st = (cudaStream_t)stream;
  // each launch's own status: cudaGetLastError here would also return (and
  // clear) an error the caller left pending before this call
  void* args[] = {&a};
  const dim3 gv((jx + 31) / 32, (iy + 3) / 4), bv(32, 4);
  const dim3 gh((jx + 31) / 32, (iy + 7) / 8, kz), bh(32, 8);
  e = cudaLaunchKernel((const void*)k_na_vertical, gv, bv, args, 0, st);
  if (e == cudaSuccess) e = cudaLaunchKernel((const void*)k_na_meridional, gh, bh, args, 0, st);
  if (e == cudaSuccess) e = cudaLaunchKernel((const void*)k_na_zonal, gh, bh, args, 0, st);
  if (e != cudaSuccess) {
    moloch_internal_set_error(cudaGetErrorString(e));
    return MOLOCH_ERR_CUDA;
  }
  return MOLOCH_OK;
}
