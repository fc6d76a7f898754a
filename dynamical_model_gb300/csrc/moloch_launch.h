// Declarations of the kernel launchers compiled in the kernel translation
// units (moloch_kernels_exact.cu: FP64 without multiply-add contraction;
// moloch_kernels_fast.cu: FP64 and FP32 with contraction).
#pragma once
#include <cuda_runtime.h>

#include "moloch_view.h"

namespace moloch {
#define MOLOCH_DECLARE_LAUNCHERS(NS)                                                                \
  namespace NS {                                                                                    \
  template <class T> int launch_prediag(const View<T>& d, cudaStream_t st, const PhaseFlags& fl);  \
  template <class T> int launch_sound(View<T>& d, cudaStream_t st, const PhaseFlags& fl);          \
  template <class T> int launch_advection(View<T>& d, cudaStream_t st);                            \
  template <class T>                                                                                \
  int launch_postdiag(View<T>& d, cudaStream_t st, const PhaseFlags& fl, const T* zk, const T* zkm1); \
  template <class T> int launch_diag(const View<T>& d, cudaStream_t st);                           \
  int diag_parts(int nj, int ni);                                                                   \
  void set_timer(KernelTimer* t);                                                                   \
  }
MOLOCH_DECLARE_LAUNCHERS(kexact)
MOLOCH_DECLARE_LAUNCHERS(kfast)
namespace kfast {
// TMA tensor maps of the staged column kernel for both advected-field
// buffer sets of an FP32 domain, written to `out` (column_maps_bytes()
// bytes, 64-byte aligned); false when the domain does not qualify (kz > 64,
// jx not a multiple of 4) or the driver cannot encode them
int column_maps_bytes();
// bytes of one set of tensor maps (one box shape, one buffer-set parity)
int column_map_set_bytes();
bool build_column_maps(const View<float>& v, void* out);
template <class T> int blaunch_step(const Batch<T>& b, cudaStream_t st, const PhaseFlags& fl, int& cur, int& fcur);
template <class T> int blaunch_advection(const Batch<T>& b, cudaStream_t st, int& cur, int& fcur);
}
#undef MOLOCH_DECLARE_LAUNCHERS

// idealized initial state on the device (moloch_init.cu)
namespace init {
struct IdealArgs {
  int nj, ni, kz, rotllr;
  double dx, ztop, zh, a0;
  int nhills;
  double hill_h[4], hill_j[4], hill_i[4], hill_r[4];
  double pert_amp;
  int pert_levels;
  unsigned long long seed;
};
template <class T>
int launch_ideal(const IdealArgs& a, const double* zita, const double* zitah, double* zeta, double* fmz,
                 double* fmzf, double* hx, double* hy, double* ulat, double* vlat, T* t, T* pai, T* qv,
                 cudaStream_t st);
template <class T> int launch_fill(T* p, size_t n, double value, cudaStream_t st);

// Direct host uploads: a kernel that reads the caller's host array through
// the host page tables (NVLink-C2C; the device reports pageable memory
// access): dst[(kk*ni + i)*nj + j] = src[A + kk*P + i*Rw + j], the interior
// of a Fortran-layout array (0-based kk < nk, i < ni, j < nj) in the bulk type.
// wide: the source is device memory (a staging copy) and the grid fills the
// GPU; otherwise one small block per SM, for a host source read while
// steps run beside it
template <class T>
int launch_upload_direct(T* dst, const double* src, long A, long P, long Rw, int nj, int ni, int nk, cudaStream_t st,
                         bool wide);
// Fortran layout of an output field in device memory: every element of an
// array with bounds (lb0:lb0+n1-1, lb1:lb1+n2-1, 1:nk) from the dense
// device field, halo indices wrapped periodically
template <class T>
int launch_output_layout(double* dst, const T* src, int lb0, int n1, int lb1, int n2, int nk, int nj, int ni,
                         cudaStream_t st);
}  // namespace init
}  // namespace moloch
