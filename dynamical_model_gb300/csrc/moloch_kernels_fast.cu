// FP64 and FP32-storage kernels with multiply-add contraction allowed.
#define MOLOCH_KNS kfast
#define MOLOCH_NR_DDIV 1  // FP64 WAF limiter quotient by Newton-Raphson (div_nr)
#include "../../include/moloch_gb300.h"
#include "moloch_kernels.cuh"

namespace moloch {
namespace kfast {
template int launch_prediag<double>(const View<double>&, cudaStream_t, const PhaseFlags&);
template int launch_sound<double>(View<double>&, cudaStream_t, const PhaseFlags&);
template int launch_advection<double>(View<double>&, cudaStream_t);
template int launch_postdiag<double>(View<double>&, cudaStream_t, const PhaseFlags&, const double*, const double*);
template int launch_diag<double>(const View<double>&, cudaStream_t);
template int launch_prediag<float>(const View<float>&, cudaStream_t, const PhaseFlags&);
template int launch_sound<float>(View<float>&, cudaStream_t, const PhaseFlags&);
template int launch_advection<float>(View<float>&, cudaStream_t);
template int launch_postdiag<float>(View<float>&, cudaStream_t, const PhaseFlags&, const float*, const float*);
template int launch_diag<float>(const View<float>&, cudaStream_t);
template int blaunch_step<double>(const Batch<double>&, cudaStream_t, const PhaseFlags&, int&, int&);
template int blaunch_step<float>(const Batch<float>&, cudaStream_t, const PhaseFlags&, int&, int&);
template int blaunch_advection<double>(const Batch<double>&, cudaStream_t, int&, int&);
template int blaunch_advection<float>(const Batch<float>&, cudaStream_t, int&, int&);
}  // namespace kfast
}  // namespace moloch

// ---- tensor maps of the staged column kernel --------------------------------
#include <mutex>

namespace moloch {
namespace kfast {
namespace {
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (EncodeTiledFn)p;
  });
  return fn;
}
// dense FP32 field (nj, ni, nk), j fastest, as boxes of 32 x rows x levels
bool map3(EncodeTiledFn fn, CUtensorMap* m, const float* base, int nj, int ni, int nk, int rows, int levels) {
  const cuuint64_t dims[3] = {(cuuint64_t)nj, (cuuint64_t)ni, (cuuint64_t)nk};
  const cuuint64_t strides[2] = {(cuuint64_t)nj * 4, (cuuint64_t)nj * ni * 4};
  const cuuint32_t box[3] = {32, (cuuint32_t)rows, (cuuint32_t)levels};
  const cuuint32_t es[3] = {1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, es,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
}  // namespace

int column_maps_bytes() { return (int)(2 * kColumnMapConfigs * sizeof(ColumnMaps)); }
int column_map_set_bytes() { return (int)sizeof(ColumnMaps); }

// the box shapes of the staged column kernels, in the order of the configs
// (ColumnMaps sets 2 cfg + buffer-set parity)
static const int kMapRows[kColumnMapConfigs] = {kTmRows, 12, 16};
static const int kMapLevels[kColumnMapConfigs] = {kKCT, TwCfg<12>::kct, TwCfg<16>::kct};

bool build_column_maps(const View<float>& v, void* out) {
  if (v.kz > kTmMaxKz || v.kz < 2 || v.nj % 4 != 0 || ((uintptr_t)out & 63)) return false;
  EncodeTiledFn fn = encode_tiled();
  if (!fn) return false;
  static std::once_flag attr;
  std::call_once(attr, [] {
    cudaFuncSetAttribute(k_sound_column_tm<float, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTmSmem);
    cudaFuncSetAttribute(k_sound_column_tm<float, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, kTmSmem);
    cudaFuncSetAttribute(k_sound_column_tw<float, 0, 12>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         TwCfg<12>::smem);
    cudaFuncSetAttribute(k_sound_column_tw<float, 1, 12>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         TwCfg<12>::smem);
    cudaFuncSetAttribute(k_sound_column_tw<float, 0, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         TwCfg<16>::smem);
    cudaFuncSetAttribute(k_sound_column_tw<float, 1, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         TwCfg<16>::smem);
    cudaFuncSetAttribute(kb_sound_column_tw<float, 0, kTwRows>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         TwCfg<kTwRows>::smem);
    cudaFuncSetAttribute(kb_sound_column_tw<float, 1, kTwRows>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         TwCfg<kTwRows>::smem);
  });
  ColumnMaps* cm = static_cast<ColumnMaps*>(out);
  const int nj = v.nj, ni = v.ni, kz = v.kz;
  for (int cfg = 0; cfg < kColumnMapConfigs; ++cfg) {
    const int r = kMapRows[cfg], l = kMapLevels[cfg];
    for (int set = 0; set < 2; ++set) {
      CUtensorMap* m = cm[2 * cfg + set].m;
      const bool ok =
          map3(fn, &m[CM_W], v.w, nj, ni, kz + 1, r, l) && map3(fn, &m[CM_FMZF], v.fmzf, nj, ni, kz + 1, r, l) &&
          map3(fn, &m[CM_QV], v.fset[set][5], nj, ni, kz, r, l) &&
          map3(fn, &m[CM_TET], v.fset[set][0], nj, ni, kz, r, l) &&
          map3(fn, &m[CM_PAI], v.fset[set][1], nj, ni, kz, r, l) && map3(fn, &m[CM_QSAT], v.qsat, nj, ni, kz, r, l) &&
          map3(fn, &m[CM_ZD], v.zdiv2b, nj, ni, kz, r, l) && map3(fn, &m[CM_FMZ], v.fmz, nj, ni, kz, r, l) &&
          map3(fn, &m[CM_T], v.t, nj, ni, kz, r, l) && map3(fn, &m[CM_QC], v.fset[set][6], nj, ni, kz, r, l) &&
          map3(fn, &m[CM_QWL], v.qwltot, nj, ni, kz, r, l) && map3(fn, &m[CM_QWI], v.qwitot, nj, ni, kz, r, l) &&
          map3(fn, &m[CM_S], v.s, nj, ni, kz + 1, r, l);
      if (!ok) return false;
    }
  }
  return cudaGetLastError() == cudaSuccess;
}
}  // namespace kfast
}  // namespace moloch

// ---- arithmetic check of the FP32 quotient with one correction --------------
namespace moloch {
namespace kfast {
__global__ void k_check_division(const float* __restrict__ a, const float* __restrict__ b, float* __restrict__ qc,
                                 float* __restrict__ qi, int n) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    qc[q] = div_corr(a[q], b[q]);
    qi[q] = a[q] / b[q];
  }
}
__global__ void k_check_division_f64(const double* __restrict__ a, const double* __restrict__ b,
                                     double* __restrict__ qn, double* __restrict__ qi, int n) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    qn[q] = qdiv(a[q], b[q]);  // div_nr in this build
    qi[q] = a[q] / b[q];
  }
}
}  // namespace kfast
}  // namespace moloch

// div_corr (the quotient of the FP32 Exner/theta update) and CUDA's IEEE
// FP32 quotient of the same device arrays, for tests of its error bound
extern "C" int moloch_gpu_check_division(const float* a, const float* b, float* q_corr, float* q_ieee, int n,
                                         void* stream) {
  if (!a || !b || !q_corr || !q_ieee || n < 0) return MOLOCH_ERR_ARG;
  if (n == 0) return MOLOCH_OK;
  const int blocks = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
  moloch::kfast::k_check_division<<<blocks, 256, 0, (cudaStream_t)stream>>>(a, b, q_corr, q_ieee, n);
  return cudaPeekAtLastError() == cudaSuccess ? MOLOCH_OK : MOLOCH_ERR_CUDA;
}
extern "C" int moloch_gpu_check_division_f64(const double* a, const double* b, double* q_nr, double* q_ieee, int n,
                                             void* stream) {
  if (!a || !b || !q_nr || !q_ieee || n < 0) return MOLOCH_ERR_ARG;
  if (n == 0) return MOLOCH_OK;
  const int blocks = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
  moloch::kfast::k_check_division_f64<<<blocks, 256, 0, (cudaStream_t)stream>>>(a, b, q_nr, q_ieee, n);
  return cudaPeekAtLastError() == cudaSuccess ? MOLOCH_OK : MOLOCH_ERR_CUDA;
}
