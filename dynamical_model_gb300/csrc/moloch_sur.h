// Learned acoustic-cycle surrogate: device buffers and the launch entry the
// step uses (defined in moloch_mlp.cu).
#pragma once
#include <cuda_runtime.h>

#include "moloch_view.h"

namespace moloch {
namespace mlp {

struct SurLayer {
  int in = 0, out = 0;  // out x in, row-major (in contiguous)
  float* W = nullptr;   // FP32 master weights
  float* b = nullptr;   // bias
  float *gW = nullptr, *gb = nullptr;  // gradients
  float *mW = nullptr, *vW = nullptr, *mb = nullptr, *vb = nullptr;  // Adam moments
  void* Wb = nullptr;   // BF16 copy [out][in]  (forward B operand)
  void* WT = nullptr;   // BF16 transpose [in][out] (backward B operand)
};

struct Surrogate {
  int kz = 0;
  int nin = 0, kin = 0;   // 45 * kz features, padded to a multiple of 64
  int nout = 0, nop = 0;  // 5 * kz increments, padded to a multiple of 64
  int hid = 256;
  SurLayer L[4];
  float *xmean = nullptr, *xstd = nullptr, *ymean = nullptr, *ystd = nullptr;  // 5 * kz each
  // dataset (raw, then normalised and shuffled in place)
  int cap = 0, npairs = 0, ntrain = 0;
  float* Xraw = nullptr;  // [cap][kin]
  void* Xb = nullptr;     // BF16 [cap][kin]
  float* T = nullptr;     // [cap][nop]
  float* snap = nullptr;  // [cols][5 kz]
  int* cols = nullptr;    // sampled columns
  int max_cols = 0;
  // training scratch (batch rows)
  int batch = 0;
  void *Xbat = nullptr, *XbatT = nullptr, *dY = nullptr, *dYT = nullptr;
  void *H[3] = {}, *HT[3] = {}, *dZ[3] = {}, *dZT[3] = {};
  float *Tbat = nullptr, *Y = nullptr, *loss = nullptr;
  float* lpart = nullptr;  // per-block partial sums of the loss
  float *Z[3] = {}, *dH[3] = {};
  int* perm = nullptr;
  int adam_t = 0;  // Adam step count
  // inference scratch (one row per column of the attached domain)
  int ninf = 0;
  void* Xinf = nullptr;
  void* Hinf[3] = {};
  float* Yinf = nullptr;
  int* ctl = nullptr;                   // device control block (see moloch_mlp.cu)
  unsigned long long* counts = nullptr;  // [4] cycles, plain cycles, judge cycles, judge rejections
  double* jacc = nullptr;               // judge sums
  float* jsnap = nullptr;               // judge cycles: pre-cycle state, 5 fields
  int judge_every = 6;                  // plain-loop judge every n-th sound() call (0: never)
  int max_interval = 96;                // judge interval cap after failing verdicts
  float tol = 0.3f;                     // judge: largest relative RMS error of the increments
  float* env = nullptr;   // [nop] largest |normalised target| seen in training
  float threshold = 4.f;  // accepted: |y| <= threshold * env for every output
  bool ready = false;  // normalisation statistics exist
};

// one surrogate cycle before sound(): features, MLP, check, decision,
// commit (the plain substeps then skip); returns the kernel count
int sur_cycle(Surrogate* s, View<float>& v, cudaStream_t st, int nsound, int outpar);
// after sound(): the judge's comparison on judge cycles
int sur_after(Surrogate* s, View<float>& v, cudaStream_t st);

}  // namespace mlp
}  // namespace moloch
