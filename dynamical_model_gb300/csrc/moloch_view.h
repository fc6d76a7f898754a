// Device-side view of one MOLOCH domain: pointers into HBM plus the scalars
// a step needs.  Shared by the kernel translation units and the host API.
//
// Layout (all 3-D fields): dense, j fastest, then i, then k -- the
// reference's Fortran column-major order without the halo rings:
//     idx(j, i, k) = (j-1) + nj * ((i-1) + ni * (k-1))      (1-based j, i, k)
// Threads map to j, so every warp access is a contiguous row segment.
// Periodic halos are not stored: stencils wrap their indices.  The three
// places where the reference reads a halo that is OLDER than the interior
// (nompi/mod_moloch.F90:716-735: pai filled before its update, ud/vd copied
// after divdamp changed the interior but not the ring) are kept in small
// edge buffers written by the kernel that owns the old values.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

namespace moloch {

// default limit of a bounded device wait: about one second of SM clock
constexpr long long kDefaultSpinCycles = 2000000000LL;

constexpr int kNumAdvected = 10;  // tetav pai ux vx wx qv qc qi qr qs (mod_moloch.F90:911-920)

template <class T>
struct View {
  int nj, ni, kz;
  int pl;  // nj * ni, one level
  int rotllr;

  // prognostic state
  T* ubuf[2];
  T* vbuf[2];
  int cur;  // which of ubuf/vbuf holds the current u, v
  T* w;     // kz+1 levels
  T* pai;
  T* tetav;
  T* t;
  T* q[5];  // qv qc qi qr qs
  // diagnostics
  T* p;
  T* qsat;
  T* tvirt;
  T* rho;
  T* ps;  // one level
  T* qwltot;
  T* qwitot;
  // work
  T* s;       // kz+1 levels
  T* deltaw;  // kz+1 levels
  T* zdiv2a;  // horizontal divergence (Equation 16)
  T* zdiv2b;  // after divdamp and the vertical s term
  double* wp;    // Thomas down-sweep values (FP64 in every mode), kz+1 levels
  double* wwkw;  // Thomas pivot ratios (FP64 in every mode), kz+1 levels
  T* ux;
  T* vx;
  T* wx;
  T* wz;  // kNumAdvected fields (vertical WAF result)
  // the ten advected fields live in two buffer sets; the horizontal WAF
  // step writes the other set (fset[fcur ^ 1]) and the sets swap roles
  T* fset[2][kNumAdvected];
  int fcur;
  T* pf;
  T* tf;
  T* fscr;  // filter output scratch
  // edge buffers of stale halos (see header)
  T* eu_j;  // u before divdamp at j = 1, one per (i, k)    [ud(nj+1, i)]
  T* eu_i;  // u before divdamp at i = ni, one per (j, k)   [ud(j, 0)]
  T* ev_j;  // v before divdamp at j = nj, per (i, k)       [vd(0, i)]
  T* ev_i;  // v before divdamp at i = 1, per (j, k)        [vd(j, ni+1)]
  T* ep_j;  // pai before its update at j = nj, per (i, k)  [pai(0, i)]
  T* ep_i;  // pai before its update at i = ni, per (j, k)  [pai(j, 0)]

  // static 3-D metric terms (computed once on the host in FP64)
  const T* fmz;
  const T* fmzf;  // kz+1 levels
  const T* zeta;
  const T* dz;
  const T* rfw;   // 2 / (fmz(j) + fmz(j-1))
  const T* rfs;   // 2 / (fmz(i) + fmz(i-1))
  const T* wafu;  // wafone zrfmu
  const T* wafd;  // wafone zrfmd
  const T* wafn;  // wafone zrfmn
  const T* wafs;  // wafone zrfms
  const T* wafe;  // wafone zrfme
  const T* wafw;  // wafone zrfmw
  // static 2-D terms
  const T* hx;
  const T* hy;
  const T* mx;
  const T* mu;
  const T* mv;
  const T* rmu;
  const T* rmv;
  const T* mx2;
  const T* coru;
  const T* corv;
  // 1-D level tables
  const T* gzitak;   // kz+1
  const T* gzitakh;  // kz
  const T* xknu;     // kz
  const T* cdamp;    // xknu(k) * ddamp
  const T* ffilt;    // kz (zero in the reference)

  // scalars of sound() (dts) and wafone() (dta)
  T dts, dtrdx, dtrdy, dtrdz, zcs2, ddamp2, egdts;
  double dts_d, dtrdz_d, zcs2_d, egdts_d;
  T dtrdx_a, dtrdy_a, dtrdz_a;  // wafone: dta/dx, dta/dx, 0.5*dta/dzita
  T anu2;

  // launch shape chosen by the autotuner: levels per k_waf_horizontal block
  int hz_levels;
  int kmarch;      // sound kernel variants, bit mask: 1 divergence, 2 damping, 4 momentum
                   // k-marching; 8 momentum as warp strips; 16 divergence + damping fused;
                   // 32 column solve staged by TMA with its column state in TMEM;
                   // 64 with 8: momentum strips with two columns per lane; 128 / 256 with
                   // 32: two words of column state a level, 12 / 16 compute warps; 512
                   // with 16: the fused strips over two levels per warp
  int vfields;     // advected fields per thread of k_waf_vertical: 1, 2, 5 or 10
  int srows;       // rows per warp strip of the momentum strips
  int stag4;       // 1: k_stag_from_x4 (FP32, jx a multiple of 4)

  // set when a learned surrogate stands in for sound(): the plain sound
  // kernels return at once while *sur_skip == 1 (the surrogate's cycle was
  // accepted); nullptr when no surrogate is attached
  const int* sur_skip;

  // staged column kernel (k_sound_column_tm, FP32 storage): host pointer to
  // the two sets of TMA tensor maps (one per advected-field buffer set),
  // nullptr when the kernel cannot run on this domain
  const void* cmaps;
  // device word set by a bounded wait that gave up (MOLOCH_ERR_TIMEOUT)
  int* kerr;
  long long spin_cycles;  // limit of every such wait, in SM clock cycles
  int fault_skip_job;     // test hook: a job the producer leaves unissued (-1: none)

  // diagnostics
  double* dpart;  // per-block partial reductions
  double* dres;   // final reduction (device)
  int dparts;

  // point the named field pointers at the current buffer set
  void bind_fields() {
    tetav = fset[fcur][0];
    pai = fset[fcur][1];
    ux = fset[fcur][2];
    vx = fset[fcur][3];
    wx = fset[fcur][4];
    for (int n = 0; n < 5; ++n) q[n] = fset[fcur][5 + n];
  }
};

// Kernel kinds, for per-kernel CUDA-event timing (moloch_gpu_profile_step).
enum KernelKind {
  KK_PREDIAG = 0, KK_SOUND_DIV, KK_SOUND_DAMP, KK_SOUND_COLUMN, KK_LAP_FILTER, KK_PAI_UPDATE,
  KK_SOUND_MOMENTUM, KK_WAF_VERTICAL, KK_WAF_HORIZONTAL, KK_STAG_FROM_X,
  KK_FILTER_INCREMENT, KK_POSTDIAG, KK_DIAG, KK_SOUND_DIVDAMP, KK_SOUND_COLUMN_TM, KK_COUNT
};

// Optional event recorder: when a launcher is given one, it records a CUDA
// event on the launching stream before and after every kernel.
struct KernelTimer {
  static constexpr int kCap = 4096;
  cudaEvent_t ev[kCap];
  int kind[kCap / 2];
  int n = 0;  // events recorded
  bool ok = true;
  void mark(int k, cudaStream_t st, bool begin) {
    if (n >= kCap) { ok = false; return; }
    if (begin) kind[n / 2] = k;
    cudaEventRecord(ev[n++], st);
  }
};

// Batched launch over the members of an ensemble.  Every batched kernel
// takes a 1-D grid that walks a tile table of (member, bx, by, bz) entries
// and reads the member's view from views[cur][fcur] (the u/v buffer and
// field-set parities the step is at when the kernel runs).
// TK_CHUNK tiles cover kKC levels each (the k-marching sound kernels);
// TK_MSTRIP tiles are blocks of 4 momentum warp strips (30 columns x kMomR
// rows) of one level; TK_DSTRIP tiles blocks of 4 divergence/damping warp
// strips (29 columns x kDDR rows).  The persistent ensemble kernel runs
// 32 x 8 thread blocks: its column tiles (TK_COLUMN8, TK_VERTICAL8) are 8
// rows high, given as (member, bx, 2 by8, .) so that the 32 x 4 column
// bodies' row index by * 4 + threadIdx.y covers rows 8 by8 .. 8 by8 + 7, and
// its strip tiles (TK_MSTRIP8, TK_DSTRIP8) are blocks of 8 warp strips.
// TK_COLTW tiles are the 32 x kTwRows column tiles of the batched staged
// column solve, (member, tile x, tile y, .), of the FP32 members with tensor
// maps (jx a multiple of 4, kz <= 64); TK_COLREST the TK_COLUMN tiles of the
// other members, which the one-thread column kernel takes beside it.
// TK_DSTRIP2 tiles are blocks of 4 divergence/damping warp strips over a
// pair of levels, (member, block, level pair, .).
constexpr int kKC = 4;
constexpr int kTwRows = 12;
constexpr int kMomJ = 30, kMomR = 32;
constexpr int kDDJ = 29, kDDR = 32;
constexpr int kDDLevels = 2;  // levels per warp of the two-level fused divergence/damping strips
enum TileKind {
  TK_POINT = 0, TK_COLUMN, TK_VERTICAL, TK_HORIZONTAL, TK_CHUNK, TK_MSTRIP, TK_DSTRIP,
  TK_COLUMN8, TK_VERTICAL8, TK_MSTRIP8, TK_DSTRIP8, TK_COLTW, TK_COLREST, TK_DSTRIP2, TK_COUNT
};
template <class T>
struct Batch {
  const View<T>* views[2][2];   // device arrays, one view per member
  const int4* tiles[TK_COUNT];  // device tile tables
  int ntiles[TK_COUNT];
  int hstrip = 0;               // horizontal WAF as warp strips (tiles: member, block, level)
  int kmarch = 0;               // k-marching sound kernels on TK_CHUNK tiles (bit mask as View::kmarch)
  int vfields = 1;              // fields per thread of the vertical WAF (TK_VERTICAL tiles follow it)
  int mrows = kMomR;            // rows per momentum warp strip (TK_MSTRIP tiles follow it)
  // batched staged column solve (FP32 members with tensor maps): device
  // array of ColumnMaps, two buffer-set parities per member (zeros for the
  // members without), or nullptr when no member has maps; its bounded waits
  // report through kerr
  const void* cmaps = nullptr;
  int* kerr = nullptr;
  long long spin = 0;
};

// launch counts per phase are returned by the launchers so the API can
// account for every kernel it starts
struct PhaseFlags {
  int divfilter;
  int filterpai;
  int filtertheta;
  int nsound;
  int nadv;
};

}  // namespace moloch
