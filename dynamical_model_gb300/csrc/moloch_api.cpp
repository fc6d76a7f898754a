// C-ABI implementation of the GB300 MOLOCH step (include/moloch_gb300.h).
//
// Compiled by the host C++ compiler with -ffp-contract=off: the static
// metric terms computed here (init_moloch's derived arrays and the
// reciprocals the kernels reuse) must round exactly like the reference's
// FP64 expressions, which never fuse a multiply with an add.
//
// Host-side flow, mirroring the reference program:
//   allocate_moloch  -> moloch_gpu_create     (device arena for one domain)
//   init_moloch      -> moloch_gpu_upload * n, moloch_gpu_init
//   moloch(i,lprint) -> moloch_gpu_step        (or moloch_gpu_run for a loop)
// Device layout and kernel map: moloch_view.h, moloch_kernels.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <cstdlib>
#include <string>
#include <thread>
#include <vector>

#include "../../include/moloch_gb300.h"
#include "moloch_constants.h"
#include "moloch_launch.h"
#include "moloch_persist.h"
#include "moloch_sur.h"
#include "moloch_view.h"

using namespace moloch;

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CUDA_TRY(x)                                                                          \
  do {                                                                                       \
    cudaError_t e_ = (x);                                                                    \
    if (e_ != cudaSuccess) return fail(MOLOCH_ERR_CUDA, "%s: %s (%s:%d)", #x,               \
                                       cudaGetErrorString(e_), __FILE__, __LINE__);          \
  } while (0)

// expected Fortran bounds of each field (see the table in moloch_gb300.h)
struct FieldShape {
  int ndim;
  int lb[4], ub[4];
};

FieldShape shape_of(int f, int nj, int ni, int kz) {
  FieldShape s{};
  auto set3 = [&](int l1, int u1, int l2, int u2, int l3, int u3) {
    s.ndim = 3;
    s.lb[0] = l1; s.ub[0] = u1; s.lb[1] = l2; s.ub[1] = u2; s.lb[2] = l3; s.ub[2] = u3;
  };
  auto set2 = [&](int l1, int u1, int l2, int u2) {
    s.ndim = 2;
    s.lb[0] = l1; s.ub[0] = u1; s.lb[1] = l2; s.ub[1] = u2;
  };
  switch (f) {
    case MOLOCH_F_U: set3(-1, nj + 2, 0, ni + 1, 1, kz); break;
    case MOLOCH_F_V: set3(0, nj + 1, -1, ni + 2, 1, kz); break;
    case MOLOCH_F_W: set3(1, nj, 1, ni, 1, kz + 1); break;
    case MOLOCH_F_PAI: case MOLOCH_F_T: case MOLOCH_F_TETAV: case MOLOCH_F_FMZ:
    case MOLOCH_F_QV: case MOLOCH_F_QC: case MOLOCH_F_QI: case MOLOCH_F_QR: case MOLOCH_F_QS:
      set3(0, nj + 1, 0, ni + 1, 1, kz); break;
    case MOLOCH_F_QX:
      set3(0, nj + 1, 0, ni + 1, 1, kz);
      s.ndim = 4; s.lb[3] = 1; s.ub[3] = 5; break;
    case MOLOCH_F_P: case MOLOCH_F_TVIRT: case MOLOCH_F_QSAT: case MOLOCH_F_RHO:
      set3(1, nj, 1, ni, 1, kz); break;
    case MOLOCH_F_PS: set2(0, nj + 1, 0, ni + 1); break;
    case MOLOCH_F_ZETA: set3(-1, nj + 2, -1, ni + 2, 1, kz); break;
    case MOLOCH_F_FMZF: set3(1, nj, 1, ni, 1, kz + 1); break;
    case MOLOCH_F_HT: set2(-1, nj + 2, -1, ni + 2); break;
    case MOLOCH_F_MSFX: case MOLOCH_F_ULAT: case MOLOCH_F_VLAT: set2(1, nj, 1, ni); break;
    case MOLOCH_F_MSFU: case MOLOCH_F_HX: set2(0, nj + 1, 1, ni); break;
    case MOLOCH_F_MSFV: case MOLOCH_F_HY: set2(1, nj, 0, ni + 1); break;
    case MOLOCH_F_ZITA: s.ndim = 1; s.lb[0] = 1; s.ub[0] = kz + 1; break;
    case MOLOCH_F_ZITAH: s.ndim = 1; s.lb[0] = 1; s.ub[0] = kz; break;
    case MOLOCH_F_S: set3(1, nj, 1, ni, 1, kz + 1); break;
    case MOLOCH_F_DELTAW: set3(0, nj + 1, 0, ni + 1, 1, kz + 1); break;
    default: s.ndim = 0;
  }
  return s;
}

inline int wrap(int x, int n) {
  int y = (x - 1) % n;
  if (y < 0) y += n;
  return y;  // 0-based interior index of 1-based x with period n
}

// interior (1..nj, 1..ni, 1..nk) of a bounded host array -> dense j-fastest
void gather_interior(const double* base, const FieldShape& s, int nj, int ni, int nk, int level4,
                     std::vector<double>& out) {
  long n1 = s.ub[0] - s.lb[0] + 1, n2 = s.ndim >= 2 ? s.ub[1] - s.lb[1] + 1 : 1;
  long n3 = s.ndim >= 3 ? s.ub[2] - s.lb[2] + 1 : 1;
  out.resize((size_t)nj * ni * nk);
  long off4 = (long)level4 * n1 * n2 * n3;
  for (int k = 1; k <= nk; ++k)
    for (int i = 1; i <= ni; ++i) {  // rows are contiguous in j
      long q = off4 + (long)(s.ndim >= 3 ? k - s.lb[2] : 0) * n1 * n2 +
               (long)(s.ndim >= 2 ? i - s.lb[1] : 0) * n1 + (1 - s.lb[0]);
      std::memcpy(&out[(size_t)nj * ((i - 1) + (size_t)ni * (k - 1))], base + q, sizeof(double) * nj);
    }
}

// dense interior -> bounded host array; halo positions get periodic images
void scatter_periodic(const std::vector<double>& in, const FieldShape& s, int nj, int ni, int nk,
                      int level4, double* base) {
  long n1 = s.ub[0] - s.lb[0] + 1, n2 = s.ndim >= 2 ? s.ub[1] - s.lb[1] + 1 : 1;
  long n3 = s.ndim >= 3 ? s.ub[2] - s.lb[2] + 1 : 1;
  long off4 = (long)level4 * n1 * n2 * n3;
  int k1 = s.ndim >= 3 ? s.lb[2] : 1, k2 = s.ndim >= 3 ? s.ub[2] : 1;
  int i1 = s.ndim >= 2 ? s.lb[1] : 1, i2 = s.ndim >= 2 ? s.ub[1] : 1;
  for (int k = k1; k <= k2; ++k)
    for (int i = i1; i <= i2; ++i)
      for (int j = s.lb[0]; j <= s.ub[0]; ++j) {
        long q = off4 + (long)(k - k1) * n1 * n2 + (long)(i - i1) * n1 + (j - s.lb[0]);
        int kk = (k >= 1 && k <= nk) ? k - 1 : (k < 1 ? 0 : nk - 1);
        base[q] = in[(size_t)wrap(j, nj) + (size_t)nj * (wrap(i, ni) + (size_t)ni * kk)];
      }
}

// host threads for the layout conversion of uploads and downloads
// (MOLOCH_HOST_THREADS overrides; default: the hardware threads, at most 32)
unsigned host_threads() {
  static unsigned n = [] {
    const char* e = std::getenv("MOLOCH_HOST_THREADS");
    long v = e ? std::strtol(e, nullptr, 10) : 0;
    if (v <= 0) v = (long)std::thread::hardware_concurrency();
    return (unsigned)std::max(1L, std::min(v, 32L));
  }();
  return n;
}

// fn(begin, end) over [0, n) split across the host threads
template <class F>
void host_parallel(size_t n, F&& fn) {
  const unsigned nt = (unsigned)std::min<size_t>(host_threads(), (n + 7) / 8);
  if (nt <= 1) {
    fn((size_t)0, n);
    return;
  }
  std::vector<std::thread> th;
  th.reserve(nt - 1);
  for (unsigned t = 1; t < nt; ++t) th.emplace_back([&, t] { fn(n * t / nt, n * (t + 1) / nt); });
  fn((size_t)0, n / nt);
  for (auto& x : th) x.join();
}

double gzita(double zita, double ztop, double a0) {  // nompi/mod_zita.F90:109-120
  double ratio = zita / ztop;
  double r2 = ratio * ratio, r3 = r2 * ratio;
  return (((0.0 - 1.0 * a0) * ratio - (3.0 - 2.0 * a0) * r2) + (2.0 - 1.0 * a0) * r3) + 1.0;
}

}  // namespace

// ---------------------------------------------------------------------------
struct moloch_handle {
  moloch_grid_t grid{};
  moloch_params_t prm{};
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int elem = 8;  // bytes per element of the bulk type
  void* arena = nullptr;
  size_t arena_bytes = 0;
  View<double> vd{};
  View<float> vf{};
  bool initialized = false;
  long long kernels = 0;
  int kernels_per_step = 0;
  // one graph per field-buffer parity at the start of a step (advection
  // swaps the two buffer sets, so odd mo_nadv alternates between them)
  cudaGraph_t graph[2] = {nullptr, nullptr};
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  double* hres = nullptr;  // pinned diag result
  // output path: device snapshot of t and ps, copied to pinned host memory
  // on a second stream while the step stream runs on
  void* out_dev = nullptr;
  void* out_host = nullptr;
  void* out_f64 = nullptr;  // Fortran-layout FP64 t and ps, for registered output arrays
  cudaStream_t out_stream = nullptr;
  cudaEvent_t out_taken = nullptr, out_done = nullptr;
  bool out_pending = false;
  void* stage = nullptr;   // pinned staging buffer, one 3-D field (kz+1 levels) of doubles
  size_t stage_bytes = 0;
  // the two halves of `stage` as a ring for streamed transfers: the event
  // of a half is recorded after the copy that last used it
  cudaEvent_t stage_ev[2] = {nullptr, nullptr};
  bool stage_busy[2] = {false, false};
  // host copies of the static inputs (dense interiors)
  std::vector<double> zeta, fmz, fmzf, msfx, msfu, msfv, hx, hy, ulat, vlat, zita, zitah;
  unsigned uploaded = 0;  // bit per field id
  // uploads of prognostic fields by kernels that read the caller's host
  // arrays through the host page tables (-1: not decided yet, 0: pinned
  // staging and host threads, 1: direct)
  int host_direct = -1;
  // direct uploads run on their own stream into a device staging copy of
  // the field, so they overlap the steps already issued; a device copy on
  // the step stream then commits the field in stream order.  Per field id:
  // staging buffer, "read done" event (upload stream), "committed" event
  // (step stream, after which the staging buffer may be refilled)
  cudaStream_t up_stream = nullptr;
  void* up_stage[MOLOCH_F_COUNT] = {};
  size_t up_stage_bytes[MOLOCH_F_COUNT] = {};
  // host ranges the caller registered (pinned): uploads from them are DMA
  // copies of the whole Fortran array into an FP64 staging buffer on the
  // upload stream, then a gather/convert kernel on the step stream
  std::vector<std::pair<const char*, size_t>> pinned;
  cudaEvent_t up_read[MOLOCH_F_COUNT] = {};
  cudaEvent_t up_commit[MOLOCH_F_COUNT] = {};
  // attached acoustic-cycle surrogate (FP32 storage only): each sound()
  // call first runs the surrogate; the plain substeps skip on acceptance
  moloch::mlp::Surrogate* sur = nullptr;
  // TMA tensor maps of the staged column kernel (FP32 storage), one set per
  // advected-field buffer set
  alignas(64) unsigned char cmaps[10240];
  int nj() const { return grid.jx; }
  int ni() const { return grid.iy; }
  int kz() const { return grid.kz; }
};

namespace {

PhaseFlags flags_of(const moloch_handle* h) {
  PhaseFlags f;
  f.divfilter = h->prm.mo_divfilter;
  f.filterpai = h->prm.do_filterpai;
  f.filtertheta = h->prm.do_filtertheta;
  f.nsound = h->prm.mo_nsound;
  f.nadv = h->prm.mo_nadv;
  return f;
}

// carve the arena; returns bytes needed when base == nullptr
template <class T>
size_t layout(View<T>& v, char* base, const moloch_handle* h) {
  size_t off = 0;
  const size_t pl = (size_t)h->nj() * h->ni(), kz = h->kz();
  const size_t n3 = pl * kz, n3p = pl * (kz + 1), ne = (size_t)std::max(h->nj(), h->ni()) * kz;
  auto take = [&](size_t bytes) -> void* {
    off = (off + 255) & ~size_t(255);
    void* p = base ? base + off : nullptr;
    off += bytes;
    return p;
  };
  auto T3 = [&]() { return (T*)take(sizeof(T) * n3); };
  auto T3p = [&]() { return (T*)take(sizeof(T) * n3p); };
  auto T2 = [&]() { return (T*)take(sizeof(T) * pl); };
  auto T1 = [&](size_t n) { return (T*)take(sizeof(T) * n); };
  v.ubuf[0] = T3(); v.ubuf[1] = T3(); v.vbuf[0] = T3(); v.vbuf[1] = T3();
  v.w = T3p(); v.t = T3();
  for (int set = 0; set < 2; ++set)
    for (int n = 0; n < kNumAdvected; ++n) v.fset[set][n] = T3();
  v.fcur = 0;
  v.bind_fields();
  v.p = T3(); v.qsat = T3(); v.tvirt = T3(); v.rho = T3(); v.ps = T2();
  v.qwltot = T3(); v.qwitot = T3();
  v.s = T3p(); v.deltaw = T3p(); v.zdiv2a = T3(); v.zdiv2b = T3();
  v.wp = (double*)take(sizeof(double) * n3p);
  v.wwkw = (double*)take(sizeof(double) * n3p);
  v.wz = (T*)take(sizeof(T) * n3 * kNumAdvected);
  const bool filt = h->prm.do_filterpai || h->prm.do_filtertheta;
  v.pf = h->prm.do_filterpai ? T3() : nullptr;
  v.tf = h->prm.do_filtertheta ? T3() : nullptr;
  v.fscr = filt ? T3() : nullptr;
  v.eu_j = T1(ne); v.eu_i = T1(ne); v.ev_j = T1(ne); v.ev_i = T1(ne); v.ep_j = T1(ne); v.ep_i = T1(ne);
  v.fmz = T3(); v.fmzf = T3p(); v.zeta = T3(); v.dz = T3();
  v.rfw = T3(); v.rfs = T3();
  v.wafu = T3(); v.wafd = T3(); v.wafn = T3(); v.wafs = T3(); v.wafe = T3(); v.wafw = T3();
  v.hx = T2(); v.hy = T2(); v.mx = T2(); v.mu = T2(); v.mv = T2(); v.rmu = T2(); v.rmv = T2();
  v.mx2 = T2(); v.coru = T2(); v.corv = T2();
  v.gzitak = T1(kz + 1); v.gzitakh = T1(kz); v.xknu = T1(kz); v.cdamp = T1(kz); v.ffilt = T1(kz);
  const int parts = kfast::diag_parts(h->nj(), h->ni());
  v.dpart = (double*)take(sizeof(double) * 9 * parts);
  v.dres = (double*)take(sizeof(double) * 16);
  v.kerr = (int*)take(sizeof(int));
  v.dparts = parts;
  v.nj = h->nj(); v.ni = h->ni(); v.kz = h->kz(); v.pl = (int)pl; v.rotllr = h->prm.rotllr;
  v.cur = 0;
  v.hz_levels = 1;
  v.kmarch = 0;
  v.vfields = 1;
  v.srows = kMomR;
  v.stag4 = 0;
  v.sur_skip = nullptr;
  v.cmaps = nullptr;
  v.spin_cycles = kDefaultSpinCycles;
  v.fault_skip_job = -1;
  return off + 256;
}

// host <-> device through the handle's pinned staging buffer (one 3-D
// field); the bulk type conversion happens while filling the buffer
template <class T>
int upload_dense(moloch_handle* h, T* dst, const std::vector<double>& src) {
  const size_t bytes = sizeof(T) * src.size();
  if (bytes > h->stage_bytes) return fail(MOLOCH_ERR_ARG, "upload of %zu bytes exceeds staging", bytes);
  CUDA_TRY(cudaStreamSynchronize(h->stream));  // staging buffer free again
  T* st = (T*)h->stage;
  host_parallel(src.size(), [&](size_t q0, size_t q1) {
    for (size_t q = q0; q < q1; ++q) st[q] = (T)src[q];
  });
  CUDA_TRY(cudaMemcpyAsync(dst, st, bytes, cudaMemcpyHostToDevice, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return MOLOCH_OK;
}

template <class T>
int download_dense(moloch_handle* h, const T* src, size_t n, std::vector<double>& out) {
  const size_t bytes = sizeof(T) * n;
  if (bytes > h->stage_bytes) return fail(MOLOCH_ERR_ARG, "download of %zu bytes exceeds staging", bytes);
  out.resize(n);
  CUDA_TRY(cudaMemcpyAsync(h->stage, src, bytes, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  const T* st = (const T*)h->stage;
  if (sizeof(T) == sizeof(double))
    std::memcpy(out.data(), st, bytes);
  else
    for (size_t q = 0; q < n; ++q) out[q] = (double)st[q];
  return MOLOCH_OK;
}

// Streamed transfer of one field between a bounded host array (Fortran
// layout, halo rings included) and its dense device copy.  The field is cut
// into level chunks that fit one half of the pinned staging buffer; host
// threads convert a chunk (interior gather + bulk-type conversion, or
// periodic scatter + conversion back) while the other half is in flight.
// An upload returns once its chunks are staged: the copies complete in
// stream order before any later work of the handle.
int stage_wait(moloch_handle* h, int slot) {
  if (h->stage_busy[slot]) {
    CUDA_TRY(cudaEventSynchronize(h->stage_ev[slot]));
    h->stage_busy[slot] = false;
  }
  return MOLOCH_OK;
}

template <class T>
int upload_streamed(moloch_handle* h, T* dst, const double* base, const FieldShape& s, int nj, int ni, int nk,
                    int level4) {
  const long n1 = s.ub[0] - s.lb[0] + 1, n2 = s.ndim >= 2 ? s.ub[1] - s.lb[1] + 1 : 1;
  const long n3 = s.ndim >= 3 ? s.ub[2] - s.lb[2] + 1 : 1;
  const long off4 = (long)level4 * n1 * n2 * n3;
  const size_t plane = (size_t)nj * ni;
  const int chunk = (int)std::max<size_t>(1, (h->stage_bytes / 2) / (sizeof(T) * plane));
  int slot = 0;
  for (int k0 = 0; k0 < nk; k0 += chunk, slot ^= 1) {
    const int k1 = std::min(nk, k0 + chunk);
    int rc = stage_wait(h, slot);
    if (rc) return rc;
    T* st = (T*)((char*)h->stage + slot * (h->stage_bytes / 2));
    host_parallel((size_t)(k1 - k0) * ni, [&](size_t r0, size_t r1) {
      for (size_t r = r0; r < r1; ++r) {
        const int kk = k0 + (int)(r / ni), i = (int)(r % ni) + 1;
        const long q = off4 + (long)(s.ndim >= 3 ? kk + 1 - s.lb[2] : 0) * n1 * n2 +
                       (long)(s.ndim >= 2 ? i - s.lb[1] : 0) * n1 + (1 - s.lb[0]);
        const double* src = base + q;
        T* o = st + r * nj;
        for (int j = 0; j < nj; ++j) o[j] = (T)src[j];
      }
    });
    CUDA_TRY(cudaMemcpyAsync(dst + (size_t)k0 * plane, st, sizeof(T) * plane * (k1 - k0), cudaMemcpyHostToDevice,
                             h->stream));
    CUDA_TRY(cudaEventRecord(h->stage_ev[slot], h->stream));
    h->stage_busy[slot] = true;
  }
  return MOLOCH_OK;
}

template <class T>
int download_streamed(moloch_handle* h, const T* src, const FieldShape& s, int nj, int ni, int nk, int level4,
                      double* base) {
  const long n1 = s.ub[0] - s.lb[0] + 1, n2 = s.ndim >= 2 ? s.ub[1] - s.lb[1] + 1 : 1;
  const long n3 = s.ndim >= 3 ? s.ub[2] - s.lb[2] + 1 : 1;
  const long off4 = (long)level4 * n1 * n2 * n3;
  const int k1b = s.ndim >= 3 ? s.lb[2] : 1, i1 = s.ndim >= 2 ? s.lb[1] : 1, i2 = s.ndim >= 2 ? s.ub[1] : 1;
  const size_t plane = (size_t)nj * ni;
  const int chunk = (int)std::max<size_t>(1, (h->stage_bytes / 2) / (sizeof(T) * plane));
  const int nchunks = (nk + chunk - 1) / chunk;
  auto issue = [&](int c) -> int {
    const int slot = c & 1, k0 = c * chunk, k1 = std::min(nk, k0 + chunk);
    int rc = stage_wait(h, slot);
    if (rc) return rc;
    T* st = (T*)((char*)h->stage + slot * (h->stage_bytes / 2));
    CUDA_TRY(cudaMemcpyAsync(st, src + (size_t)k0 * plane, sizeof(T) * plane * (k1 - k0), cudaMemcpyDeviceToHost,
                             h->stream));
    CUDA_TRY(cudaEventRecord(h->stage_ev[slot], h->stream));
    h->stage_busy[slot] = true;
    return MOLOCH_OK;
  };
  int rc = issue(0);
  if (rc) return rc;
  for (int c = 0; c < nchunks; ++c) {
    if (c + 1 < nchunks && (rc = issue(c + 1))) return rc;
    const int slot = c & 1, k0 = c * chunk, k1 = std::min(nk, k0 + chunk);
    if ((rc = stage_wait(h, slot))) return rc;
    const T* st = (const T*)((const char*)h->stage + slot * (h->stage_bytes / 2));
    const int nrow_i = i2 - i1 + 1;
    host_parallel((size_t)(k1 - k0) * nrow_i, [&](size_t r0, size_t r1) {
      for (size_t r = r0; r < r1; ++r) {
        const int kk = k0 + (int)(r / nrow_i), i = i1 + (int)(r % nrow_i);
        const long q = off4 + (long)(s.ndim >= 3 ? kk + 1 - k1b : 0) * n1 * n2 + (long)(i - i1) * n1;
        const T* row = st + ((size_t)(kk - k0) * ni + wrap(i, ni)) * nj;
        double* o = base + q;
        for (int j = s.lb[0]; j <= s.ub[0]; ++j) o[j - s.lb[0]] = (double)row[wrap(j, nj)];
      }
    });
  }
  return MOLOCH_OK;
}

// Direct uploads need the device to read pageable host memory through the
// host page tables (NVLink-C2C on GB300).  Downloads and the output path
// stay staged: a kernel writing into host pages the caller has not touched
// yet (a fresh array) takes a page fault per page (measured 32 ms for a
// 125 MB field against 4 ms staged), and the output copy overlaps the next
// steps anyway.
bool use_direct(moloch_handle* h) {
  if (h->host_direct < 0) {
    int dev = 0, pma = 0, pt = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, dev);
    cudaDeviceGetAttribute(&pt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev);
    h->host_direct = (pma && pt) ? 1 : 0;
  }
  return h->host_direct == 1;
}

// interior of a Fortran-layout field into the dense device copy: a kernel
// on the upload stream reads the caller's array into the field's staging
// buffer (concurrently with the steps already issued on the step stream),
// then the step stream copies the staging buffer into the field after the
// work issued before.  Returns when the kernel is done (the caller may
// change the array afterwards).  fid: field id of the staging slot.
bool is_pinned(const moloch_handle* h, const void* p, size_t bytes) {
  const char* a = (const char*)p;
  for (const auto& r : h->pinned)
    if (a >= r.first && a + bytes <= r.first + r.second) return true;
  return false;
}

template <class T>
int upload_direct(moloch_handle* h, int fid, T* dst, const double* base, const FieldShape& s, int nj, int ni, int nk,
                  int level4) {
  const long n1 = s.ub[0] - s.lb[0] + 1, n2 = s.ndim >= 2 ? s.ub[1] - s.lb[1] + 1 : 1;
  const long n3 = s.ndim >= 3 ? s.ub[2] - s.lb[2] + 1 : 1;
  const long off4 = (long)level4 * n1 * n2 * n3;
  const long A = (s.ndim >= 3 ? (1 - s.lb[2]) * n1 * n2 : 0) + (s.ndim >= 2 ? (1 - s.lb[1]) * n1 : 0) + (1 - s.lb[0]);
  const long P = s.ndim >= 3 ? n1 * n2 : 0, Rw = s.ndim >= 2 ? n1 : 0;
  const size_t slice = sizeof(double) * (size_t)n1 * n2 * n3;  // the host array of this field (one tracer)
  const double* src = base + off4;
  const bool dma = is_pinned(h, src, slice);
  const size_t bytes = dma ? slice : sizeof(T) * (size_t)nj * ni * nk;
  if (!h->up_stream) {  // highest priority: its few blocks slip in between the blocks of running steps
    int lo = 0, hi = 0;
    CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    CUDA_TRY(cudaStreamCreateWithPriority(&h->up_stream, cudaStreamNonBlocking, hi));
  }
  if (!h->up_read[fid]) {
    CUDA_TRY(cudaEventCreateWithFlags(&h->up_read[fid], cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&h->up_commit[fid], cudaEventDisableTiming));
    CUDA_TRY(cudaEventRecord(h->up_commit[fid], h->stream));
  }
  if (h->up_stage_bytes[fid] < bytes) {
    CUDA_TRY(cudaStreamWaitEvent(h->up_stream, h->up_commit[fid], 0));
    CUDA_TRY(cudaStreamSynchronize(h->up_stream));
    if (h->up_stage[fid]) CUDA_TRY(cudaFree(h->up_stage[fid]));
    CUDA_TRY(cudaMalloc(&h->up_stage[fid], bytes));
    h->up_stage_bytes[fid] = bytes;
  }
  // the previous commit of this field has read the staging buffer
  CUDA_TRY(cudaStreamWaitEvent(h->up_stream, h->up_commit[fid], 0));
  if (dma) {  // copy engine: the Fortran array as it is; gather/convert on the step stream
    CUDA_TRY(cudaMemcpyAsync(h->up_stage[fid], src, slice, cudaMemcpyHostToDevice, h->up_stream));
    CUDA_TRY(cudaEventRecord(h->up_read[fid], h->up_stream));
    CUDA_TRY(cudaStreamWaitEvent(h->stream, h->up_read[fid], 0));
    moloch::init::launch_upload_direct<T>(dst, (const double*)h->up_stage[fid], A, P, Rw, nj, ni, nk, h->stream, true);
  } else {  // a small kernel reads the host array through the host page tables
    moloch::init::launch_upload_direct<T>((T*)h->up_stage[fid], src, A, P, Rw, nj, ni, nk, h->up_stream, false);
    CUDA_TRY(cudaEventRecord(h->up_read[fid], h->up_stream));
    CUDA_TRY(cudaStreamWaitEvent(h->stream, h->up_read[fid], 0));
    CUDA_TRY(cudaMemcpyAsync(dst, h->up_stage[fid], bytes, cudaMemcpyDeviceToDevice, h->stream));
  }
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaEventRecord(h->up_commit[fid], h->stream));
  CUDA_TRY(cudaEventSynchronize(h->up_read[fid]));
  return MOLOCH_OK;
}

// device pointer of a prognostic/diagnostic field in the bulk type
template <class T>
T* field_ptr(View<T>& v, int f) {
  switch (f) {
    case MOLOCH_F_U: return v.ubuf[v.cur];  // current buffer of the ping-pong pair
    case MOLOCH_F_V: return v.vbuf[v.cur];
    case MOLOCH_F_W: return v.w;
    case MOLOCH_F_PAI: return v.pai;
    case MOLOCH_F_T: return v.t;
    case MOLOCH_F_TETAV: return v.tetav;
    case MOLOCH_F_QV: return v.q[0];
    case MOLOCH_F_QC: return v.q[1];
    case MOLOCH_F_QI: return v.q[2];
    case MOLOCH_F_QR: return v.q[3];
    case MOLOCH_F_QS: return v.q[4];
    case MOLOCH_F_P: return v.p;
    case MOLOCH_F_TVIRT: return v.tvirt;
    case MOLOCH_F_QSAT: return v.qsat;
    case MOLOCH_F_RHO: return v.rho;
    case MOLOCH_F_PS: return v.ps;
    case MOLOCH_F_S: return v.s;
    case MOLOCH_F_DELTAW: return v.deltaw;
    default: return nullptr;
  }
}

bool is_static(int f) {
  switch (f) {
    case MOLOCH_F_ZETA: case MOLOCH_F_FMZ: case MOLOCH_F_FMZF: case MOLOCH_F_HT:
    case MOLOCH_F_MSFX: case MOLOCH_F_MSFU: case MOLOCH_F_MSFV: case MOLOCH_F_HX: case MOLOCH_F_HY:
    case MOLOCH_F_ULAT: case MOLOCH_F_VLAT: case MOLOCH_F_ZITA: case MOLOCH_F_ZITAH:
      return true;
    default:
      return false;
  }
}

std::vector<double>* static_store(moloch_handle* h, int f) {
  switch (f) {
    case MOLOCH_F_ZETA: return &h->zeta;
    case MOLOCH_F_FMZ: return &h->fmz;
    case MOLOCH_F_FMZF: return &h->fmzf;
    case MOLOCH_F_MSFX: return &h->msfx;
    case MOLOCH_F_MSFU: return &h->msfu;
    case MOLOCH_F_MSFV: return &h->msfv;
    case MOLOCH_F_HX: return &h->hx;
    case MOLOCH_F_HY: return &h->hy;
    case MOLOCH_F_ULAT: return &h->ulat;
    case MOLOCH_F_VLAT: return &h->vlat;
    case MOLOCH_F_ZITA: return &h->zita;
    case MOLOCH_F_ZITAH: return &h->zitah;
    default: return nullptr;
  }
}

// init_moloch (nompi/mod_moloch.F90:219-268) and the static terms the
// kernels reuse, all in FP64 with the reference's evaluation order.
template <class T>
int init_impl(moloch_handle* h, View<T>& v) {
  const int nj = h->nj(), ni = h->ni(), kz = h->kz();
  const size_t pl = (size_t)nj * ni;
  const moloch_params_t& P = h->prm;
  auto I2 = [&](int j, int i) { return (size_t)wrap(j, nj) + (size_t)nj * wrap(i, ni); };
  auto I3 = [&](int j, int i, int k) { return I2(j, i) + pl * (size_t)(k - 1); };
  const std::vector<double>&fmz = h->fmz, &fmzf = h->fmzf;

  // scalars (moloch :285-286, sound :495-498, divdamp :863,884, wafone :951-956)
  const double dzita = h->zita[kz - 1];  // mo_dzita = zita(kz) (regcm_dynamical_core.F90:121)
  const double dta = P.dt / (double)P.mo_nadv;
  const double dts = dta / (double)P.mo_nsound;
  const double dtrdx = dts / P.dx, dtrdy = dts / P.dx, dtrdz = dts / dzita;
  const double zcs2 = (dtrdz * dtrdz) * kRdrcv;
  const double ddamp = 0.125 * (P.dx / dts);
  const double ddamp2 = (kXdamp * 0.015625) / dts;
  const double dtrdx_a = dta / P.dx, dtrdy_a = dta / P.dx;
  const double dtrdz_a = 0.5 * (dta / dzita);
  v.dts = (T)dts; v.dtrdx = (T)dtrdx; v.dtrdy = (T)dtrdy; v.dtrdz = (T)dtrdz; v.zcs2 = (T)zcs2;
  v.ddamp2 = (T)ddamp2; v.egdts = (T)(kEgrav * dts);
  v.dts_d = dts; v.dtrdz_d = dtrdz; v.zcs2_d = zcs2; v.egdts_d = kEgrav * dts;
  v.dtrdx_a = (T)dtrdx_a; v.dtrdy_a = (T)dtrdy_a; v.dtrdz_a = (T)dtrdz_a;
  v.anu2 = (T)P.mo_anu2;

  // 1-D tables
  std::vector<double> gzk(kz + 1), gzkh(kz), xknu(kz), cdamp(kz), ffilt(kz, 0.0);
  for (int k = 1; k <= kz + 1; ++k) gzk[k - 1] = gzita(h->zita[k - 1], P.mo_ztop, P.mo_a0);
  for (int k = 1; k <= kz; ++k) gzkh[k - 1] = gzita(h->zitah[k - 1], P.mo_ztop, P.mo_a0);
  for (int k = 1; k <= kz; ++k) {  // allocate_moloch :207-210
    xknu[k - 1] = kXdamp + (1.0 - kXdamp) * std::sin((0.5 * kPi) * (1.0 - (double)(k - 1) / (double)(kz - 1)));
    cdamp[k - 1] = xknu[k - 1] * ddamp;
  }
  int rc;
  if ((rc = upload_dense<T>(h, (T*)v.gzitak, gzk))) return rc;
  if ((rc = upload_dense<T>(h, (T*)v.gzitakh, gzkh))) return rc;
  if ((rc = upload_dense<T>(h, (T*)v.xknu, xknu))) return rc;
  if ((rc = upload_dense<T>(h, (T*)v.cdamp, cdamp))) return rc;
  if ((rc = upload_dense<T>(h, (T*)v.ffilt, ffilt))) return rc;

  // 2-D terms (init_moloch :252-256); msfu/msfv/hx/hy halos are periodic
  std::vector<double> a(pl), b(pl);
  auto up2 = [&](const T* dst, const std::vector<double>& src) { return upload_dense<T>(h, (T*)dst, src); };
  for (int i = 1; i <= ni; ++i)
    for (int j = 1; j <= nj; ++j) {
      a[I2(j, i)] = kEomeg2 * std::sin(h->ulat[I2(j, i)] * kDegrad);
      b[I2(j, i)] = kEomeg2 * std::sin(h->vlat[I2(j, i)] * kDegrad);
    }
  if ((rc = up2(v.coru, a)) || (rc = up2(v.corv, b))) return rc;
  for (size_t q = 0; q < pl; ++q) a[q] = h->msfx[q] * h->msfx[q];
  if ((rc = up2(v.mx2, a)) || (rc = up2(v.mx, h->msfx))) return rc;
  if ((rc = up2(v.mu, h->msfu)) || (rc = up2(v.mv, h->msfv))) return rc;
  for (size_t q = 0; q < pl; ++q) { a[q] = 1.0 / h->msfu[q]; b[q] = 1.0 / h->msfv[q]; }
  if ((rc = up2(v.rmu, a)) || (rc = up2(v.rmv, b))) return rc;
  if ((rc = up2(v.hx, h->hx)) || (rc = up2(v.hy, h->hy))) return rc;

  // 3-D static terms
  const size_t n3 = pl * kz;
  std::vector<double> rfw(n3), rfs(n3), wu(n3), wd(n3), wn(n3), ws(n3), we(n3), ww(n3), dz(n3);
  host_parallel((size_t)kz * ni, [&](size_t r0, size_t r1) {
    for (size_t r = r0; r < r1; ++r) {
      const int k = (int)(r / ni) + 1, i = (int)(r % ni) + 1;
      for (int j = 1; j <= nj; ++j) {
        const size_t q = I3(j, i, k);
        const double f = fmz[q];
        rfw[q] = 2.0 / (f + fmz[I3(j - 1, i, k)]);   // sound :584
        rfs[q] = 2.0 / (f + fmz[I3(j, i - 1, k)]);   // sound :585
        wu[q] = (dtrdz_a * f) / fmzf[I2(j, i) + pl * (size_t)(k - 1)];  // wafone :1011
        wd[q] = (dtrdz_a * f) / fmzf[I2(j, i) + pl * (size_t)k];        // wafone :1012
        const double fn = fmz[I3(j, i + 1, k)], fs = fmz[I3(j, i - 1, k)];
        const double fe = fmz[I3(j + 1, i, k)], fw = fmz[I3(j - 1, i, k)];
        const double rmvn = 1.0 / h->msfv[I2(j, i + 1)], rmvs = 1.0 / h->msfv[I2(j, i)];
        const double mxx = h->msfx[I2(j, i)], muu = h->msfu[I2(j, i)];
        if (P.rotllr) {
          const double zhxvtn = (dtrdy_a * rmvn) * mxx, zhxvts = (dtrdy_a * rmvs) * mxx;  // :1120-1121
          wn[q] = ((zhxvtn * 2.0) * f) / (f + fn);
          ws[q] = ((zhxvts * 2.0) * f) / (f + fs);
          const double zcostx = dtrdx_a * muu;  // :1177
          we[q] = ((zcostx * 2.0) * f) / (f + fe);
          ww[q] = ((zcostx * 2.0) * f) / (f + fw);
        } else {  // :1230-1231, :1287-1288
          wn[q] = ((dtrdy_a * 2.0) * f) / (f + fn);
          ws[q] = ((dtrdy_a * 2.0) * f) / (f + fs);
          we[q] = ((dtrdx_a * 2.0) * f) / (f + fe);
          ww[q] = ((dtrdx_a * 2.0) * f) / (f + fw);
        }
        dz[q] = dzita / f;  // layer thickness for the column sums
      }
    }
  });
  auto up3 = [&](const T* dst, const std::vector<double>& src) { return upload_dense<T>(h, (T*)dst, src); };
  if ((rc = up3(v.fmz, fmz)) || (rc = up3(v.fmzf, fmzf)) || (rc = up3(v.zeta, h->zeta))) return rc;
  if ((rc = up3(v.rfw, rfw)) || (rc = up3(v.rfs, rfs)) || (rc = up3(v.wafu, wu)) || (rc = up3(v.wafd, wd)))
    return rc;
  if ((rc = up3(v.wafn, wn)) || (rc = up3(v.wafs, ws)) || (rc = up3(v.wafe, we)) || (rc = up3(v.wafw, ww)))
    return rc;
  if ((rc = up3(v.dz, dz))) return rc;
  // w(:,:,1) = 0 (:260-262); s, deltaw zero (reset_tendencies :1313-1325 --
  // the kernels never write s(1), deltaw(1), deltaw(kz+1), which therefore
  // keep this zero for the whole run)
  CUDA_TRY(cudaMemsetAsync(v.w, 0, sizeof(T) * pl, h->stream));
  CUDA_TRY(cudaMemsetAsync(v.s, 0, sizeof(T) * pl * (kz + 1), h->stream));
  CUDA_TRY(cudaMemsetAsync(v.deltaw, 0, sizeof(T) * pl * (kz + 1), h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  if constexpr (sizeof(T) == sizeof(float)) {
    v.cmaps = nullptr;
    if (kfast::column_maps_bytes() <= (int)sizeof(h->cmaps) && kfast::build_column_maps(v, h->cmaps))
      v.cmaps = h->cmaps;
  }
  return MOLOCH_OK;
}

// one phase or a whole step on the handle's stream; returns kernel count
template <class T>
int launch_phase(moloch_handle* h, View<T>& v, int phase) {
  const PhaseFlags fl = flags_of(h);
  const bool exact = h->prm.mode == MOLOCH_FP64_EXACT;
  const T* zk = v.zeta + (size_t)v.pl * (v.kz - 1);
  const T* zkm1 = v.zeta + (size_t)v.pl * (v.kz - 2);
  int n = 0;
  if constexpr (sizeof(T) == sizeof(double)) {
    if (exact) {
      switch (phase) {
        case 0: n = kexact::launch_prediag<T>(v, h->stream, fl); break;
        case 1: n = kexact::launch_sound<T>(v, h->stream, fl); break;
        case 2: n = kexact::launch_advection<T>(v, h->stream); break;
        case 3: n = kexact::launch_postdiag<T>(v, h->stream, fl, zk, zkm1); break;
        case 4: n = kexact::launch_diag<T>(v, h->stream); break;
      }
      return n;
    }
  }
  if constexpr (sizeof(T) == sizeof(float)) {
    if (phase == 1 && h->sur) {
      // parity of the u/v buffer flips of the plain loop, which a committed
      // cycle's u, v must land on
      const int flips = fl.nsound * ((v.kmarch & 16) ? 2 : 1);
      n = moloch::mlp::sur_cycle(h->sur, v, h->stream, fl.nsound, flips & 1);
      n += kfast::launch_sound<T>(v, h->stream, fl);
      return n + moloch::mlp::sur_after(h->sur, v, h->stream);
    }
  }
  switch (phase) {
    case 0: n = kfast::launch_prediag<T>(v, h->stream, fl); break;
    case 1: n = kfast::launch_sound<T>(v, h->stream, fl); break;
    case 2: n = kfast::launch_advection<T>(v, h->stream); break;
    case 3: n = kfast::launch_postdiag<T>(v, h->stream, fl, zk, zkm1); break;
    case 4: n = kfast::launch_diag<T>(v, h->stream); break;
  }
  return n;
}

template <class T>
int launch_step(moloch_handle* h, View<T>& v) {
  int n = launch_phase(h, v, 0);
  for (int a = 0; a < h->prm.mo_nadv; ++a) {
    n += launch_phase(h, v, 1);
    n += launch_phase(h, v, 2);
  }
  n += launch_phase(h, v, 3);
  return n;
}

int step_kernels(moloch_handle* h) {
  if (h->elem == 8) return launch_step(h, h->vd);
  return launch_step(h, h->vf);
}

void drop_graphs(moloch_handle* h) {
  for (int q = 0; q < 2; ++q) {
    if (h->gexec[q]) { cudaGraphExecDestroy(h->gexec[q]); h->gexec[q] = nullptr; }
    if (h->graph[q]) { cudaGraphDestroy(h->graph[q]); h->graph[q] = nullptr; }
  }
}

int check_launch(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(MOLOCH_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return MOLOCH_OK;
}

// reads and clears the flag a bounded device wait sets when it gives up
int check_kerr(moloch_handle* h) {
  int* kerr = h->elem == 8 ? h->vd.kerr : h->vf.kerr;
  int v = 0;
  CUDA_TRY(cudaMemcpyAsync(&v, kerr, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  if (!v) return MOLOCH_OK;
  CUDA_TRY(cudaMemsetAsync(kerr, 0, sizeof(int), h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return fail(MOLOCH_ERR_TIMEOUT, "a bounded device wait of the column solve gave up; the state is invalid");
}

int read_diag(moloch_handle* h, moloch_diag_t* diag) {
  int n = h->elem == 8 ? launch_phase(h, h->vd, 4) : launch_phase(h, h->vf, 4);
  h->kernels += n;
  int rc;
  if ((rc = check_launch("diag"))) return rc;
  const double* dres = h->elem == 8 ? h->vd.dres : h->vf.dres;
  CUDA_TRY(cudaMemcpyAsync(h->hres, dres, sizeof(double) * 9, cudaMemcpyDeviceToHost, h->stream));
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  if ((rc = check_kerr(h))) return rc;
  moloch_diag_t d{};
  d.maxps = h->hres[0]; d.minps = h->hres[1];
  d.maxu = h->hres[2]; d.minu = h->hres[3]; d.maxv = h->hres[4]; d.minv = h->hres[5];
  d.mass = h->hres[6]; d.energy = h->hres[7];
  d.nonfinite = (int)h->hres[8];
  const bool bad = d.nonfinite > 0 || !std::isfinite(d.maxps) || !std::isfinite(d.minps);
  d.status = bad ? MOLOCH_ERR_CFL : MOLOCH_OK;
  if (diag) *diag = d;
  if (bad) return fail(MOLOCH_ERR_CFL, "CFL VIOLATION: %d non-finite ps values", d.nonfinite);
  return MOLOCH_OK;
}

}  // namespace

// ===========================================================================
extern "C" {

const char* moloch_gpu_last_error(void) { return g_err.c_str(); }

// error text from the other translation units of the library
void moloch_internal_set_error(const char* msg) { g_err = msg ? msg : ""; }

void moloch_gpu_default_params(moloch_params_t* p) {
  if (!p) return;
  std::memset(p, 0, sizeof *p);
  p->dt = 30.0;
  p->dx = 3.0 * 1000.0;
  p->mo_ztop = 36000.0;
  p->mo_h = 12000.0;
  p->mo_a0 = 0.0;
  p->mo_anu2 = 0.6;
  p->mo_nadv = 3;
  p->mo_nsound = 5;
  p->mode = MOLOCH_FP64;
  p->rotllr = 1;
}

int moloch_gpu_create(const moloch_grid_t* grid, const moloch_params_t* params, void* stream,
                      moloch_handle_t** out) {
  g_err.clear();
  if (!grid || !params || !out) return fail(MOLOCH_ERR_ARG, "null argument");
  *out = nullptr;
  if (grid->jx < 4 || grid->iy < 4 || grid->kz < 4)
    return fail(MOLOCH_ERR_ARG, "grid %dx%dx%d too small (need jx, iy, kz >= 4)", grid->jx, grid->iy, grid->kz);
  if ((double)grid->jx * grid->iy * (grid->kz + 1) > 2.0e9)
    return fail(MOLOCH_ERR_ARG, "grid too large for one handle");
  if (params->mode < MOLOCH_FP64 || params->mode > MOLOCH_FP32_MIXED)
    return fail(MOLOCH_ERR_ARG, "unknown mode %d", params->mode);
  if (params->mo_nadv < 1 || params->mo_nsound < 1 || !(params->dt > 0) || !(params->dx > 0))
    return fail(MOLOCH_ERR_ARG, "bad time parameters");
  moloch_handle* h = new moloch_handle();
  h->grid = *grid;
  h->prm = *params;
  h->elem = params->mode == MOLOCH_FP32_MIXED ? 4 : 8;
  if (stream) {
    h->stream = (cudaStream_t)stream;
  } else {
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete h;
      return fail(MOLOCH_ERR_CUDA, "stream: %s", cudaGetErrorString(e));
    }
    h->own_stream = true;
  }
  size_t bytes = h->elem == 8 ? layout(h->vd, nullptr, h) : layout(h->vf, nullptr, h);
  cudaError_t e = cudaMalloc(&h->arena, bytes);
  if (e != cudaSuccess) {
    if (h->own_stream) cudaStreamDestroy(h->stream);
    delete h;
    cudaGetLastError();
    return fail(MOLOCH_ERR_NOMEM, "device arena of %zu bytes: %s", bytes, cudaGetErrorString(e));
  }
  h->arena_bytes = bytes;
  if (h->elem == 8) layout(h->vd, (char*)h->arena, h); else layout(h->vf, (char*)h->arena, h);
  cudaMemsetAsync(h->arena, 0, bytes, h->stream);  // getmem zero-fills (mod_memutil.F90:1249)
  e = cudaMallocHost(&h->hres, sizeof(double) * 16);
  if (e == cudaSuccess) {
    h->stage_bytes = sizeof(double) * (size_t)grid->jx * grid->iy * (grid->kz + 1);
    e = cudaMallocHost(&h->stage, h->stage_bytes);
  }
  for (int q = 0; q < 2 && e == cudaSuccess; ++q) e = cudaEventCreateWithFlags(&h->stage_ev[q], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    cudaFree(h->arena);
    if (h->own_stream) cudaStreamDestroy(h->stream);
    delete h;
    return fail(MOLOCH_ERR_CUDA, "create: %s", cudaGetErrorString(e));
  }
  *out = h;
  return MOLOCH_OK;
}

int moloch_gpu_upload(moloch_handle_t* h, int field, const double* host_base, const int* lb, const int* ub) {
  g_err.clear();
  if (!h || !host_base || !lb || !ub) return fail(MOLOCH_ERR_ARG, "null argument");
  const int nj = h->nj(), ni = h->ni(), kz = h->kz();
  FieldShape s = shape_of(field, nj, ni, kz);
  if (s.ndim == 0) return fail(MOLOCH_ERR_ARG, "unknown field %d", field);
  for (int d = 0; d < s.ndim; ++d)
    if (lb[d] != s.lb[d] || ub[d] != s.ub[d])
      return fail(MOLOCH_ERR_BOUNDS, "field %d dim %d: bounds %d:%d, expected %d:%d", field, d + 1, lb[d], ub[d],
                  s.lb[d], s.ub[d]);
  if (field == MOLOCH_F_ZITA || field == MOLOCH_F_ZITAH) {
    std::vector<double>* st = static_store(h, field);
    st->assign(host_base, host_base + (s.ub[0] - s.lb[0] + 1));
    h->uploaded |= 1u << field;
    return MOLOCH_OK;
  }
  const int nk = s.ndim >= 3 ? s.ub[2] : 1;
  std::vector<double> dense;
  if (field == MOLOCH_F_HT) {  // not used by the step; accepted for completeness
    h->uploaded |= 1u << field;
    return MOLOCH_OK;
  }
  if (is_static(field)) {
    gather_interior(host_base, s, nj, ni, nk, 0, dense);
    *static_store(h, field) = dense;
    h->uploaded |= 1u << field;
    if (h->initialized) h->initialized = false;  // statics changed: init again
    return MOLOCH_OK;
  }
  const long nall = (long)(s.ub[0] - s.lb[0] + 1) * (s.ndim >= 2 ? s.ub[1] - s.lb[1] + 1 : 1) *
                    (s.ndim >= 3 ? s.ub[2] - s.lb[2] + 1 : 1);
  // registered (pinned) host arrays always go by DMA; others by the direct
  // kernel where the device can read pageable memory, else staged
  const bool direct = use_direct(h) || is_pinned(h, host_base, sizeof(double) * nall * (field == MOLOCH_F_QX ? 5 : 1));
  auto up = [&](int f, int level4) -> int {
    if (h->elem == 8) {
      double* p = field_ptr(h->vd, f);
      if (!p) return fail(MOLOCH_ERR_ARG, "field %d cannot be uploaded", f);
      return direct ? upload_direct<double>(h, f, p, host_base, s, nj, ni, nk, level4)
                    : upload_streamed<double>(h, p, host_base, s, nj, ni, nk, level4);
    }
    float* p = field_ptr(h->vf, f);
    if (!p) return fail(MOLOCH_ERR_ARG, "field %d cannot be uploaded", f);
    return direct ? upload_direct<float>(h, f, p, host_base, s, nj, ni, nk, level4)
                  : upload_streamed<float>(h, p, host_base, s, nj, ni, nk, level4);
  };
  if (field == MOLOCH_F_QX) {
    for (int n = 0; n < 5; ++n) {
      int rc = up(MOLOCH_F_QV + n, n);
      if (rc) return rc;
      h->uploaded |= 1u << (MOLOCH_F_QV + n);
    }
    return MOLOCH_OK;
  }
  const int rc = up(field, 0);
  if (!rc) h->uploaded |= 1u << field;
  return rc;
}

int moloch_gpu_host_register(moloch_handle_t* h, const void* ptr, size_t bytes) {
  g_err.clear();
  if (!h || !ptr || !bytes) return fail(MOLOCH_ERR_ARG, "null argument");
  if (is_pinned(h, ptr, bytes)) return MOLOCH_OK;
  CUDA_TRY(cudaHostRegister(const_cast<void*>(ptr), bytes, cudaHostRegisterDefault));
  h->pinned.emplace_back((const char*)ptr, bytes);
  return MOLOCH_OK;
}

int moloch_gpu_host_unregister(moloch_handle_t* h, const void* ptr) {
  g_err.clear();
  if (!h || !ptr) return fail(MOLOCH_ERR_ARG, "null argument");
  for (size_t q = 0; q < h->pinned.size(); ++q)
    if (h->pinned[q].first == (const char*)ptr) {
      if (h->up_stream) CUDA_TRY(cudaStreamSynchronize(h->up_stream));  // no copy from it in flight
      CUDA_TRY(cudaHostUnregister(const_cast<void*>(ptr)));
      h->pinned.erase(h->pinned.begin() + q);
      return MOLOCH_OK;
    }
  return fail(MOLOCH_ERR_ARG, "range not registered with this handle");
}

int moloch_gpu_host_direct(moloch_handle_t* h, int enable) {
  g_err.clear();
  if (!h) return fail(MOLOCH_ERR_ARG, "null handle");
  if (enable >= 0) {
    h->host_direct = -1;
    const bool can = use_direct(h);
    h->host_direct = (enable && can) ? 1 : 0;
  }
  return use_direct(h) ? 1 : 0;
}

int moloch_gpu_init(moloch_handle_t* h) {
  g_err.clear();
  if (!h) return fail(MOLOCH_ERR_ARG, "null handle");
  const int need[] = {MOLOCH_F_U, MOLOCH_F_V, MOLOCH_F_W, MOLOCH_F_PAI, MOLOCH_F_T, MOLOCH_F_QV, MOLOCH_F_QC,
                      MOLOCH_F_QI, MOLOCH_F_QR, MOLOCH_F_QS, MOLOCH_F_ZETA, MOLOCH_F_FMZ, MOLOCH_F_FMZF,
                      MOLOCH_F_MSFX, MOLOCH_F_MSFU, MOLOCH_F_MSFV, MOLOCH_F_HX, MOLOCH_F_HY, MOLOCH_F_ULAT,
                      MOLOCH_F_VLAT, MOLOCH_F_ZITA, MOLOCH_F_ZITAH};
  for (int f : need)
    if (!(h->uploaded & (1u << f))) return fail(MOLOCH_ERR_STATE, "init before field %d was uploaded", f);
  int rc = h->elem == 8 ? init_impl(h, h->vd) : init_impl(h, h->vf);
  if (rc) return rc;
  for (int q = 0; q < 2; ++q) {
    if (h->gexec[q]) { cudaGraphExecDestroy(h->gexec[q]); h->gexec[q] = nullptr; }
    if (h->graph[q]) { cudaGraphDestroy(h->graph[q]); h->graph[q] = nullptr; }
  }
  h->initialized = true;
  return MOLOCH_OK;
}

int moloch_gpu_step(moloch_handle_t* h, int istep, int lprint, moloch_diag_t* diag) {
  g_err.clear();
  (void)istep;  // the reference uses istep only in its printout (:412)
  if (!h) return fail(MOLOCH_ERR_ARG, "null handle");
  if (!h->initialized) return fail(MOLOCH_ERR_STATE, "step before moloch_gpu_init");
  int n = step_kernels(h);
  h->kernels += n;
  h->kernels_per_step = n;
  int rc = check_launch("step");
  if (rc) return rc;
  if (lprint) return read_diag(h, diag);
  return MOLOCH_OK;
}

int moloch_gpu_run(moloch_handle_t* h, int nsteps, int use_graph) {
  g_err.clear();
  if (!h) return fail(MOLOCH_ERR_ARG, "null handle");
  if (!h->initialized) return fail(MOLOCH_ERR_STATE, "run before moloch_gpu_init");
  if (nsteps < 0) return fail(MOLOCH_ERR_ARG, "nsteps < 0");
  if (!use_graph) {
    for (int s = 0; s < nsteps; ++s) {
      int n = step_kernels(h);
      h->kernels += n;
      h->kernels_per_step = n;
      int rc = check_launch("run");
      if (rc) return rc;
    }
    return MOLOCH_OK;
  }
  for (int st = 0; st < nsteps; ++st) {
    const int par = h->elem == 8 ? h->vd.fcur : h->vf.fcur;
    const int cur = h->elem == 8 ? h->vd.cur : h->vf.cur;
    if (cur != 0) {  // after a lone sound() phase the u/v pair is swapped: no graph for this step
      h->kernels += step_kernels(h);
      int rc = check_launch("run");
      if (rc) return rc;
      continue;
    }
    if (!h->gexec[par]) {
      // capture advances the host-side buffer bookkeeping like a real step;
      // it is restored below so the replay starts from the same state
      View<double> vd0 = h->vd;
      View<float> vf0 = h->vf;
      CUDA_TRY(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
      int n = step_kernels(h);
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamEndCapture(h->stream, &g);
      h->vd = vd0;
      h->vf = vf0;
      if (e != cudaSuccess) return fail(MOLOCH_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
      h->graph[par] = g;
      CUDA_TRY(cudaGraphInstantiate(&h->gexec[par], h->graph[par], 0));
      h->kernels_per_step = n;
    }
    CUDA_TRY(cudaGraphLaunch(h->gexec[par], h->stream));
    h->kernels += h->kernels_per_step;
    // the same bookkeeping the captured step performed
    if (h->elem == 8) { h->vd.fcur ^= (h->prm.mo_nadv & 1); h->vd.bind_fields(); h->vd.cur = 0; }
    else { h->vf.fcur ^= (h->prm.mo_nadv & 1); h->vf.bind_fields(); h->vf.cur = 0; }
  }
  return check_launch("graph replay");
}

int moloch_gpu_phase(moloch_handle_t* h, int phase) {
  g_err.clear();
  if (!h) return fail(MOLOCH_ERR_ARG, "null handle");
  if (!h->initialized) return fail(MOLOCH_ERR_STATE, "phase before moloch_gpu_init");
  if (phase < 0 || phase > 3) return fail(MOLOCH_ERR_ARG, "phase %d", phase);
  int n = h->elem == 8 ? launch_phase(h, h->vd, phase) : launch_phase(h, h->vf, phase);
  h->kernels += n;
  return check_launch("phase");
}

int moloch_gpu_download(moloch_handle_t* h, int field, double* host_base, const int* lb, const int* ub) {
  g_err.clear();
  if (!h || !host_base || !lb || !ub) return fail(MOLOCH_ERR_ARG, "null argument");
  const int nj = h->nj(), ni = h->ni(), kz = h->kz();
  FieldShape s = shape_of(field, nj, ni, kz);
  if (s.ndim == 0) return fail(MOLOCH_ERR_ARG, "unknown field %d", field);
  for (int d = 0; d < s.ndim; ++d)
    if (lb[d] != s.lb[d] || ub[d] != s.ub[d])
      return fail(MOLOCH_ERR_BOUNDS, "field %d dim %d: bounds %d:%d, expected %d:%d", field, d + 1, lb[d], ub[d],
                  s.lb[d], s.ub[d]);
  if (field == MOLOCH_F_ZITA || field == MOLOCH_F_ZITAH) {
    std::vector<double>* st = static_store(h, field);
    if (st->empty()) return fail(MOLOCH_ERR_STATE, "field %d not uploaded", field);
    std::memcpy(host_base, st->data(), sizeof(double) * st->size());
    return MOLOCH_OK;
  }
  const int nk = s.ndim >= 3 ? s.ub[2] : 1;
  std::vector<double> dense;
  if (is_static(field)) {
    std::vector<double>* st = static_store(h, field);
    if (!st || st->empty()) return fail(MOLOCH_ERR_STATE, "field %d not available", field);
    scatter_periodic(*st, s, nj, ni, nk, 0, host_base);
    return MOLOCH_OK;
  }
  auto down = [&](int f, int k, int level4) -> int {
    return h->elem == 8 ? download_streamed<double>(h, field_ptr(h->vd, f), s, nj, ni, k, level4, host_base)
                        : download_streamed<float>(h, field_ptr(h->vf, f), s, nj, ni, k, level4, host_base);
  };
  if (field == MOLOCH_F_QX) {
    for (int n = 0; n < 5; ++n) {
      int rc = down(MOLOCH_F_QV + n, kz, n);
      if (rc) return rc;
    }
    return MOLOCH_OK;
  }
  return down(field, nk, 0);
}

// Output path (the fields the reference driver writes every iout steps,
// nompi/regcm_dynamical_core.F90:203-216): t and ps are copied on the device
// into a snapshot in stream order, and the snapshot goes to pinned host
// memory on a second stream, so the caller's next steps overlap the copy.
int moloch_gpu_output_start(moloch_handle_t* h) {
  g_err.clear();
  if (!h || !h->initialized) return fail(MOLOCH_ERR_STATE, "output before moloch_gpu_init");
  if (h->out_pending) return fail(MOLOCH_ERR_STATE, "output_start twice without output_finish");
  const size_t pl = (size_t)h->nj() * h->ni(), n3 = pl * h->kz();
  const size_t bytes = (n3 + pl) * h->elem;
  if (!h->out_dev) {
    CUDA_TRY(cudaMalloc(&h->out_dev, bytes));
    CUDA_TRY(cudaMallocHost(&h->out_host, bytes));
    int lo = 0, hi = 0;  // highest priority: its copies and kernels slip in beside the running steps
    CUDA_TRY(cudaDeviceGetStreamPriorityRange(&lo, &hi));
    CUDA_TRY(cudaStreamCreateWithPriority(&h->out_stream, cudaStreamNonBlocking, hi));
    CUDA_TRY(cudaEventCreateWithFlags(&h->out_taken, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&h->out_done, cudaEventDisableTiming));
  }
  const void* t = h->elem == 8 ? (const void*)h->vd.t : (const void*)h->vf.t;
  const void* ps = h->elem == 8 ? (const void*)h->vd.ps : (const void*)h->vf.ps;
  CUDA_TRY(cudaMemcpyAsync(h->out_dev, t, n3 * h->elem, cudaMemcpyDeviceToDevice, h->stream));
  CUDA_TRY(cudaMemcpyAsync((char*)h->out_dev + n3 * h->elem, ps, pl * h->elem, cudaMemcpyDeviceToDevice, h->stream));
  CUDA_TRY(cudaEventRecord(h->out_taken, h->stream));
  CUDA_TRY(cudaStreamWaitEvent(h->out_stream, h->out_taken, 0));
  CUDA_TRY(cudaMemcpyAsync(h->out_host, h->out_dev, bytes, cudaMemcpyDeviceToHost, h->out_stream));
  CUDA_TRY(cudaEventRecord(h->out_done, h->out_stream));
  h->out_pending = true;
  return MOLOCH_OK;
}

int moloch_gpu_output_finish(moloch_handle_t* h, double* t_host, const int* t_lb, const int* t_ub, double* ps_host,
                             const int* ps_lb, const int* ps_ub) {
  g_err.clear();
  if (!h || !h->out_pending) return fail(MOLOCH_ERR_STATE, "output_finish without output_start");
  const int nj = h->nj(), ni = h->ni(), kz = h->kz();
  const FieldShape st = shape_of(MOLOCH_F_T, nj, ni, kz), sp = shape_of(MOLOCH_F_PS, nj, ni, kz);
  for (int d = 0; d < st.ndim; ++d)
    if (t_host && (t_lb[d] != st.lb[d] || t_ub[d] != st.ub[d])) return fail(MOLOCH_ERR_BOUNDS, "output t bounds");
  for (int d = 0; d < sp.ndim; ++d)
    if (ps_host && (ps_lb[d] != sp.lb[d] || ps_ub[d] != sp.ub[d])) return fail(MOLOCH_ERR_BOUNDS, "output ps bounds");
  const size_t pl = (size_t)nj * ni, n3 = pl * kz;
  auto host_len = [](const FieldShape& s, int nk) {
    return (size_t)(s.ub[0] - s.lb[0] + 1) * (s.ub[1] - s.lb[1] + 1) * nk;
  };
  if ((!t_host || is_pinned(h, t_host, sizeof(double) * host_len(st, kz))) &&
      (!ps_host || is_pinned(h, ps_host, sizeof(double) * host_len(sp, 1)))) {
    // registered destinations: a kernel lays the snapshot out in Fortran
    // order (halo rings included) in device memory, the copy engine moves
    // it into the caller's arrays -- no host-side scatter, no SMs on the
    // host link
    const size_t lt = host_len(st, kz), lp = host_len(sp, 1);
    if (!h->out_f64) CUDA_TRY(cudaMalloc(&h->out_f64, sizeof(double) * (lt + lp)));
    double* dt = (double*)h->out_f64;
    double* dp = dt + lt;
    auto put = [&](const FieldShape& s, int nk, size_t off, double* dev, double* dst, size_t len) -> int {
      const int n1 = s.ub[0] - s.lb[0] + 1, n2 = s.ub[1] - s.lb[1] + 1;
      if (h->elem == 8)
        moloch::init::launch_output_layout<double>(dev, (const double*)h->out_dev + off, s.lb[0], n1, s.lb[1], n2, nk,
                                                   nj, ni, h->out_stream);
      else
        moloch::init::launch_output_layout<float>(dev, (const float*)h->out_dev + off, s.lb[0], n1, s.lb[1], n2, nk,
                                                  nj, ni, h->out_stream);
      CUDA_TRY(cudaMemcpyAsync(dst, dev, sizeof(double) * len, cudaMemcpyDeviceToHost, h->out_stream));
      return MOLOCH_OK;
    };
    int rc = MOLOCH_OK;
    if (t_host) rc = put(st, kz, 0, dt, t_host, lt);
    if (!rc && ps_host) rc = put(sp, 1, n3, dp, ps_host, lp);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(h->out_stream));
    h->out_pending = false;
    return rc;
  }
  CUDA_TRY(cudaEventSynchronize(h->out_done));
  h->out_pending = false;
  auto scatter = [&](const FieldShape& s, int nk, size_t off, double* base) {
    const long n1 = s.ub[0] - s.lb[0] + 1, n2 = s.ub[1] - s.lb[1] + 1;
    const int i1 = s.lb[1], nrow_i = s.ub[1] - s.lb[1] + 1;
    host_parallel((size_t)nk * nrow_i, [&](size_t r0, size_t r1) {
      for (size_t r = r0; r < r1; ++r) {
        const int kk = (int)(r / nrow_i), i = i1 + (int)(r % nrow_i);
        double* o = base + (long)kk * n1 * n2 + (long)(i - i1) * n1;
        const size_t row = off + ((size_t)kk * ni + wrap(i, ni)) * nj;
        if (h->elem == 8) {
          const double* src = (const double*)h->out_host + row;
          for (int j = s.lb[0]; j <= s.ub[0]; ++j) o[j - s.lb[0]] = src[wrap(j, nj)];
        } else {
          const float* src = (const float*)h->out_host + row;
          for (int j = s.lb[0]; j <= s.ub[0]; ++j) o[j - s.lb[0]] = (double)src[wrap(j, nj)];
        }
      }
    });
  };
  if (t_host) scatter(st, kz, 0, t_host);
  if (ps_host) scatter(sp, 1, n3, ps_host);
  return MOLOCH_OK;
}

// Idealized initial state computed on the device (param() and
// fill_atmosphere() as in moloch_gpu_setup_idealized, one thread per
// column): the prognostic fields are written in place in the bulk type, the
// FP64 static fields come back to the host copies init uses, then
// moloch_gpu_init runs as after a Fortran caller's uploads.
int moloch_gpu_setup_idealized_device(moloch_handle_t* h, const moloch_ideal_t* ideal) {
  g_err.clear();
  if (!h || !ideal) return fail(MOLOCH_ERR_ARG, "null argument");
  const int nj = h->nj(), ni = h->ni(), kz = h->kz();
  if (kz < 2) return fail(MOLOCH_ERR_ARG, "kz >= 2");
  const moloch_params_t& P = h->prm;
  const size_t pl = (size_t)nj * ni;
  // zita levels (model_zitaf / model_zitah), 1-based with kz+2 entries
  std::vector<double> zita(kz + 2, 0.0), zitah(kz + 2, 0.0);
  const double dz = P.mo_ztop / (double)kz;
  zita[kz + 1] = 0.0;
  for (int k = kz; k >= 1; --k) zita[k] = zita[k + 1] + dz;
  zitah[kz] = dz * 0.5;
  for (int k = kz - 1; k >= 1; --k) zitah[k] = zitah[k + 1] + dz;
  moloch::init::IdealArgs a{};
  a.nj = nj; a.ni = ni; a.kz = kz; a.rotllr = P.rotllr;
  a.dx = P.dx; a.ztop = P.mo_ztop; a.zh = P.mo_h; a.a0 = P.mo_a0;
  a.nhills = std::min(ideal->nhills, 4);
  for (int n = 0; n < 4; ++n) {
    a.hill_h[n] = ideal->hill_h[n]; a.hill_j[n] = ideal->hill_j[n];
    a.hill_i[n] = ideal->hill_i[n]; a.hill_r[n] = ideal->hill_r[n];
  }
  a.pert_amp = ideal->pert_amp; a.pert_levels = ideal->pert_levels; a.seed = ideal->seed;
  // FP64 scratch: zita, zitah, zeta, fmz, fmzf, hx, hy, ulat, vlat
  const size_t n_z = 2 * (size_t)(kz + 2), n3 = pl * kz, n3p = pl * (kz + 1);
  double* dev = nullptr;
  CUDA_TRY(cudaMalloc(&dev, sizeof(double) * (n_z + 2 * n3 + n3p + 4 * pl)));
  double *dzita = dev, *dzitah = dev + (kz + 2), *dzeta = dev + n_z, *dfmz = dzeta + n3, *dfmzf = dfmz + n3;
  double *dhx = dfmzf + n3p, *dhy = dhx + pl, *dulat = dhy + pl, *dvlat = dulat + pl;
  auto done = [&](int rc) { cudaFree(dev); return rc; };
  if (cudaMemcpyAsync(dzita, zita.data(), sizeof(double) * (kz + 2), cudaMemcpyHostToDevice, h->stream) ||
      cudaMemcpyAsync(dzitah, zitah.data(), sizeof(double) * (kz + 2), cudaMemcpyHostToDevice, h->stream))
    return done(fail(MOLOCH_ERR_CUDA, "setup_idealized_device: copy of the zita levels"));
  using moloch::init::launch_fill;
  using moloch::init::launch_ideal;
  if (h->elem == 8) {
    View<double>& v = h->vd;
    launch_ideal<double>(a, dzita, dzitah, dzeta, dfmz, dfmzf, dhx, dhy, dulat, dvlat, v.t, v.pai, v.q[0], h->stream);
    for (int n = 1; n < 5; ++n) launch_fill<double>(v.q[n], pl * kz, 0.0, h->stream);
    launch_fill<double>(v.ubuf[v.cur], pl * kz, ideal->u0, h->stream);
    launch_fill<double>(v.vbuf[v.cur], pl * kz, ideal->v0, h->stream);
    launch_fill<double>(v.w, pl * (kz + 1), 0.0, h->stream);
  } else {
    View<float>& v = h->vf;
    launch_ideal<float>(a, dzita, dzitah, dzeta, dfmz, dfmzf, dhx, dhy, dulat, dvlat, v.t, v.pai, v.q[0], h->stream);
    for (int n = 1; n < 5; ++n) launch_fill<float>(v.q[n], pl * kz, 0.0, h->stream);
    launch_fill<float>(v.ubuf[v.cur], pl * kz, ideal->u0, h->stream);
    launch_fill<float>(v.vbuf[v.cur], pl * kz, ideal->v0, h->stream);
    launch_fill<float>(v.w, pl * (kz + 1), 0.0, h->stream);
  }
  if (cudaGetLastError() != cudaSuccess) return done(fail(MOLOCH_ERR_CUDA, "setup_idealized_device: launch"));
  h->zeta.resize(n3); h->fmz.resize(n3); h->fmzf.resize(n3p);
  h->hx.resize(pl); h->hy.resize(pl); h->ulat.resize(pl); h->vlat.resize(pl);
  struct { double* dst; const double* src; size_t n; } cp[] = {
      {h->zeta.data(), dzeta, n3}, {h->fmz.data(), dfmz, n3}, {h->fmzf.data(), dfmzf, n3p},
      {h->hx.data(), dhx, pl}, {h->hy.data(), dhy, pl}, {h->ulat.data(), dulat, pl}, {h->vlat.data(), dvlat, pl}};
  for (auto& x : cp)
    if (cudaMemcpyAsync(x.dst, x.src, sizeof(double) * x.n, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess)
      return done(fail(MOLOCH_ERR_CUDA, "setup_idealized_device: copy of the static fields"));
  if (cudaStreamSynchronize(h->stream) != cudaSuccess)
    return done(fail(MOLOCH_ERR_CUDA, "setup_idealized_device: %s", cudaGetErrorString(cudaGetLastError())));
  cudaFree(dev);
  h->msfx.assign(pl, 1.0); h->msfu.assign(pl, 1.0); h->msfv.assign(pl, 1.0);
  h->zita.assign(zita.begin() + 1, zita.begin() + kz + 2);
  h->zitah.assign(zitah.begin() + 1, zitah.begin() + kz + 1);
  const int fields[] = {MOLOCH_F_U, MOLOCH_F_V, MOLOCH_F_W, MOLOCH_F_PAI, MOLOCH_F_T, MOLOCH_F_QV, MOLOCH_F_QC,
                        MOLOCH_F_QI, MOLOCH_F_QR, MOLOCH_F_QS, MOLOCH_F_ZETA, MOLOCH_F_FMZ, MOLOCH_F_FMZF,
                        MOLOCH_F_MSFX, MOLOCH_F_MSFU, MOLOCH_F_MSFV, MOLOCH_F_HX, MOLOCH_F_HY, MOLOCH_F_ULAT,
                        MOLOCH_F_VLAT, MOLOCH_F_ZITA, MOLOCH_F_ZITAH};
  for (int f : fields) h->uploaded |= 1u << f;
  h->initialized = false;
  return moloch_gpu_init(h);
}

int moloch_gpu_sync(moloch_handle_t* h) {
  g_err.clear();
  if (!h) return fail(MOLOCH_ERR_ARG, "null handle");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  return check_kerr(h);
}

int moloch_gpu_set_wait_limit(moloch_handle_t* h, long long cycles, int skip_job) {
  g_err.clear();
  if (!h) return fail(MOLOCH_ERR_ARG, "null handle");
  if (cycles <= 0) cycles = kDefaultSpinCycles;
  h->vd.spin_cycles = h->vf.spin_cycles = cycles;
  h->vd.fault_skip_job = h->vf.fault_skip_job = skip_job < 0 ? -1 : skip_job;
  drop_graphs(h);  // both are kernel parameters baked into captured graphs
  return MOLOCH_OK;
}

void* moloch_gpu_stream(moloch_handle_t* h) { return h ? (void*)h->stream : nullptr; }

long long moloch_gpu_kernel_count(moloch_handle_t* h) { return h ? h->kernels : -1; }

static const char* const kKindNames[KK_COUNT] = {
    "k_prediag", "k_sound_div", "k_sound_damp", "k_sound_column", "k_lap_filter", "k_pai_update",
    "k_sound_momentum", "k_waf_vertical", "k_waf_horizontal", "k_stag_from_x",
    "k_filter_increment", "k_postdiag", "k_diag", "k_sound_divdamp", "k_sound_column_tm"};

int moloch_gpu_kernel_kinds(void) { return KK_COUNT; }

const char* moloch_gpu_kernel_name(int kind) { return (kind >= 0 && kind < KK_COUNT) ? kKindNames[kind] : ""; }

int moloch_gpu_profile_step(moloch_handle_t* h, double* ms_by_kind, int* launches_by_kind, int nkinds) {
  g_err.clear();
  if (!h) return fail(MOLOCH_ERR_ARG, "null handle");
  if (!h->initialized) return fail(MOLOCH_ERR_STATE, "profile before moloch_gpu_init");
  KernelTimer* tm = new KernelTimer();
  for (int q = 0; q < KernelTimer::kCap; ++q)
    if (cudaEventCreate(&tm->ev[q]) != cudaSuccess) {
      for (int r = 0; r < q; ++r) cudaEventDestroy(tm->ev[r]);
      delete tm;
      return fail(MOLOCH_ERR_CUDA, "event create");
    }
  kfast::set_timer(tm);
  kexact::set_timer(tm);
  int n = step_kernels(h);
  kfast::set_timer(nullptr);
  kexact::set_timer(nullptr);
  h->kernels += n;
  int rc = check_launch("profile");
  if (!rc && cudaStreamSynchronize(h->stream) != cudaSuccess) rc = fail(MOLOCH_ERR_CUDA, "profile sync");
  if (!rc && !tm->ok) rc = fail(MOLOCH_ERR_ARG, "too many kernels to profile one step");
  if (!rc) {
    for (int q = 0; q + 1 < tm->n; q += 2) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, tm->ev[q], tm->ev[q + 1]);
      int k = tm->kind[q / 2];
      if (k < nkinds) {
        if (ms_by_kind) ms_by_kind[k] += ms;
        if (launches_by_kind) launches_by_kind[k] += 1;
      }
    }
  }
  for (int q = 0; q < KernelTimer::kCap; ++q) cudaEventDestroy(tm->ev[q]);
  delete tm;
  return rc;
}

// ---- autotuner --------------------------------------------------------------
// Tunable launch shapes, in order: [0] levels per k_waf_horizontal block.
// horizontal WAF launch shape: 1..8 = levels per 32x8 tile block, >= 16 =
// rows per warp strip
static const int kTuneCandidates[][7] = {{1, 2, 4, 8, 16, 32, 64}};
// [0] horizontal WAF shape, [1] sound kernel variants (bit mask:
// 1 divergence, 2 damping, 4 momentum k-marching; 8 momentum warp strips;
// 16 divergence and damping fused in warp strips, which overrides 1 and 2),
// [2] advected fields per thread of the vertical WAF (1, 2, 5, 10),
// [3] rows per warp strip of the momentum strips, [4] the staggering back
// from the cross points four columns per thread (1) or one (0)
static const int kTuneCount = 5;
static const int kStripRowCandidates[4] = {4, 8, 16, 32};
static const int kVFieldCandidates[4] = {1, 2, 5, 10};
static bool valid_vfields(int f) { return f == 1 || f == 2 || f == 5 || f == 10; }

int moloch_gpu_tuning_count(void) { return kTuneCount; }

int moloch_gpu_set_tuning(moloch_handle_t* h, const int* choice, int n) {
  g_err.clear();
  if (!h || (n > 0 && !choice)) return fail(MOLOCH_ERR_ARG, "null argument");
  // every slot is checked before any is applied
  if (n > 0 && (choice[0] < 1 || choice[0] > 64)) return fail(MOLOCH_ERR_ARG, "hz_levels %d", choice[0]);
  if (n > 1 && (choice[1] < 0 || choice[1] > 1023 || (choice[1] & 384) == 384))
    return fail(MOLOCH_ERR_ARG, "kmarch %d", choice[1]);
  if (n > 2 && !valid_vfields(choice[2])) return fail(MOLOCH_ERR_ARG, "vertical fields per thread %d", choice[2]);
  if (n > 3 && (choice[3] < 4 || choice[3] > 64))
    return fail(MOLOCH_ERR_ARG, "rows per momentum strip %d", choice[3]);
  if (n > 4 && (choice[4] < 0 || choice[4] > 1)) return fail(MOLOCH_ERR_ARG, "staggering variant %d", choice[4]);
  if (n > 0) { h->vd.hz_levels = choice[0]; h->vf.hz_levels = choice[0]; }
  if (n > 1) { h->vd.kmarch = choice[1]; h->vf.kmarch = choice[1]; }
  if (n > 2) { h->vd.vfields = choice[2]; h->vf.vfields = choice[2]; }
  if (n > 3) { h->vd.srows = choice[3]; h->vf.srows = choice[3]; }
  if (n > 4) { h->vd.stag4 = choice[4]; h->vf.stag4 = choice[4]; }
  for (int q = 0; q < 2; ++q) {  // launch shapes are baked into captured graphs
    if (h->gexec[q]) { cudaGraphExecDestroy(h->gexec[q]); h->gexec[q] = nullptr; }
    if (h->graph[q]) { cudaGraphDestroy(h->graph[q]); h->graph[q] = nullptr; }
  }
  return MOLOCH_OK;
}

int moloch_gpu_autotune(moloch_handle_t* h, int* choice, double* best_ms, int n) {
  g_err.clear();
  if (!h || !choice || n < kTuneCount) return fail(MOLOCH_ERR_ARG, "need %d choice slots", kTuneCount);
  if (!h->initialized) return fail(MOLOCH_ERR_STATE, "autotune before moloch_gpu_init");
  // time advection() (the tuned kernel's phase) on a copy of the view: the
  // state is advanced but the step the caller sees is unchanged in shape
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  double best = 1e30;
  int pick = h->elem == 8 ? h->vd.hz_levels : h->vf.hz_levels;
  for (int c = 0; c < 7; ++c) {
    const int cand = kTuneCandidates[0][c];
    if (cand < 16 && cand > h->kz()) continue;
    h->vd.hz_levels = cand;
    h->vf.hz_levels = cand;
    float ms = 0.f, tot = 0.f;
    for (int rep = 0; rep < 3; ++rep) {  // first repeat warms up
      cudaEventRecord(e0, h->stream);
      int nk = h->elem == 8 ? launch_phase(h, h->vd, 2) : launch_phase(h, h->vf, 2);
      h->kernels += nk;
      cudaEventRecord(e1, h->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        cudaEventDestroy(e0); cudaEventDestroy(e1);
        return fail(MOLOCH_ERR_CUDA, "autotune: %s", cudaGetErrorString(cudaGetLastError()));
      }
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) tot += ms;
    }
    if (tot < best) { best = tot; pick = cand; }
  }
  h->vd.hz_levels = pick;
  h->vf.hz_levels = pick;
  // sound point kernels: one level per thread or k-marching (each of the
  // three), timed on sound()
  double best1 = 1e30;
  int pick1 = h->elem == 8 ? h->vd.kmarch : h->vf.kmarch;
  const bool staged_ok = h->elem == 4 && h->vf.cmaps != nullptr;
  for (int cand = 0; cand < 1024; ++cand) {
    if ((cand & 384) && (!(cand & 32) || (cand & 384) == 384)) continue;  // one staged-column variant
    if ((cand & 512) && !(cand & 16)) continue;  // levels per warp of the fused strips
    if ((cand & 64) && (h->elem != 4 || !(cand & 8) || h->nj() % 2)) continue;  // two-column strips: FP32, jx even
    if ((cand & 12) == 12) continue;  // strips replace the k-marching momentum
    if ((cand & 16) && (cand & 3)) continue;  // the fused kernel replaces both
    if ((cand & 32) && !staged_ok) continue;  // staged column solve: FP32 domains with tensor maps
    h->vd.kmarch = cand;
    h->vf.kmarch = cand;
    float ms = 0.f, tot = 0.f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0, h->stream);
      int nk = h->elem == 8 ? launch_phase(h, h->vd, 1) : launch_phase(h, h->vf, 1);
      h->kernels += nk;
      cudaEventRecord(e1, h->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        cudaEventDestroy(e0); cudaEventDestroy(e1);
        return fail(MOLOCH_ERR_CUDA, "autotune: %s", cudaGetErrorString(cudaGetLastError()));
      }
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) tot += ms;
    }
    if (tot < best1) { best1 = tot; pick1 = cand; }
  }
  h->vd.kmarch = pick1;
  h->vf.kmarch = pick1;
  // vertical WAF: fields per thread, timed on advection()
  double best2 = 1e30;
  int pick2 = h->elem == 8 ? h->vd.vfields : h->vf.vfields;
  for (int cand : kVFieldCandidates) {
    h->vd.vfields = cand;
    h->vf.vfields = cand;
    float ms = 0.f, tot = 0.f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0, h->stream);
      int nk = h->elem == 8 ? launch_phase(h, h->vd, 2) : launch_phase(h, h->vf, 2);
      h->kernels += nk;
      cudaEventRecord(e1, h->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        cudaEventDestroy(e0); cudaEventDestroy(e1);
        return fail(MOLOCH_ERR_CUDA, "autotune: %s", cudaGetErrorString(cudaGetLastError()));
      }
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) tot += ms;
    }
    if (tot < best2) { best2 = tot; pick2 = cand; }
  }
  h->vd.vfields = pick2;
  h->vf.vfields = pick2;
  // rows per warp strip of the momentum strips, timed on sound() with the
  // variants chosen above
  double best3 = 1e30;
  int pick3 = h->elem == 8 ? h->vd.srows : h->vf.srows;
  for (int cand : kStripRowCandidates) {
    h->vd.srows = cand;
    h->vf.srows = cand;
    float ms = 0.f, tot = 0.f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0, h->stream);
      int nk = h->elem == 8 ? launch_phase(h, h->vd, 1) : launch_phase(h, h->vf, 1);
      h->kernels += nk;
      cudaEventRecord(e1, h->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        cudaEventDestroy(e0); cudaEventDestroy(e1);
        return fail(MOLOCH_ERR_CUDA, "autotune: %s", cudaGetErrorString(cudaGetLastError()));
      }
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) tot += ms;
    }
    if (tot < best3) { best3 = tot; pick3 = cand; }
  }
  h->vd.srows = pick3;
  h->vf.srows = pick3;
  // staggering back from the cross points (FP32, jx a multiple of 4), timed
  // on advection()
  double best4 = 0.0;
  int pick4 = 0;
  if (h->elem == 4 && h->nj() % 4 == 0) {
    best4 = 1e30;
    for (int cand = 0; cand < 2; ++cand) {
      h->vf.stag4 = cand;
      float ms = 0.f, tot = 0.f;
      for (int rep = 0; rep < 3; ++rep) {
        cudaEventRecord(e0, h->stream);
        h->kernels += launch_phase(h, h->vf, 2);
        cudaEventRecord(e1, h->stream);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
          cudaEventDestroy(e0); cudaEventDestroy(e1);
          return fail(MOLOCH_ERR_CUDA, "autotune: %s", cudaGetErrorString(cudaGetLastError()));
        }
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0) tot += ms;
      }
      if (tot < best4) { best4 = tot; pick4 = cand; }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  choice[0] = pick;
  choice[1] = pick1;
  choice[2] = pick2;
  choice[3] = pick3;
  choice[4] = pick4;
  if (best_ms) {
    best_ms[0] = best / 2.0; best_ms[1] = best1 / 2.0; best_ms[2] = best2 / 2.0; best_ms[3] = best3 / 2.0;
    best_ms[4] = best4 / 2.0;
  }
  return moloch_gpu_set_tuning(h, choice, kTuneCount);
}

// ---- ensembles --------------------------------------------------------------
}  // extern "C"

struct moloch_ensemble {
  std::vector<moloch_handle*> m;
  int elem = 4;
  cudaStream_t stream = nullptr;
  void* dev = nullptr;  // views + tile tables
  Batch<double> bd{};
  Batch<float> bf{};
  std::vector<int4> tiles[TK_COUNT];
  cudaGraph_t graph[2] = {nullptr, nullptr};
  cudaGraphExec_t gexec[2] = {nullptr, nullptr};
  int hz_levels = 4;
  int kmarch = 0;
  int vfields = 1;
  int mrows = kMomR;  // rows per momentum warp strip of the one-launch-per-kernel mode
  int cur = 0, fcur = 0;
  long long kernels = 0;
  int kernels_per_step = 0;
  PhaseFlags fl{};
  // persistent mode: one cooperative launch per step walking a phase
  // program (one per field-set parity at the step's start)
  int persistent = 0;
  const persist::Phase* prog[2] = {nullptr, nullptr};
  int nphases = 0;
  persist::Ctl* ctl = nullptr;
  int* perr = nullptr;
  unsigned long long* pstamps = nullptr;  // per-phase timestamps (profiling)
  int pvariant = 1;  // persistent kernel built for 3 blocks per SM
  int pgrid = 0;
  size_t psmem = 0;
  long long pspin = kDefaultSpinCycles;
  int skip_block = -1, skip_barrier = -1;
};

namespace {

void ens_drop_graphs(moloch_ensemble* e) {
  for (int q = 0; q < 2; ++q) {
    if (e->gexec[q]) { cudaGraphExecDestroy(e->gexec[q]); e->gexec[q] = nullptr; }
    if (e->graph[q]) { cudaGraphDestroy(e->graph[q]); e->graph[q] = nullptr; }
  }
}

// Tile tables of every kernel kind over all members.  Column-like tiles are
// ordered by decreasing work (kz, then member) so the longest blocks start
// first and the tail of each launch stays short.
void ens_tiles(moloch_ensemble* e) {
  for (int t = 0; t < TK_COUNT; ++t) e->tiles[t].clear();
  const int n = (int)e->m.size();
  std::vector<int> order(n);
  for (int q = 0; q < n; ++q) order[q] = q;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return e->m[a]->kz() > e->m[b]->kz(); });
  for (int q : order) {
    const int nj = e->m[q]->nj(), ni = e->m[q]->ni(), kz = e->m[q]->kz();
    const int tj = (nj + 31) / 32;
    for (int z = 0; z < kz; ++z)
      for (int y = 0; y < (ni + 7) / 8; ++y)
        for (int x = 0; x < tj; ++x) e->tiles[TK_POINT].push_back(make_int4(q, x, y, z));
    for (int y = 0; y < (ni + 3) / 4; ++y)
      for (int x = 0; x < tj; ++x) e->tiles[TK_COLUMN].push_back(make_int4(q, x, y, 0));
    if (e->elem == 4 && e->m[q]->vf.cmaps) {
      for (int y = 0; y < (ni + kTwRows - 1) / kTwRows; ++y)
        for (int x = 0; x < tj; ++x) e->tiles[TK_COLTW].push_back(make_int4(q, x, y, 0));
    } else {
      for (int y = 0; y < (ni + 3) / 4; ++y)
        for (int x = 0; x < tj; ++x) e->tiles[TK_COLREST].push_back(make_int4(q, x, y, 0));
    }
    for (int y = 0; y < (ni + 3) / 4; ++y)
      for (int x = 0; x < tj * (kNumAdvected / e->vfields); ++x) e->tiles[TK_VERTICAL].push_back(make_int4(q, x, y, 0));
    for (int z = 0; z < (kz + kKC - 1) / kKC; ++z)
      for (int y = 0; y < (ni + 7) / 8; ++y)
        for (int x = 0; x < tj; ++x) e->tiles[TK_CHUNK].push_back(make_int4(q, x, y, z));
    // the persistent kernel's 32 x 8 blocks: column tiles 8 rows high
    // (by = 2 by8 for the 32 x 4 column bodies), 8 strips per item
    for (int y = 0; y < (ni + 7) / 8; ++y)
      for (int x = 0; x < tj; ++x) e->tiles[TK_COLUMN8].push_back(make_int4(q, x, 2 * y, 0));
    for (int y = 0; y < (ni + 7) / 8; ++y)
      for (int x = 0; x < tj * (kNumAdvected / e->vfields); ++x)
        e->tiles[TK_VERTICAL8].push_back(make_int4(q, x, 2 * y, 0));
    {
      const int nmstrips = ((nj + kMomJ - 1) / kMomJ) * ((ni + e->mrows - 1) / e->mrows);
      for (int z = 0; z < kz; ++z)
        for (int x = 0; x < (nmstrips + 3) / 4; ++x) e->tiles[TK_MSTRIP].push_back(make_int4(q, x, z, 0));
      const int nstrips = ((nj + kMomJ - 1) / kMomJ) * ((ni + kMomR - 1) / kMomR);  // persistent kernel
      const int ndstrips = ((nj + kDDJ - 1) / kDDJ) * ((ni + kDDR - 1) / kDDR);
      for (int z = 0; z < kz; ++z)
        for (int x = 0; x < (ndstrips + 3) / 4; ++x) e->tiles[TK_DSTRIP].push_back(make_int4(q, x, z, 0));
      for (int z = 0; z < (kz + kDDLevels - 1) / kDDLevels; ++z)
        for (int x = 0; x < (ndstrips + 3) / 4; ++x) e->tiles[TK_DSTRIP2].push_back(make_int4(q, x, z, 0));
      for (int z = 0; z < kz; ++z)
        for (int x = 0; x < (nstrips + 7) / 8; ++x) e->tiles[TK_MSTRIP8].push_back(make_int4(q, x, z, 0));
      for (int z = 0; z < kz; ++z)
        for (int x = 0; x < (ndstrips + 7) / 8; ++x) e->tiles[TK_DSTRIP8].push_back(make_int4(q, x, z, 0));
    }
    if (e->hz_levels >= 16) {  // warp strips: 4 strips of hz_levels rows per block, every level
      const int nstrips = ((nj + 27) / 28) * ((ni + e->hz_levels - 1) / e->hz_levels);
      for (int z = 0; z < kz; ++z)
        for (int x = 0; x < (nstrips + 3) / 4; ++x) e->tiles[TK_HORIZONTAL].push_back(make_int4(q, x, z, 0));
    } else {
      const int hz = std::min(e->hz_levels, kz);
      for (int z = 0; z < (kz + hz - 1) / hz; ++z)
        for (int y = 0; y < (ni + 7) / 8; ++y)
          for (int x = 0; x < tj; ++x) e->tiles[TK_HORIZONTAL].push_back(make_int4(q, x, y, z));
    }
  }
}

// upload views (4 parities x members) and tile tables into one device block
template <class T>
int ens_upload(moloch_ensemble* e, Batch<T>& b, View<T> moloch_handle::*vm) {
  const int n = (int)e->m.size();
  size_t bytes = 4 * n * sizeof(View<T>);
  for (int t = 0; t < TK_COUNT; ++t) bytes += ((e->tiles[t].size() * sizeof(int4) + 255) & ~size_t(255));
  // the members' tensor maps for the batched staged column solve (FP32
  // members with maps: jx a multiple of 4, kz <= 64)
  const size_t set_bytes = (size_t)kfast::column_map_set_bytes();
  const size_t cm_bytes = 2 * set_bytes * (size_t)n;
  bool staged = false;
  for (auto* h : e->m) staged = staged || (e->elem == 4 && h->vf.cmaps != nullptr);
  bytes += staged ? ((cm_bytes + 255) & ~size_t(255)) : 0;
  // persistent mode: two phase programs, the barrier/queue words, the error word
  const size_t prog_bytes = ((sizeof(persist::Phase) * persist::kMaxPhases + 255) & ~size_t(255));
  const size_t stamp_bytes = sizeof(unsigned long long) * (persist::kMaxPhases + 1);
  const size_t pbytes = 2 * prog_bytes + ((sizeof(persist::Ctl) + 255) & ~size_t(255)) + 256 + stamp_bytes;
  if (e->dev) cudaFree(e->dev);
  e->dev = nullptr;
  e->prog[0] = e->prog[1] = nullptr;
  e->ctl = nullptr;
  e->perr = nullptr;
  CUDA_TRY(cudaMalloc(&e->dev, bytes + pbytes + 1024));
  std::vector<View<T>> hv(4 * (size_t)n);
  for (int cur = 0; cur < 2; ++cur)
    for (int fc = 0; fc < 2; ++fc)
      for (int q = 0; q < n; ++q) {
        View<T> v = e->m[q]->*vm;
        v.cur = cur;
        v.fcur = fc;
        v.hz_levels = e->hz_levels >= 16 ? e->hz_levels : std::min(e->hz_levels, v.kz);
        v.vfields = e->vfields;
        v.bind_fields();
        hv[(size_t)(cur * 2 + fc) * n + q] = v;
      }
  char* p = (char*)e->dev;
  CUDA_TRY(cudaMemcpy(p, hv.data(), hv.size() * sizeof(View<T>), cudaMemcpyHostToDevice));
  for (int cur = 0; cur < 2; ++cur)
    for (int fc = 0; fc < 2; ++fc) b.views[cur][fc] = (const View<T>*)(p + (size_t)(cur * 2 + fc) * n * sizeof(View<T>));
  size_t off = ((4 * n * sizeof(View<T>)) + 255) & ~size_t(255);
  for (int t = 0; t < TK_COUNT; ++t) {
    CUDA_TRY(cudaMemcpy(p + off, e->tiles[t].data(), e->tiles[t].size() * sizeof(int4), cudaMemcpyHostToDevice));
    b.tiles[t] = (const int4*)(p + off);
    b.ntiles[t] = (int)e->tiles[t].size();
    b.hstrip = e->hz_levels >= 16;
    b.kmarch = e->kmarch;
    b.vfields = e->vfields;
    b.mrows = e->mrows;
    off += (e->tiles[t].size() * sizeof(int4) + 255) & ~size_t(255);
  }
  b.cmaps = nullptr;
  if (staged) {  // the 12-row boxes (map config 1) of each member, both parities
    std::vector<unsigned char> hm(cm_bytes, 0);
    for (int q = 0; q < n; ++q)
      if (e->m[q]->vf.cmaps)
        std::memcpy(hm.data() + 2 * set_bytes * q,
                    static_cast<const unsigned char*>(e->m[q]->vf.cmaps) + 2 * set_bytes, 2 * set_bytes);
    CUDA_TRY(cudaMemcpy(p + off, hm.data(), cm_bytes, cudaMemcpyHostToDevice));
    b.cmaps = p + off;
    off += (cm_bytes + 255) & ~size_t(255);
  }
  if (!e->pgrid) {
    int dev = 0, sms = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    e->pgrid = persist::blocks_per_sm<T>(e->pvariant, &e->psmem) * sms;
  }
  // persistent-mode programs (empty when the tuning has a variant the
  // persistent kernel does not carry)
  e->nphases = 0;
  for (int f = 0; f < 2; ++f) {
    std::vector<persist::Phase> prog;
    const int prc = persist::program<T>(b, e->fl, f, e->pgrid, prog);
    if (prc == 0) {
      CUDA_TRY(cudaMemcpy(p + off, prog.data(), prog.size() * sizeof(persist::Phase), cudaMemcpyHostToDevice));
      e->prog[f] = (const persist::Phase*)(p + off);
      e->nphases = (int)prog.size();
    }
    off += prog_bytes;
  }
  e->ctl = (persist::Ctl*)(p + off);
  off += (sizeof(persist::Ctl) + 255) & ~size_t(255);
  e->perr = (int*)(p + off);
  b.kerr = e->perr;
  b.spin = e->pspin > 0 ? e->pspin : kDefaultSpinCycles;
  off += 256;
  e->pstamps = (unsigned long long*)(p + off);
  CUDA_TRY(cudaMemset(e->perr, 0, sizeof(int)));
  if (e->persistent && (!e->nphases || !e->pgrid)) e->persistent = 0;
  return MOLOCH_OK;
}

int ens_build(moloch_ensemble* e) {
  ens_drop_graphs(e);
  ens_tiles(e);
  return e->elem == 8 ? ens_upload(e, e->bd, &moloch_handle::vd) : ens_upload(e, e->bf, &moloch_handle::vf);
}

template <class T>
int ens_step_persistent(moloch_ensemble* e, const Batch<T>& b, bool stamps = false) {
  persist::Args<T> a;
  a.views = b.views[0][0];  // the four parities follow one another, n views each
  a.nmembers = (int)e->m.size();
  a.prog = e->prog[e->fcur];
  a.nphases = e->nphases;
  a.ctl = e->ctl;
  a.err = e->perr;
  a.spin = e->pspin;
  a.skip_block = e->skip_block;
  a.skip_barrier = e->skip_barrier;
  a.stamps = stamps ? e->pstamps : nullptr;
  cudaMemsetAsync(e->ctl, 0, persist::ctl_bytes(e->nphases), e->stream);
  persist::launch<T>(a, e->pvariant, e->pgrid, e->psmem, e->stream);
  e->fcur ^= (e->fl.nadv & 1);
  e->cur = 0;
  return 1;
}

int ens_step_kernels(moloch_ensemble* e) {
  if (e->persistent)
    return e->elem == 8 ? ens_step_persistent(e, e->bd) : ens_step_persistent(e, e->bf);
  return e->elem == 8 ? kfast::blaunch_step(e->bd, e->stream, e->fl, e->cur, e->fcur)
                      : kfast::blaunch_step(e->bf, e->stream, e->fl, e->cur, e->fcur);
}

// members' own handles see the state the ensemble left them in
void ens_sync_members(moloch_ensemble* e) {
  for (auto* h : e->m) {
    if (h->elem == 8) { h->vd.cur = e->cur; h->vd.fcur = e->fcur; h->vd.bind_fields(); }
    else { h->vf.cur = e->cur; h->vf.fcur = e->fcur; h->vf.bind_fields(); }
    for (int q = 0; q < 2; ++q) {  // member graphs captured for the other parity stay valid
      (void)q;
    }
  }
}

}  // namespace

extern "C" {

int moloch_gpu_ensemble_create(int n, moloch_handle_t* const* members, moloch_ensemble_t** out) {
  g_err.clear();
  if (n < 1 || !members || !out) return fail(MOLOCH_ERR_ARG, "need members");
  *out = nullptr;
  moloch_handle* h0 = members[0];
  for (int q = 0; q < n; ++q) {
    moloch_handle* h = members[q];
    if (!h || !h->initialized) return fail(MOLOCH_ERR_STATE, "member %d not initialized", q);
    if (h->prm.mode == MOLOCH_FP64_EXACT) return fail(MOLOCH_ERR_ARG, "ensembles run the FP64 or FP32-storage builds");
    if (h->elem != h0->elem || h->prm.mo_nadv != h0->prm.mo_nadv || h->prm.mo_nsound != h0->prm.mo_nsound ||
        h->prm.mo_divfilter != h0->prm.mo_divfilter || h->prm.do_filterpai || h->prm.do_filtertheta ||
        h->stream != h0->stream)
      return fail(MOLOCH_ERR_ARG, "member %d: mode, nadv, nsound, filters and stream must match (pai/theta filters unsupported)", q);
    const int cur = h->elem == 8 ? h->vd.cur : h->vf.cur;
    const int fc = h->elem == 8 ? h->vd.fcur : h->vf.fcur;
    const int fc0 = h0->elem == 8 ? h0->vd.fcur : h0->vf.fcur;
    if (cur != 0 || fc != fc0) return fail(MOLOCH_ERR_STATE, "member %d is at a different buffer parity", q);
  }
  moloch_ensemble* e = new moloch_ensemble();
  e->m.assign(members, members + n);
  e->elem = h0->elem;
  e->stream = h0->stream;
  e->fl = flags_of(h0);
  e->fcur = h0->elem == 8 ? h0->vd.fcur : h0->vf.fcur;
  int rc = ens_build(e);
  if (rc) {
    if (e->dev) cudaFree(e->dev);
    delete e;
    return rc;
  }
  *out = e;
  return MOLOCH_OK;
}

int moloch_gpu_ensemble_run(moloch_ensemble_t* e, int nsteps, int use_graph) {
  g_err.clear();
  if (!e) return fail(MOLOCH_ERR_ARG, "null ensemble");
  for (int st = 0; st < nsteps; ++st) {
    if (!use_graph) {
      int n = ens_step_kernels(e);
      e->kernels += n;
      e->kernels_per_step = n;
    } else {
      const int par = e->fcur;
      if (!e->gexec[par]) {
        const int c0 = e->cur, f0 = e->fcur;
        CUDA_TRY(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
        int n = ens_step_kernels(e);
        cudaGraph_t g = nullptr;
        cudaError_t err = cudaStreamEndCapture(e->stream, &g);
        e->cur = c0; e->fcur = f0;
        if (err != cudaSuccess) return fail(MOLOCH_ERR_CUDA, "ensemble capture: %s", cudaGetErrorString(err));
        e->graph[par] = g;
        CUDA_TRY(cudaGraphInstantiate(&e->gexec[par], g, 0));
        e->kernels_per_step = n;
      }
      CUDA_TRY(cudaGraphLaunch(e->gexec[par], e->stream));
      e->kernels += e->kernels_per_step;
      e->fcur ^= (e->fl.nadv & 1);
      e->cur = 0;
    }
    int rc = check_launch("ensemble step");
    if (rc) return rc;
  }
  ens_sync_members(e);
  return MOLOCH_OK;
}

int moloch_gpu_ensemble_autotune(moloch_ensemble_t* e, int* choice, double* best_ms, int nchoice) {
  g_err.clear();
  if (!e || !choice || nchoice < kTuneCount) return fail(MOLOCH_ERR_ARG, "need %d choice slots", kTuneCount);
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  double best = 1e30;
  int pick = e->hz_levels;
  for (int c = 0; c < 7; ++c) {
    e->hz_levels = kTuneCandidates[0][c];
    int rc = ens_build(e);
    if (rc) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
    float ms = 0.f, tot = 0.f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0, e->stream);
      e->kernels += e->elem == 8 ? kfast::blaunch_advection(e->bd, e->stream, e->cur, e->fcur)
                                 : kfast::blaunch_advection(e->bf, e->stream, e->cur, e->fcur);
      cudaEventRecord(e1, e->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        cudaEventDestroy(e0); cudaEventDestroy(e1);
        return fail(MOLOCH_ERR_CUDA, "ensemble autotune: %s", cudaGetErrorString(cudaGetLastError()));
      }
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) tot += ms;
    }
    if (tot < best) { best = tot; pick = e->hz_levels; }
  }
  e->hz_levels = pick;
  // sound point kernels: one level per thread or k-marching (each of the
  // three), timed on whole steps
  const PhaseFlags fl = flags_of(e->m[0]);
  double best1 = 1e30;
  int pick1 = e->kmarch;
  bool staged_ok = false;
  for (auto* h : e->m) staged_ok = staged_ok || (e->elem == 4 && h->vf.cmaps != nullptr);
  for (int c2 = 0; c2 < 128; ++c2) {
    const int cand = (c2 & 63) | ((c2 & 64) ? 512 : 0);
    if ((cand & 12) == 12) continue;  // strips replace the k-marching momentum
    if ((cand & 16) && (cand & 3)) continue;  // the fused kernel replaces both
    if ((cand & 32) && !staged_ok) continue;  // batched staged column solve: FP32 members with tensor maps
    if ((cand & 512) && !(cand & 16)) continue;  // two levels per warp of the fused strips
    e->kmarch = cand;
    int rc = ens_build(e);
    if (rc) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
    float ms = 0.f, tot = 0.f;
    for (int rep = 0; rep < 2; ++rep) {
      cudaEventRecord(e0, e->stream);
      e->kernels += e->elem == 8 ? kfast::blaunch_step(e->bd, e->stream, fl, e->cur, e->fcur)
                                 : kfast::blaunch_step(e->bf, e->stream, fl, e->cur, e->fcur);
      cudaEventRecord(e1, e->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        cudaEventDestroy(e0); cudaEventDestroy(e1);
        return fail(MOLOCH_ERR_CUDA, "ensemble autotune: %s", cudaGetErrorString(cudaGetLastError()));
      }
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) tot += ms;
    }
    if (tot < best1) { best1 = tot; pick1 = cand; }
  }
  e->kmarch = pick1;
  // vertical WAF: fields per thread, timed on advection()
  double best2 = 1e30;
  int pick2 = e->vfields;
  for (int cand : kVFieldCandidates) {
    e->vfields = cand;
    int rc = ens_build(e);
    if (rc) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
    float ms = 0.f, tot = 0.f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0, e->stream);
      e->kernels += e->elem == 8 ? kfast::blaunch_advection(e->bd, e->stream, e->cur, e->fcur)
                                 : kfast::blaunch_advection(e->bf, e->stream, e->cur, e->fcur);
      cudaEventRecord(e1, e->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        cudaEventDestroy(e0); cudaEventDestroy(e1);
        return fail(MOLOCH_ERR_CUDA, "ensemble autotune: %s", cudaGetErrorString(cudaGetLastError()));
      }
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) tot += ms;
    }
    if (tot < best2) { best2 = tot; pick2 = cand; }
  }
  e->vfields = pick2;
  // rows per momentum warp strip (when the strips run), timed on whole steps
  double best3 = 0.0;
  if (e->kmarch & 8) {
    best3 = 1e30;
    int pick3 = e->mrows;
    for (int cand : kStripRowCandidates) {
      e->mrows = cand;
      int rc = ens_build(e);
      if (rc) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
      float ms = 0.f, tot = 0.f;
      for (int rep = 0; rep < 2; ++rep) {
        cudaEventRecord(e0, e->stream);
        e->kernels += e->elem == 8 ? kfast::blaunch_step(e->bd, e->stream, fl, e->cur, e->fcur)
                                   : kfast::blaunch_step(e->bf, e->stream, fl, e->cur, e->fcur);
        cudaEventRecord(e1, e->stream);
        if (cudaEventSynchronize(e1) != cudaSuccess) {
          cudaEventDestroy(e0); cudaEventDestroy(e1);
          return fail(MOLOCH_ERR_CUDA, "ensemble autotune: %s", cudaGetErrorString(cudaGetLastError()));
        }
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0) tot += ms;
      }
      if (tot < best3) { best3 = tot; pick3 = cand; }
    }
    e->mrows = pick3;
  }
  // one cooperative launch per step (the persistent kernel) against one
  // launch per kernel, timed on whole steps, when the persistent kernel
  // carries the chosen variants
  const bool pok = e->elem == 8 ? persist::supports<double>(e->hz_levels, e->kmarch, e->vfields)
                                : persist::supports<float>(e->hz_levels, e->kmarch, e->vfields);
  // mode 0: one launch per kernel; 1 + v: the persistent kernel built for
  // 2 + v blocks per SM
  double tmode[1 + persist::kVariants];
  for (double& t : tmode) t = 1e30;
  for (int mode = 0; mode < (pok ? 1 + persist::kVariants : 1); ++mode) {
    e->persistent = mode ? 1 : 0;
    if (mode && e->pvariant != mode - 1) {
      e->pvariant = mode - 1;
      e->pgrid = 0;
    }
    int rc = ens_build(e);
    if (rc) { cudaEventDestroy(e0); cudaEventDestroy(e1); return rc; }
    if (mode && !e->persistent) continue;  // no resident blocks
    float ms = 0.f, tot = 0.f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0, e->stream);
      e->kernels += ens_step_kernels(e);
      cudaEventRecord(e1, e->stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        cudaEventDestroy(e0); cudaEventDestroy(e1);
        return fail(MOLOCH_ERR_CUDA, "ensemble autotune: %s", cudaGetErrorString(cudaGetLastError()));
      }
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) tot += ms;
    }
    tmode[mode] = tot;
  }
  if (pok && e->perr) {
    int v = 0;
    CUDA_TRY(cudaMemcpy(&v, e->perr, sizeof(int), cudaMemcpyDeviceToHost));
    if (v) {
      CUDA_TRY(cudaMemset(e->perr, 0, sizeof(int)));
      cudaEventDestroy(e0); cudaEventDestroy(e1);
      e->persistent = 0;
      return fail(MOLOCH_ERR_TIMEOUT, "ensemble autotune: a grid-barrier wait of the persistent kernel gave up");
    }
  }
  int bestm = 0;
  for (int mode = 1; mode < 1 + persist::kVariants; ++mode)
    if (tmode[mode] < tmode[bestm]) bestm = mode;
  e->persistent = bestm ? 1 : 0;
  if (bestm && e->pvariant != bestm - 1) {
    e->pvariant = bestm - 1;
    e->pgrid = 0;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  choice[0] = pick;
  choice[1] = pick1;
  choice[2] = pick2;
  choice[3] = e->mrows;
  choice[4] = 0;  // the batched staggering kernel takes one column per thread
  if (best_ms) {
    best_ms[0] = best / 2.0; best_ms[1] = best1; best_ms[2] = best2 / 2.0; best_ms[3] = best3; best_ms[4] = 0.0;
  }
  ens_sync_members(e);
  return ens_build(e);
}

int moloch_gpu_ensemble_set_tuning(moloch_ensemble_t* e, const int* choice, int nchoice) {
  g_err.clear();
  if (!e || (nchoice > 0 && !choice)) return fail(MOLOCH_ERR_ARG, "null argument");
  // every slot is checked before any is applied
  if (nchoice > 0 && (choice[0] < 1 || choice[0] > 64)) return fail(MOLOCH_ERR_ARG, "hz_levels %d", choice[0]);
  if (nchoice > 1 && (choice[1] < 0 || (choice[1] & ~(63 | 512))))
    return fail(MOLOCH_ERR_ARG, "kmarch %d", choice[1]);
  if (nchoice > 2 && !valid_vfields(choice[2]))
    return fail(MOLOCH_ERR_ARG, "vertical fields per thread %d", choice[2]);
  if (nchoice > 3 && (choice[3] < 4 || choice[3] > 64))
    return fail(MOLOCH_ERR_ARG, "rows per momentum strip %d", choice[3]);
  if (nchoice > 4 && (choice[4] < 0 || choice[4] > 1)) return fail(MOLOCH_ERR_ARG, "staggering variant %d", choice[4]);
  if (nchoice > 0) e->hz_levels = choice[0];
  if (nchoice > 1) e->kmarch = choice[1];
  if (nchoice > 2) e->vfields = choice[2];
  if (nchoice > 3) e->mrows = choice[3];
  return ens_build(e);
}

long long moloch_gpu_ensemble_kernel_count(moloch_ensemble_t* e) { return e ? e->kernels : -1; }

int moloch_gpu_ensemble_set_persistent(moloch_ensemble_t* e, int on) {
  g_err.clear();
  if (!e) return fail(MOLOCH_ERR_ARG, "null ensemble");
  if (on < 0 || on > 4) return fail(MOLOCH_ERR_ARG, "persistent %d: 0 off, 1 default, 2-4 blocks per SM", on);
  if (on) {
    const bool ok = e->elem == 8 ? persist::supports<double>(e->hz_levels, e->kmarch, e->vfields)
                                 : persist::supports<float>(e->hz_levels, e->kmarch, e->vfields);
    if (!ok)
      return fail(MOLOCH_ERR_ARG,
                  "the persistent kernel does not carry this tuning (hz_levels %d, kmarch %d, vfields %d): "
                  "horizontal WAF tiles (1-8 levels), 1 or 2 vertical fields per thread, no %s",
                  e->hz_levels, e->kmarch, e->vfields,
                  e->elem == 8 ? "fused divergence/damping strips" : "k-marching momentum");
  }
  if (on >= 2 && on - 2 != e->pvariant) {
    e->pvariant = on - 2;
    e->pgrid = 0;  // resident blocks of the other build
  }
  e->persistent = on ? 1 : 0;
  int rc = ens_build(e);
  if (rc) return rc;
  if (on && !e->persistent) return fail(MOLOCH_ERR_CUDA, "persistent kernel: no resident blocks or no program");
  return MOLOCH_OK;
}

int moloch_gpu_ensemble_persistent(moloch_ensemble_t* e) { return e ? (e->persistent ? e->pvariant + 2 : 0) : -1; }

int moloch_gpu_ensemble_profile_step(moloch_ensemble_t* e, double* ms_by_kind, int* launches_by_kind, int nkinds) {
  g_err.clear();
  if (!e) return fail(MOLOCH_ERR_ARG, "null ensemble");
  CUDA_TRY(cudaStreamSynchronize(e->stream));
  if (e->persistent) {
    const int np = e->nphases;
    const int f0 = e->fcur;
    e->kernels += e->elem == 8 ? ens_step_persistent(e, e->bd, true) : ens_step_persistent(e, e->bf, true);
    int rc = check_launch("ensemble profile");
    if (rc) return rc;
    std::vector<unsigned long long> st(np + 1);
    std::vector<persist::Phase> prog(np);
    CUDA_TRY(cudaMemcpyAsync(st.data(), e->pstamps, st.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                             e->stream));
    CUDA_TRY(cudaMemcpyAsync(prog.data(), e->prog[f0], prog.size() * sizeof(persist::Phase), cudaMemcpyDeviceToHost,
                             e->stream));
    CUDA_TRY(cudaStreamSynchronize(e->stream));
    for (int p = 0; p < np; ++p) {
      const int k = persist::phase_kernel_kind(prog[p].kind);
      if (k < nkinds) {
        if (ms_by_kind) ms_by_kind[k] += (double)(st[p + 1] - st[p]) * 1e-6;
        if (launches_by_kind) launches_by_kind[k] += 1;
      }
    }
    ens_sync_members(e);
    return moloch_gpu_ensemble_sync(e);
  }
  KernelTimer* tm = new KernelTimer();
  for (int q = 0; q < KernelTimer::kCap; ++q)
    if (cudaEventCreate(&tm->ev[q]) != cudaSuccess) {
      for (int r = 0; r < q; ++r) cudaEventDestroy(tm->ev[r]);
      delete tm;
      return fail(MOLOCH_ERR_CUDA, "event create");
    }
  kfast::set_timer(tm);
  int n = ens_step_kernels(e);
  kfast::set_timer(nullptr);
  e->kernels += n;
  int rc = check_launch("ensemble profile");
  if (!rc && cudaStreamSynchronize(e->stream) != cudaSuccess) rc = fail(MOLOCH_ERR_CUDA, "ensemble profile sync");
  if (!rc && !tm->ok) rc = fail(MOLOCH_ERR_ARG, "too many kernels to profile one step");
  if (!rc) {
    for (int q = 0; q + 1 < tm->n; q += 2) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, tm->ev[q], tm->ev[q + 1]);
      const int k = tm->kind[q / 2];
      if (k < nkinds) {
        if (ms_by_kind) ms_by_kind[k] += ms;
        if (launches_by_kind) launches_by_kind[k] += 1;
      }
    }
  }
  for (int q = 0; q < KernelTimer::kCap; ++q) cudaEventDestroy(tm->ev[q]);
  delete tm;
  ens_sync_members(e);
  return rc;
}

int moloch_gpu_ensemble_set_wait_limit(moloch_ensemble_t* e, long long cycles, int skip_block, int skip_barrier) {
  g_err.clear();
  if (!e) return fail(MOLOCH_ERR_ARG, "null ensemble");
  e->pspin = cycles > 0 ? cycles : kDefaultSpinCycles;
  e->skip_block = skip_block;
  e->skip_barrier = skip_barrier;
  ens_drop_graphs(e);  // the launch arguments are baked into captured graphs
  return MOLOCH_OK;
}

int moloch_gpu_ensemble_sync(moloch_ensemble_t* e) {
  g_err.clear();
  if (!e) return fail(MOLOCH_ERR_ARG, "null ensemble");
  CUDA_TRY(cudaStreamSynchronize(e->stream));
  int rc = check_launch("ensemble");
  if (rc) return rc;
  if (e->perr) {
    int v = 0;
    CUDA_TRY(cudaMemcpy(&v, e->perr, sizeof(int), cudaMemcpyDeviceToHost));
    if (v) {
      CUDA_TRY(cudaMemset(e->perr, 0, sizeof(int)));
      return fail(MOLOCH_ERR_TIMEOUT, "a bounded wait of an ensemble kernel gave up (a grid barrier of the "
                                      "persistent kernel or a staged copy of the batched column solve); "
                                      "the steps since the last sync did not complete");
    }
  }
  return MOLOCH_OK;
}

int moloch_gpu_ensemble_destroy(moloch_ensemble_t* e) {
  if (!e) return MOLOCH_OK;
  cudaStreamSynchronize(e->stream);
  ens_drop_graphs(e);
  if (e->dev) cudaFree(e->dev);
  delete e;
  return MOLOCH_OK;
}

}  // extern "C"

// accessors for the surrogate translation unit (moloch_mlp.cu)
moloch::View<float>* moloch_internal_viewf(moloch_handle_t* h) {
  return (h && h->elem == 4 && h->initialized) ? &h->vf : nullptr;
}
cudaStream_t moloch_internal_stream(moloch_handle_t* h) { return h->stream; }
int moloch_internal_nadv(moloch_handle_t* h) { return h->prm.mo_nadv; }
int moloch_internal_nsound(moloch_handle_t* h) { return h->prm.mo_nsound; }
// attach (s != nullptr) or detach; the plain kernels read the skip flag
// through the view, and captured graphs are rebuilt on the next step
int moloch_internal_attach(moloch_handle_t* h, moloch::mlp::Surrogate* s) {
  if (h->elem != 4) return fail(MOLOCH_ERR_ARG, "the surrogate needs FP32 storage (MOLOCH_FP32_MIXED)");
  CUDA_TRY(cudaStreamSynchronize(h->stream));
  h->sur = s;
  h->vf.sur_skip = s ? s->ctl : nullptr;  // ctl[0]: the cycle's commit flag
  drop_graphs(h);
  return MOLOCH_OK;
}

extern "C" {

int moloch_internal_describe(moloch_handle_t* h, moloch_grid_t* g, moloch_params_t* p) {
  if (!h || !g || !p) return fail(MOLOCH_ERR_ARG, "null argument");
  *g = h->grid;
  *p = h->prm;
  return MOLOCH_OK;
}

int moloch_gpu_destroy(moloch_handle_t* h) {
  if (!h) return MOLOCH_OK;
  cudaStreamSynchronize(h->stream);
  for (int q = 0; q < 2; ++q) {
    if (h->gexec[q]) cudaGraphExecDestroy(h->gexec[q]);
    if (h->graph[q]) cudaGraphDestroy(h->graph[q]);
  }
  if (h->arena) cudaFree(h->arena);
  if (h->hres) cudaFreeHost(h->hres);
  if (h->stage) cudaFreeHost(h->stage);
  if (h->out_stream) cudaStreamSynchronize(h->out_stream);
  if (h->out_dev) cudaFree(h->out_dev);
  if (h->out_f64) cudaFree(h->out_f64);
  if (h->out_host) cudaFreeHost(h->out_host);
  if (h->out_stream) cudaStreamDestroy(h->out_stream);
  if (h->out_taken) cudaEventDestroy(h->out_taken);
  if (h->out_done) cudaEventDestroy(h->out_done);
  for (int q = 0; q < 2; ++q)
    if (h->stage_ev[q]) cudaEventDestroy(h->stage_ev[q]);
  if (h->up_stream) {
    cudaStreamSynchronize(h->up_stream);
    cudaStreamDestroy(h->up_stream);
  }
  for (const auto& r : h->pinned) cudaHostUnregister(const_cast<char*>(r.first));
  for (int f = 0; f < MOLOCH_F_COUNT; ++f) {
    if (h->up_stage[f]) cudaFree(h->up_stage[f]);
    if (h->up_read[f]) cudaEventDestroy(h->up_read[f]);
    if (h->up_commit[f]) cudaEventDestroy(h->up_commit[f]);
  }
  if (h->own_stream) cudaStreamDestroy(h->stream);
  delete h;
  return MOLOCH_OK;
}

}  // extern "C"
