// Persistent ensemble step: types shared by the host (moloch_api.cpp) and
// the kernel translation unit (moloch_persist.cu).
//
// One cooperative launch advances every member of an ensemble by one MOLOCH
// step (nompi/mod_moloch.F90:272-421).  The launch walks a program of
// phases -- the kernels of the step in the order the per-kernel launches
// take (pre-diagnostics, nadv x (nsound x (divergence/damping, implicit w,
// momentum), vertical and horizontal WAF, staggering), post-diagnostics) --
// with a grid barrier between consecutive phases.  Inside a phase the
// resident blocks take (member, tile) items from a device-side work queue
// (one atomic counter per phase), so members of uneven size share the GPU
// without a static partition.  The phase bodies are the kernel bodies of the
// per-kernel launches.
#pragma once
#include <cuda_runtime.h>

#include <cstddef>
#include <vector>

#include "moloch_view.h"

namespace moloch {
namespace persist {

enum PhaseKind : int {
  PH_PREDIAG = 0, PH_DIVDAMP_STRIP, PH_DIV, PH_DIV_KM, PH_DAMP, PH_DAMP_KM, PH_COLUMN, PH_LAP_FILTER,
  PH_PAI_UPDATE, PH_MOM_STRIP, PH_MOM, PH_MOM_KM, PH_WAF_VERTICAL1, PH_WAF_VERTICAL2, PH_WAF_HORIZONTAL,
  PH_STAG, PH_POSTDIAG, PH_COUNT
};

// one phase: its body, its work items and the view parity it reads
struct Phase {
  int kind;
  int ntiles;
  const int4* tiles;  // device tile table (member, bx, by, bz)
  int par;            // views of parity (cur, fcur) = (par >> 1, par & 1)
  int a0, a1, a2;     // body arguments (strip rows; nsound, last, defer_pai; filter switches)
  int chunk;          // items a block takes from the queue at a time
};

constexpr int kMaxPhases = 1024;

// Barrier and queue words, zeroed before every launch.  count: blocks
// arrived at the current barrier; gen: barriers completed; q[p]: next item
// of phase p.
struct Ctl {
  unsigned int count;
  unsigned int gen;
  unsigned int pad[30];  // the barrier words on a 128-byte line of their own
  int q[kMaxPhases];
};
inline size_t ctl_bytes(int nphases) { return offsetof(Ctl, q) + sizeof(int) * (size_t)nphases; }

template <class T>
struct Args {
  const View<T>* views;  // 4 x nmembers: views[(cur * 2 + fcur) * nmembers + member]
  int nmembers;
  const Phase* prog;
  int nphases;
  Ctl* ctl;
  int* err;              // set to 1 by a barrier wait that gave up; cleared by the host
  long long spin;        // limit of a barrier wait, SM clock cycles
  int skip_block;        // test hook: this block leaves at barrier skip_barrier
  int skip_barrier;      // without arriving (-1: none)
  unsigned long long* stamps;  // profiling (nullptr: off): global timer (ns) at the
                               // start [0] and as block 0 leaves barrier p [p + 1]
};

// the per-kernel timing bucket (KernelKind) of each phase kind
inline int phase_kernel_kind(int ph) {
  switch (ph) {
    case PH_PREDIAG: return KK_PREDIAG;
    case PH_DIVDAMP_STRIP: return KK_SOUND_DIVDAMP;
    case PH_DIV: case PH_DIV_KM: return KK_SOUND_DIV;
    case PH_DAMP: case PH_DAMP_KM: return KK_SOUND_DAMP;
    case PH_COLUMN: return KK_SOUND_COLUMN;
    case PH_LAP_FILTER: return KK_LAP_FILTER;
    case PH_PAI_UPDATE: return KK_PAI_UPDATE;
    case PH_MOM_STRIP: case PH_MOM: case PH_MOM_KM: return KK_SOUND_MOMENTUM;
    case PH_WAF_VERTICAL1: case PH_WAF_VERTICAL2: return KK_WAF_VERTICAL;
    case PH_WAF_HORIZONTAL: return KK_WAF_HORIZONTAL;
    case PH_STAG: return KK_STAG_FROM_X;
    default: return KK_POSTDIAG;
  }
}

// The step as a phase program for the batch's tuning, starting at field-set
// parity fcur (u/v parity 0).  Returns 0, or a nonzero code when the tuning
// asks for a kernel variant the persistent kernel does not carry (FP32: the
// k-marching momentum; FP64: the fused divergence/damping strips; both: the
// horizontal WAF strips and 5 or 10 vertical-WAF fields per thread).
// grid: blocks of the launch (sets each phase's chunk to about an eighth of
// a block's share of the items).
template <class T>
int program(const Batch<T>& b, const PhaseFlags& fl, int fcur, int grid, std::vector<Phase>& out);
// whether the persistent kernel carries the variants of this tuning
template <class T>
bool supports(int hz_levels, int kmarch, int vfields);
// Kernel variants: built for 2, 3 or 4 resident blocks of 256 threads per
// SM (variant 0, 1, 2).  Resident blocks per SM of a variant (0 if it
// cannot run) and its dynamic shared memory.
constexpr int kVariants = 3;
template <class T>
int blocks_per_sm(int variant, size_t* smem);
// one cooperative launch of grid blocks of 32 x 8 threads
template <class T>
cudaError_t launch(const Args<T>& a, int variant, int grid, size_t smem, cudaStream_t st);

}  // namespace persist
}  // namespace moloch
