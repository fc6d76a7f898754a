// FP64 kernels compiled with --fmad=false: no multiply-add contraction, so
// each expression rounds exactly as the reference's FP64 evaluation order.
#define MOLOCH_KNS kexact
#include "moloch_kernels.cuh"

namespace moloch {
namespace kexact {
template int launch_prediag<double>(const View<double>&, cudaStream_t, const PhaseFlags&);
template int launch_sound<double>(View<double>&, cudaStream_t, const PhaseFlags&);
template int launch_advection<double>(View<double>&, cudaStream_t);
template int launch_postdiag<double>(View<double>&, cudaStream_t, const PhaseFlags&, const double*, const double*);
template int launch_diag<double>(const View<double>&, cudaStream_t);
}  // namespace kexact
}  // namespace moloch
