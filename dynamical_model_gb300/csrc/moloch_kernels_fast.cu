// FP64 and FP32-storage kernels with multiply-add contraction allowed.
#define MOLOCH_KNS kfast
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
