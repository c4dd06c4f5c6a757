// ILU sweep plans for FP32 factors (the templates are in sweep_impl.cuh; the
// plan's two precisions compile as separate translation units).
#include "sweep_impl.cuh"

namespace senkgpu {

template struct IluPlan<float>;
template void IluPlan<float>::sweep<float>(const SweepFactor<float> &, const float *, float *, cudaStream_t,
                                           const int *) const;

}  // namespace senkgpu
