// ILU sweep plans for FP64 factors (the templates are in sweep_impl.cuh; the
// plan's two precisions compile as separate translation units).
#include "sweep_impl.cuh"

namespace senkgpu {

template struct IluPlan<double>;
template void IluPlan<double>::sweep<double>(const SweepFactor<double> &, const double *, double *, cudaStream_t,
                                           const int *) const;

}  // namespace senkgpu
