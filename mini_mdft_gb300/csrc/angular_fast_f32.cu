// angular_fast_f32.cu -- instantiates the compile-time-shape angular
// kernels of angular_fast.cuh for storage float, arithmetic float (one
// translation unit per precision so the builds run in parallel).
#include "angular_fast.cuh"

namespace mdft {

template void ang_fast_setup<float, float>(const AngPlan&);
template void ang_fast_a2p<float, float>(const AngPlan&, const float*, Cx<float>*, bool, double, cudaStream_t);
template void ang_fast_p2a<float, float>(const AngPlan&, const Cx<float>*, float*, cudaStream_t);

}  // namespace mdft
