// angular_fast_df.cu -- instantiates the compile-time-shape angular
// kernels of angular_fast.cuh for storage double, arithmetic DF (one
// translation unit per precision so the builds run in parallel).
#include "angular_fast.cuh"

namespace mdft {

template void ang_fast_setup<double, DF>(const AngPlan&);
template void ang_fast_a2p<double, DF>(const AngPlan&, const double*, Cx<double>*, bool, double, cudaStream_t);
template void ang_fast_p2a<double, DF>(const AngPlan&, const Cx<double>*, double*, cudaStream_t);

}  // namespace mdft
